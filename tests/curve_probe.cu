// Host-side checks of the curve and key helpers of nb_curve.cuh, compiled and
// run by tests/test_curve.py (no GPU needed).
//  1. The first 2^18 Hilbert indices fill the 2^6-cell corner cube: the
//     indices of its cells are exactly 0 .. 2^18 - 1, and consecutive indices
//     are face-adjacent cells.
//  2. order_key preserves the order of doubles (negative, -0, +0, denormals,
//     infinities) and maps NaN to the key it is given; key_value inverts it.
#include "nb_curve.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <vector>

int main()
{
    const uint32_t side = 1u << 6;
    std::vector<int> cell(side * side * side, -1);
    for (uint32_t a = 0; a < side; ++a)
        for (uint32_t b = 0; b < side; ++b)
            for (uint32_t c = 0; c < side; ++c) {
                const uint32_t h = nb::hilbert_index30(a, b, c);
                if (h >= cell.size() || cell[h] != -1) {
                    std::printf("FAIL hilbert index %u of (%u %u %u)\n", h, a, b, c);
                    return 1;
                }
                cell[h] = (int)((a << 12) | (b << 6) | c);
            }
    for (size_t h = 1; h < cell.size(); ++h) {
        const int p = cell[h - 1], q = cell[h];
        const int d = std::abs((p >> 12) - (q >> 12)) + std::abs(((p >> 6) & 63) - ((q >> 6) & 63)) +
                      std::abs((p & 63) - (q & 63));
        if (d != 1) {
            std::printf("FAIL step %zu: L1 distance %d\n", h, d);
            return 1;
        }
    }
    std::vector<double> v = {-std::numeric_limits<double>::infinity(), -1e300, -2.5, -1.0, -1e-310,
                             -0.0, 0.0, 1e-310, 1e-300, 0.5, 1.0, 3.0, 1e300,
                             std::numeric_limits<double>::infinity()};
    srand(7);
    for (int i = 0; i < 10000; ++i)
        v.push_back(((double)rand() / RAND_MAX - 0.5) * std::pow(10.0, rand() % 40 - 20));
    for (size_t i = 0; i < v.size(); ++i)
        for (size_t j = 0; j < v.size(); j += 97) {
            const long long ki = nb::order_key(v[i], 0), kj = nb::order_key(v[j], 0);
            if ((v[i] < v[j]) != (ki < kj) && !(v[i] == 0.0 && v[j] == 0.0)) {
                std::printf("FAIL order of %g and %g\n", v[i], v[j]);
                return 1;
            }
        }
    for (double x : v)
        if (nb::key_value(nb::order_key(x, 0)) != x || std::signbit(nb::key_value(nb::order_key(x, 0))) != std::signbit(x)) {
            std::printf("FAIL round trip of %g\n", x);
            return 1;
        }
    if (nb::order_key(std::nan(""), 42) != 42 || nb::order_key(-std::nan(""), -7) != -7) {
        std::printf("FAIL NaN key\n");
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
