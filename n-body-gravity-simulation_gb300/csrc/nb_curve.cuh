// nb_curve.cuh -- space-filling-curve indices and order-preserving keys shared
// by the Barnes-Hut build (nb_bh.cu) and the sorted direct paths
// (nb_direct_sorted.cu, nb_batch.cu).
#pragma once

#include <cstdint>
#include <cstring>

namespace nb {

// 21 bits -> every third bit of 63 (standard magic-number spreading).
__host__ __device__ __forceinline__ uint64_t spread21(uint64_t v)
{
    v &= 0x1fffffull;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}

// Position on the Hilbert curve through a 2^10 x 2^10 x 2^10 grid (cells of a
// cube around the bodies), following J. Skilling, "Programming the Hilbert
// curve", AIP Conf. Proc. 707 (2004): the grid coordinates are turned into the
// curve's "transposed" index by reflections and exchanges from the top bit
// down, Gray-decoded, and their bits interleaved (axis 0 most significant).  Consecutive indices are
// face-adjacent cells, so a run of sorted bodies fills a compact region (the
// Morton curve jumps between distant cells at every level boundary).
__host__ __device__ __forceinline__ uint32_t hilbert_index30(uint32_t a0, uint32_t a1,
                                                          uint32_t a2)
{
    uint32_t X[3] = {a0, a1, a2};
    for (uint32_t q = 1u << 9; q > 1; q >>= 1) {
        const uint32_t p = q - 1;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (X[i] & q) {
                X[0] ^= p;  // reflect the low bits of axis 0
            } else {        // exchange the low bits of axes 0 and i
                const uint32_t t = (X[0] ^ X[i]) & p;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];
    X[2] ^= X[1];
    uint32_t t = 0;
    for (uint32_t q = 1u << 9; q > 1; q >>= 1)
        if (X[2] & q) t ^= q - 1;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    return (uint32_t)((spread21(X[0]) << 2) | (spread21(X[1]) << 1) | spread21(X[2]));
}

// The bits of a double as a 64-bit integer, and back.
__host__ __device__ __forceinline__ long long bits_of(double v)
{
#ifdef __CUDA_ARCH__
    return __double_as_longlong(v);
#else
    long long b;
    memcpy(&b, &v, sizeof b);
    return b;
#endif
}
__host__ __device__ __forceinline__ double double_of(long long b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double v;
    memcpy(&v, &b, sizeof v);
    return v;
#endif
}
// An FP64 value as a signed 64-bit key with the same order (negative values
// have their magnitude bits flipped); the min/max reduction then runs on the
// integer pipes (GB300's FP64 pipe is a small fraction of them).  NaN maps to
// the neutral key, so it is ignored as fmin/fmax ignore it.
__host__ __device__ __forceinline__ long long order_key(double v, long long nan_key)
{
    const long long b = bits_of(v);
    if ((b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll) return nan_key;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}
__host__ __device__ __forceinline__ double key_value(long long k)
{
    return double_of(k >= 0 ? k : (k ^ 0x7fffffffffffffffll));
}

} // namespace nb
