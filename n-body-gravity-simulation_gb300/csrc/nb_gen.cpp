// nb_gen.cpp -- seeded host-side generators of the synthetic workloads.
//
// The reference builds its inputs inside each test (uniform cube, mt19937
// seed 42, CPU/tests/test2_ForceBenchmark.cpp:46-58); the Plummer and
// disk+bulge systems of the benchmark configurations have no reference code.
// Random numbers come from SplitMix64 (Steele, Lea & Flood 2014), one stream per
// body keyed by (seed, body index), so every body's draws are independent of
// the others and of the number of host threads.  All arithmetic is FP64.
#include "nb_internal.h"

#include <cmath>
#include <vector>

namespace {

struct Stream {
    uint64_t s;
    Stream(uint64_t seed, uint64_t body)
        : s(seed * 0xD1B54A32D192ED03ull ^ (body + 1) * 0x9E3779B97F4A7C15ull)
    {
        next();
    }
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // uniform on (0, 1): never 0 or 1
    double u() { return ((double)(next() >> 11) + 0.5) * 0x1.0p-53; }
    double normal()
    {
        const double a = u(), b = u();
        return std::sqrt(-2.0 * std::log(a)) * std::cos(2.0 * M_PI * b);
    }
};

void isotropic(Stream &r, double len, double &x, double &y, double &z)
{
    const double c = 1.0 - 2.0 * r.u();
    const double s = std::sqrt(std::max(0.0, 1.0 - c * c));
    const double phi = 2.0 * M_PI * r.u();
    x = len * s * std::cos(phi);
    y = len * s * std::sin(phi);
    z = len * c;
}

// Aarseth, Henon & Wielen (1974): radius from the cumulative mass (truncated
// at 99.9% of the mass), speed by von Neumann rejection on
// g(q) = q^2 (1 - q^2)^(7/2), q = v / v_escape.
void plummer_body(Stream &r, double M, double a, double G, double *p, double *v)
{
    const double X1 = 0.999 * r.u();
    const double rad = a / std::sqrt(std::pow(X1, -2.0 / 3.0) - 1.0);
    isotropic(r, rad, p[0], p[1], p[2]);
    double q = 0.0;
    for (int it = 0; it < 100000; ++it) {
        q = r.u();
        const double g = 0.1 * r.u();
        if (g < q * q * std::pow(1.0 - q * q, 3.5)) break;
    }
    const double ve = std::sqrt(2.0 * G * M / a) * std::pow(1.0 + rad * rad / (a * a), -0.25);
    isotropic(r, q * ve, v[0], v[1], v[2]);
}

void to_com_frame(size_t n, const double *m, double *x, double *y, double *z, double *vx,
                  double *vy, double *vz)
{
    double M = 0, c[6] = {0, 0, 0, 0, 0, 0};
    for (size_t i = 0; i < n; ++i) {
        M += m[i];
        c[0] += m[i] * x[i]; c[1] += m[i] * y[i]; c[2] += m[i] * z[i];
        c[3] += m[i] * vx[i]; c[4] += m[i] * vy[i]; c[5] += m[i] * vz[i];
    }
    if (!(M > 0)) return;
    for (double &v : c) v /= M;
    for (size_t i = 0; i < n; ++i) {
        x[i] -= c[0]; y[i] -= c[1]; z[i] -= c[2];
        vx[i] -= c[3]; vy[i] -= c[4]; vz[i] -= c[5];
    }
}

// Inverse of the exponential disk's cumulative mass 1 - (1 + y) e^-y = u.
double disk_radius(double u)
{
    double lo = 0.0, hi = 50.0, y = 1.0;
    for (int it = 0; it < 200; ++it) {
        const double f = 1.0 - (1.0 + y) * std::exp(-y) - u;
        if (f > 0) hi = y; else lo = y;
        const double df = y * std::exp(-y);
        double yn = (df > 0) ? y - f / df : 0.5 * (lo + hi);
        if (!(yn > lo && yn < hi)) yn = 0.5 * (lo + hi);
        if (std::fabs(yn - y) < 1e-15 * (1.0 + y)) { y = yn; break; }
        y = yn;
    }
    return y;
}

} // namespace

using nb::fail;

extern "C" {

nb_status nb_gen_plummer(size_t n, uint64_t seed, double total_mass, double scale, double G,
                         double *x, double *y, double *z, double *vx, double *vy, double *vz,
                         double *m)
{
    if (!x || !y || !z || !vx || !vy || !vz || !m)
        return fail(NB_ERR_INVALID_ARGUMENT, "NULL output array");
    if (!(total_mass > 0) || !(scale > 0) || !(G > 0))
        return fail(NB_ERR_INVALID_ARGUMENT, "mass, scale and G must be positive");
    for (size_t i = 0; i < n; ++i) {
        Stream r(seed, i);
        double p[3], v[3];
        plummer_body(r, total_mass, scale, G, p, v);
        x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
        vx[i] = v[0]; vy[i] = v[1]; vz[i] = v[2];
        m[i] = total_mass / (double)n;
    }
    to_com_frame(n, m, x, y, z, vx, vy, vz);
    return NB_OK;
}

nb_status nb_gen_disk_bulge(size_t n, uint64_t seed, double total_mass, double bulge_frac,
                            double bulge_scale, double disk_scale, double disk_height,
                            double dispersion, double G, double *x, double *y, double *z,
                            double *vx, double *vy, double *vz, double *m)
{
    if (!x || !y || !z || !vx || !vy || !vz || !m)
        return fail(NB_ERR_INVALID_ARGUMENT, "NULL output array");
    if (!(bulge_frac >= 0 && bulge_frac <= 1) || !(bulge_scale > 0) || !(disk_scale > 0) ||
        !(disk_height > 0) || !(G > 0) || !(total_mass > 0))
        return fail(NB_ERR_INVALID_ARGUMENT, "bad disk+bulge parameters");
    const size_t nb = (size_t)std::llround(bulge_frac * (double)n);
    const double Mb = total_mass * bulge_frac, Md = total_mass - Mb;
    for (size_t i = 0; i < n; ++i) {
        Stream r(seed, i);
        m[i] = total_mass / (double)n;
        double p[3], v[3];
        if (i < nb) {
            plummer_body(r, Mb, bulge_scale, G, p, v);
        } else {
            const double R = disk_scale * disk_radius(0.999 * r.u());
            const double phi = 2.0 * M_PI * r.u();
            const double uz = std::min(std::max(r.u(), 5e-4), 1.0 - 5e-4);
            p[0] = R * std::cos(phi);
            p[1] = R * std::sin(phi);
            p[2] = disk_height * std::atanh(2.0 * uz - 1.0);
            const double rs = std::sqrt(R * R + p[2] * p[2]);
            const double yd = R / disk_scale;
            const double menc = Mb * rs * rs * rs / std::pow(rs * rs + bulge_scale * bulge_scale, 1.5) +
                                Md * (1.0 - (1.0 + yd) * std::exp(-yd));
            const double vc = (R > 0) ? std::sqrt(G * menc / std::max(rs, 1e-12)) : 0.0;
            const double sig = dispersion * vc;
            v[0] = -vc * std::sin(phi) + sig * r.normal();
            v[1] = vc * std::cos(phi) + sig * r.normal();
            v[2] = sig * r.normal();
        }
        x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
        vx[i] = v[0]; vy[i] = v[1]; vz[i] = v[2];
    }
    to_com_frame(n, m, x, y, z, vx, vy, vz);
    return NB_OK;
}

} // extern "C"
