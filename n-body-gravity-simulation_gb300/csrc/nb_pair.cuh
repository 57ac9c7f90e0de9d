// nb_pair.cuh -- the mixed-precision pair term shared by the all-pairs kernels
// (single system, nb_direct.cu) and the batched ensemble (nb_ensemble.cu).
//
// A body is a float4 hi = (x, y, z, m) and a float4 lo = (x - hi, y - hi,
// z - hi, 0): a double-single copy of its FP64 position.  The displacement
// (xj_hi - xi_hi) + (xj_lo - xi_lo) is exact to FP32 rounding for close pairs;
// r^-3 uses the MUFU rsqrt with one Newton step folded into the cube.
#pragma once

#include <cuda_runtime.h>

namespace nb {

__device__ __forceinline__ float rsqrt_mufu(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Padding body for the tail of a tile: massless and far away, so its pair
// term is exactly zero for every i-body.
__device__ __forceinline__ float4 far_body() { return make_float4(1.0e18f, 1.0e18f, 1.0e18f, 0.0f); }

// Kahan-compensated add of t into (s, c).  Plain FP32 adds: no product, so
// nothing can be contracted into an FMA.
__device__ __forceinline__ void kahan_add(float &s, float &c, float t)
{
    float y = t - c;
    float u = s + y;
    c = (u - s) - y;
    s = u;
}

// a += m_j (r_j - r_i) / (|r_j - r_i|^2 + eps2)^(3/2) for one (i, j) pair.
// ZERO_SOFT: eps2 == 0, where the j == i term (r2 == 0) must give 0.
template <bool ZERO_SOFT>
__device__ __forceinline__ void pair_term(const float4 &H, const float4 &L, float xh, float yh,
                                          float zh, float xl, float yl, float zl, float eps2,
                                          float &ax, float &ay, float &az)
{
    const float dx = (H.x - xh) + (L.x - xl);
    const float dy = (H.y - yh) + (L.y - yl);
    const float dz = (H.z - zh) + (L.z - zl);
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
    float inv = rsqrt_mufu(r2);
    if (ZERO_SOFT) inv = (r2 > 0.f) ? inv : 0.f;
    const float inv2 = inv * inv;
    // MUFU rsqrt is good to ~1.3e-7; y^3 with y = y0 (1 + d) is y0^3 (1 - 3d)
    // to first order and r2 y0^2 = 1 + 2d, so y^3 ~= y0^3 (2.5 - 1.5 r2 y0^2):
    // one Newton step folded into the cube leaves an O(d^2) error.
    const float corr = fmaf(-1.5f, r2 * inv2, 2.5f);
    const float s = ((H.w * inv) * inv2) * corr;
    ax = fmaf(dx, s, ax);
    ay = fmaf(dy, s, ay);
    az = fmaf(dz, s, az);
}

} // namespace nb
