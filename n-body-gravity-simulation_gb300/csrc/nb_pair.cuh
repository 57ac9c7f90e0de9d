// nb_pair.cuh -- the mixed-precision pair term shared by the all-pairs kernels
// (nb_direct.cu, nb_direct_sorted.cu) and the batched work-queue kernel
// (nb_batch.cu).
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

// (hi, lo) += s - c: a segment's Kahan pair (sum s, compensation c) added
// into a double-single accumulator with FP32 operations (two-sum of hi and s;
// the rounding error and -c go to lo).  The FP64 pipe of a GB300 SM runs at a
// small fraction of its FP32 rate, so partial sums are combined this way and
// converted to FP64 once: (double)hi + (double)lo.
__device__ __forceinline__ void ds_add_kahan(float &hi, float &lo, float s, float c)
{
    const float t = hi + s;
    const float bb = t - hi;
    const float e = (hi - (t - bb)) + (s - bb);
    hi = t;
    lo = lo + (e - c);
}

// s + e = a + b exactly (Knuth's two-sum; plain adds, nothing to contract).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// (h + l) - c as a normalised double-single S + E (|E| <= ulp(S) / 2); the
// only rounding is that of the low-order add, ~2^-48 |h|.
__device__ __forceinline__ void rel_ds(float h, float l, float c, float &S, float &E)
{
    float s, e;
    two_sum(h, -c, s, e);
    two_sum(s, e + l, S, E);
}

// (h + l) - c rounded to FP32: the S of rel_ds (one rounding of the exact
// difference, up to the ~2^-48 |h| of the low-order add) without the E.
__device__ __forceinline__ float rel_s(float h, float l, float c)
{
    float s, e;
    two_sum(h, -c, s, e);
    return s + (e + l);
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

// ---------------------------------------------------------------- packed f32x2
// sm_100-class SMs run FP32 add, multiply and FMA on register pairs at the
// FP32 pipe's lane rate for half the issue slots; each lane rounds exactly
// like the scalar operation.  The packed kernels evaluate a j-pair (two
// consecutive j of a 32-body tile) per operation against one i-body held as
// negated, duplicated pairs.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// m r^-3 of a j-pair with the folded Newton step of pair_term; ZERO_SOFT
// zeroes the r2 == 0 (j == i) lane.
template <bool ZERO_SOFT>
__device__ __forceinline__ float2 pair_scale(float2 r2, float2 m)
{
    float2 inv = make_float2(rsqrt_mufu(r2.x), rsqrt_mufu(r2.y));
    if (ZERO_SOFT) {
        inv.x = r2.x > 0.f ? inv.x : 0.f;
        inv.y = r2.y > 0.f ? inv.y : 0.f;
    }
    const float2 inv2 = mul2(inv, inv);
    const float2 corr = fma2(dup2(-1.5f), mul2(r2, inv2), dup2(2.5f));
    return mul2(mul2(mul2(m, inv), inv2), corr);
}

// A 32-body j-tile staged as 16 j-pairs side by side, so that one broadcast
// 16-byte shared-memory load yields two f32x2 operands.  hi = (x, y, z, m),
// lo = the double-single low parts (x, y, z).
struct PairTile {
    float4 s[16];  // (x_2p, x_2p+1, y_2p, y_2p+1)
    float4 t[16];  // (z_2p, z_2p+1, m_2p, m_2p+1)
    float4 e[16];  // (xlo_2p, xlo_2p+1, ylo_2p, ylo_2p+1)
    float2 f[16];  // (zlo_2p, zlo_2p+1)
};

// Lane `lane` writes its j-body into the tile (call between two __syncwarp).
__device__ __forceinline__ void pair_tile_put(PairTile &pt, int lane, float x, float y, float z,
                                              float m, float xl, float yl, float zl)
{
    float *s = reinterpret_cast<float *>(&pt.s[lane >> 1]) + (lane & 1);
    float *t = reinterpret_cast<float *>(&pt.t[lane >> 1]) + (lane & 1);
    float *e = reinterpret_cast<float *>(&pt.e[lane >> 1]) + (lane & 1);
    float *f = reinterpret_cast<float *>(&pt.f[lane >> 1]) + (lane & 1);
    s[0] = x;
    s[2] = y;
    t[0] = z;
    t[2] = m;
    e[0] = xl;
    e[2] = yl;
    f[0] = zl;
}

// The same without the low parts (a tile read only by pair_term2_far).
__device__ __forceinline__ void pair_tile_put_hi(PairTile &pt, int lane, float x, float y, float z,
                                                 float m)
{
    float *s = reinterpret_cast<float *>(&pt.s[lane >> 1]) + (lane & 1);
    float *t = reinterpret_cast<float *>(&pt.t[lane >> 1]) + (lane & 1);
    s[0] = x;
    s[2] = y;
    t[0] = z;
    t[2] = m;
}

// j-pair p of a tile as f32x2 operands.
struct JPair {
    float2 x, y, z, m, xl, yl, zl;
};
__device__ __forceinline__ JPair pair_tile_get(const PairTile &pt, int p)
{
    const float4 A = pt.s[p], B = pt.t[p], C = pt.e[p];
    JPair j;
    j.x = make_float2(A.x, A.y);
    j.y = make_float2(A.z, A.w);
    j.z = make_float2(B.x, B.y);
    j.m = make_float2(B.z, B.w);
    j.xl = make_float2(C.x, C.y);
    j.yl = make_float2(C.z, C.w);
    j.zl = pt.f[p];
    return j;
}

// The double-single pair term of pair_term for a j-pair against one i-body
// given as negated duplicated pairs (nxh = (-xh, -xh), ...).
template <bool ZERO_SOFT>
__device__ __forceinline__ void pair_term2(const JPair &j, float2 nxh, float2 nyh, float2 nzh,
                                           float2 nxl, float2 nyl, float2 nzl, float2 e2,
                                           float2 &ax, float2 &ay, float2 &az)
{
    const float2 dx = add2(add2(j.x, nxh), add2(j.xl, nxl));
    const float2 dy = add2(add2(j.y, nyh), add2(j.yl, nyl));
    const float2 dz = add2(add2(j.z, nzh), add2(j.zl, nzl));
    const float2 r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, e2)));
    const float2 s = pair_scale<ZERO_SOFT>(r2, j.m);
    ax = fma2(dx, s, ax);
    ay = fma2(dy, s, ay);
    az = fma2(dz, s, az);
}

// The plain FP32 term (coordinates already relative to a nearby origin).
// NEWTON = false leaves out the folded Newton step (12 FP32 operations instead
// of 15): m r^-3 then carries the MUFU rsqrt error three times -- measured on
// GB300 over every FP32 input in [1, 4): at most 1.25e-7 relative per rsqrt,
// RMS 3.9e-8, mean -5e-9, i.e. a mean of -1.6e-8 on the cube.
template <bool NEWTON>
__device__ __forceinline__ void pair_term2_far(const JPair &j, float2 nx, float2 ny, float2 nz,
                                               float2 e2, float2 &ax, float2 &ay, float2 &az)
{
    const float2 dx = add2(j.x, nx);
    const float2 dy = add2(j.y, ny);
    const float2 dz = add2(j.z, nz);
    const float2 r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, e2)));
    float2 s;
    if (NEWTON) {
        s = pair_scale<false>(r2, j.m);
    } else {
        const float2 inv = make_float2(rsqrt_mufu(r2.x), rsqrt_mufu(r2.y));
        s = mul2(mul2(j.m, inv), mul2(inv, inv));
    }
    ax = fma2(dx, s, ax);
    ay = fma2(dy, s, ay);
    az = fma2(dz, s, az);
}

} // namespace nb
