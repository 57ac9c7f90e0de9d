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
    float2 g[16];  // (mlo_2p, mlo_2p+1): mass low parts, written by pair_tile_put_mlo
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

// Lane `lane`'s mass low part (m - (float)m), for the double-single terms.
__device__ __forceinline__ void pair_tile_put_mlo(PairTile &pt, int lane, float ml)
{
    reinterpret_cast<float *>(&pt.g[lane >> 1])[lane & 1] = ml;
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

// Double-single displacement and softened r^2 of a j-pair against one i-body
// given as negated duplicated pairs (nxh = (-xh, -xh), ...).  Every operation
// is an explicit round-to-nearest intrinsic, so two evaluations of the same
// operands give the same bits (the near-pair exclusion below relies on it).
struct PairGeom {
    float2 dx, dy, dz, r2;
};
__device__ __forceinline__ PairGeom pair_geom(const JPair &j, float2 nxh, float2 nyh, float2 nzh,
                                              float2 nxl, float2 nyl, float2 nzl, float2 e2)
{
    PairGeom g;
    g.dx = add2(add2(j.x, nxh), add2(j.xl, nxl));
    g.dy = add2(add2(j.y, nyh), add2(j.yl, nyl));
    g.dz = add2(add2(j.z, nzh), add2(j.zl, nzl));
    g.r2 = fma2(g.dz, g.dz, fma2(g.dy, g.dy, fma2(g.dx, g.dx, e2)));
    return g;
}

// The double-single pair term of pair_term for a j-pair against one i-body.
template <bool ZERO_SOFT>
__device__ __forceinline__ void pair_term2(const JPair &j, float2 nxh, float2 nyh, float2 nzh,
                                           float2 nxl, float2 nyl, float2 nzl, float2 e2,
                                           float2 &ax, float2 &ay, float2 &az)
{
    const PairGeom g = pair_geom(j, nxh, nyh, nzh, nxl, nyl, nzl, e2);
    const float2 s = pair_scale<ZERO_SOFT>(g.r2, j.m);
    ax = fma2(g.dx, s, ax);
    ay = fma2(g.dy, s, ay);
    az = fma2(g.dz, s, az);
}

// pair_term2 for the pairs closer than a threshold: a lane whose r^2 (with
// the softening) is below thr adds nothing here and sets `hit`; the caller
// evaluates those pairs in double-single instead (pair_term_ds).  Such pairs carry the largest
// terms of a body's sum, so the FP32 rounding of their term and of the
// partial sums that hold them would dominate its error.
template <bool ZERO_SOFT>
__device__ __forceinline__ void pair_term2_excl(const JPair &j, float2 nxh, float2 nyh,
                                                float2 nzh, float2 nxl, float2 nyl, float2 nzl,
                                                float2 e2, float thr, float2 &ax, float2 &ay,
                                                float2 &az, bool &hit)
{
    const PairGeom g = pair_geom(j, nxh, nyh, nzh, nxl, nyl, nzl, e2);
    float2 s = pair_scale<ZERO_SOFT>(g.r2, j.m);
    const bool h0 = g.r2.x < thr, h1 = g.r2.y < thr;
    s.x = h0 ? 0.f : s.x;
    s.y = h1 ? 0.f : s.y;
    hit = hit || h0 || h1;
    ax = fma2(g.dx, s, ax);
    ay = fma2(g.dy, s, ay);
    az = fma2(g.dz, s, az);
}

// ---------------------------------------------------------------- double-single
// The pairs that leave the FP32 sum (pair_term2_excl) are evaluated in
// double-single arithmetic: an unevaluated sum hi + lo of two FP32 values,
// about 48 significant bits, built from error-free transformations (Knuth's
// two-sum, and the FMA product split).  On the FP32 pipe this costs a few
// dozen instructions per pair, far less than the few FP64 operations GB300's
// narrow FP64 pipe can issue per clock.
struct DS {
    float hi, lo;
};

// hi + lo with |lo| <= ulp(hi) / 2 (requires |a| >= |b| or a == 0).
__device__ __forceinline__ DS quick_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return DS{s, __fadd_rn(b, -__fsub_rn(s, a))};
}

__device__ __forceinline__ DS ds_add(DS a, DS b)
{
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return quick_two_sum(s, e);
}

// (a - b) of two normalised double-singles, exact to their ~2^-48 resolution.
__device__ __forceinline__ DS ds_sub(DS a, DS b) { return ds_add(a, DS{-b.hi, -b.lo}); }

// a * b as an unevaluated sum p + e (|e| small against |p|, not normalised):
// the FMA gives the exact error of the leading product.
__device__ __forceinline__ DS ds_mul_loose(DS a, DS b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return DS{p, e};
}

// The pair term m_j (r_j - r_i) / (|r_j - r_i|^2 + eps2)^(3/2) in
// double-single, from the double-single coordinates (relative to a common
// origin) and masses of the two bodies; t[0..2] = x, y, z components.
// r^2 = sum of the exact squares (FMA splits) with the low parts gathered in
// FP32; r^-3 = y0^3 (1 + 3h/2) from the MUFU estimate y0 and its residual
// h = 1 - r^2 y0^2 formed in double-single (h ~ 1e-7, so the dropped h^2 term
// is ~1e-14).  About 100 FP32 operations.  r^2 == 0 (coincident bodies, no
// softening) gives 0.
__device__ __forceinline__ void pair_term_ds(DS xj, DS yj, DS zj, DS mj, DS xi, DS yi, DS zi,
                                             DS eps2, DS t[3])
{
    const DS dx = ds_sub(xj, xi), dy = ds_sub(yj, yi), dz = ds_sub(zj, zi);
    const float px = __fmul_rn(dx.hi, dx.hi), py = __fmul_rn(dy.hi, dy.hi),
                pz = __fmul_rn(dz.hi, dz.hi);
    const float pex = __fmaf_rn(__fadd_rn(dx.hi, dx.hi), dx.lo, __fmaf_rn(dx.hi, dx.hi, -px));
    const float pey = __fmaf_rn(__fadd_rn(dy.hi, dy.hi), dy.lo, __fmaf_rn(dy.hi, dy.hi, -py));
    const float pez = __fmaf_rn(__fadd_rn(dz.hi, dz.hi), dz.lo, __fmaf_rn(dz.hi, dz.hi, -pz));
    float a, ae, b, be, c, ce;
    two_sum(px, py, a, ae);
    two_sum(a, pz, b, be);
    two_sum(b, eps2.hi, c, ce);
    const float lo = __fadd_rn(__fadd_rn(__fadd_rn(ae, be), __fadd_rn(ce, eps2.lo)),
                               __fadd_rn(__fadd_rn(pex, pey), pez));
    const DS r2 = quick_two_sum(c, lo);
    if (!(r2.hi > 0.f)) {
        t[0] = t[1] = t[2] = DS{0.f, 0.f};
        return;
    }
    const float y0 = rsqrt_mufu(r2.hi);
    const float u1 = __fmul_rn(r2.hi, y0);
    const float u1e = __fmaf_rn(r2.lo, y0, __fmaf_rn(r2.hi, y0, -u1));
    const float u2 = __fmul_rn(u1, y0);
    const float u2e = __fmaf_rn(u1e, y0, __fmaf_rn(u1, y0, -u2));
    const float h = __fsub_rn(__fsub_rn(1.0f, u2), u2e);  // 1 - r2 y0^2
    const float q = __fmul_rn(y0, y0);
    const float qe = __fmaf_rn(y0, y0, -q);
    const float q3 = __fmul_rn(q, y0);
    float q3e = __fmaf_rn(qe, y0, __fmaf_rn(q, y0, -q3));
    q3e = __fmaf_rn(q3, __fmul_rn(1.5f, h), q3e);
    const DS sc = ds_mul_loose(mj, DS{q3, q3e});
    t[0] = ds_mul_loose(sc, dx);
    t[1] = ds_mul_loose(sc, dy);
    t[2] = ds_mul_loose(sc, dz);
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
