// nb_direct_sorted.cu -- the mixed-precision all-pairs sum over Hilbert-sorted
// bodies with a near/far split decided per warp and per 32-body j-chunk, in
// packed FP32x2 arithmetic.
//
// Near/far.  The double-single displacement of the mixed pair term costs 6 of
// its 21 FP32 operations and is needed only when a pair is close compared with
// the distance of its bodies from the coordinate origin.  Here the origin
// moves to each warp: bodies are sorted along a Hilbert curve (the Barnes-Hut
// radix sort on Hilbert keys), so the 32*IPT consecutive bodies a warp owns are
// spatially compact.  The Hilbert curve never jumps between distant cells (the
// Morton curve does at every cell boundary), so its warp and chunk boxes are
// smaller: on a 65,536-body Plummer sphere 5 % of the chunk pairs are near
// instead of 11 %, and the kernel runs 4.7 % faster.  The warp takes the centre c of their bounding box as
// origin and stages every j-chunk (32 consecutive sorted bodies, one per lane)
// as a normalised double-single (S, E) of x - c.  A chunk whose bounding box
// lies at least kFarFactor * D from the warp's box (D: the warp box diameter)
// runs the plain FP32 term on S alone (15 FP32 operations + 1 MUFU), and a
// chunk at least kVeryFar * D away drops the folded Newton step too (12 + 1); other
// chunks take the full double-single term on S and E (21 + 1).  Decisions are
// uniform over the warp (no divergence) and a warp stages its own chunks in its
// own shared memory: no CTA-wide barrier.
//
// Packed arithmetic.  sm_100-class SMs execute FP32 add, multiply and FMA on
// register pairs (f32x2) at the FP32 pipe's lane rate but half the issue
// slots.  The scalar kernels issue ~24 instructions per interaction for 21 FP32
// operations and sit at the issue limit; here each thread evaluates two j at
// once (a j-pair, staged side by side in shared memory) against IPT i-bodies
// held as duplicated pairs, so the FP32 work issues as f32x2 and the FP32 pipe,
// not issue, bounds the kernel.  Every lane of an f32x2 operation rounds like
// its scalar counterpart.
//
// Error of a far term: S carries one FP32 rounding of x - c.  With
// |xi - c| <= D/2, |xj - c| <= r + D/2 and the subtraction's own rounding, the
// displacement error is at most 2^-24 (2r + D) <= 2^-24 r (2 + 1/kFarFactor)
// = 10 * 2^-24 r for kFarFactor = 1/8 -- about 6e-7 relative at worst, the
// order of the FP32 arithmetic of the term.  A very far term (gap >= D/4:
// displacement error <= 6 * 2^-24 r) also carries
// the MUFU rsqrt error three times, at most 3.7e-7 and on average -1.6e-8
// relative (measured over every FP32 input in [1, 4), i.e. every mantissa at
// both exponent parities); these terms are many and distant,
// so their errors average out: on a 65,536-body Plummer sphere the far /
// very-far factors (1/8, 1/4), (1/4, 1/4), (1/4, 1/2), (1/2, 1/2) and (1/2, 1)
// give the same errors (largest relative 5e-7 where S_i / |a_i| <= 10, RMS
// 2.5e-8), and (1/8, 1/4) the shortest kernel (2 % under (1/4, 1/2)).  Near terms keep the double-single
// displacement (absolute error ~2^-48 |x|) and the Newton step; every FP32
// accumulator takes 16 terms before its Kahan-compensated add, and the
// segments combine as a double-single.
#include "nb_internal.h"
#include "nb_check.cuh"
#include "nb_pair.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

namespace nb {
namespace {

constexpr int kChunk = 32;             // j-chunk = one body per lane
constexpr int kIpt = 2;                // 32-body i-chunks per warp (fixed: it sets the bits)
constexpr int kExactWarps = 8;         // warps of exact_pairs_kernel per main-kernel warp
constexpr int kExactRound = 64;        // left-out pairs evaluated per round and warp
constexpr int kResortEvals = 8;        // force evaluations per re-sort
constexpr bool kHilbertOrder = true;   // sort along the Hilbert curve (else Morton)

// Positions in sorted order relative to the root centre, split into
// double-single hi/lo parts (mass in hi.w), and the bounding box of the hi
// positions of every 32-body chunk (a warp is a chunk: box[2t] = min,
// box[2t+1] = max; lanes past n take the chunk's first body).  Blocks are
// multiples of 32 threads.
__global__ void split_sorted_kernel(const uint32_t *__restrict__ order,
                                    const double *__restrict__ x, const double *__restrict__ y,
                                    const double *__restrict__ z, const double *__restrict__ m,
                                    int n, const double *__restrict__ centre,
                                    float4 *__restrict__ hi, float4 *__restrict__ lo,
                                    float4 *__restrict__ box)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int chunk = i / kChunk, lane = threadIdx.x & 31;
    if (chunk * kChunk >= n) return;  // the whole warp is past n
    float p[3] = {0.f, 0.f, 0.f};
    const uint32_t o = i < n ? order[i] : 0u;
    if (i < n && NB_IN_RANGE(o, n)) {
        const double X = x[o] - centre[0], Y = y[o] - centre[1], Z = z[o] - centre[2];
        const float hx = __double2float_rn(X), hy = __double2float_rn(Y),
                    hz = __double2float_rn(Z);
        const float hm = __double2float_rn(m[o]);
        hi[i] = make_float4(hx, hy, hz, hm);
        lo[i] = make_float4(__double2float_rn(X - (double)hx), __double2float_rn(Y - (double)hy),
                            __double2float_rn(Z - (double)hz), __double2float_rn(m[o] - (double)hm));
        p[0] = hx;
        p[1] = hy;
        p[2] = hz;
    }
    float mn[3], mx[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float first = __shfl_sync(0xffffffffu, p[k], 0);
        mn[k] = mx[k] = i < n ? p[k] : first;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], s));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], s));
        }
    if (lane == 0) {
        box[2 * chunk] = make_float4(mn[0], mn[1], mn[2], 0.f);
        box[2 * chunk + 1] = make_float4(mx[0], mx[1], mx[2], 0.f);
    }
}

// A warp's box (the union of its IPT chunk boxes), its centre (the origin of
// every staged coordinate), and the squared thresholds of its near/far and
// left-out decisions.  Every product and sum is an explicit round-to-nearest
// intrinsic: direct_sorted_kernel and exact_pairs_kernel must take the same
// decisions bit for bit.
struct WarpGeom {
    float bmn[3], bmx[3], c[3];
    float thr2, thr2v, thr2x;
};

// The global cap of the left-out radius, squared: kExactSpacing times the
// mean body spacing of the root cube, (side^3 / n)^(1/3).  A warp of sparse
// bodies spread over a large box would otherwise get a radius that takes in
// whole dense regions, whose terms are a tiny part of its bodies' sums.
// per_n = kExactSpacing2 n^(-2/3), computed on the host.
__device__ __forceinline__ float exact_cap2(const double *__restrict__ root, float per_n)
{
    const float side = __double2float_rn(root[3]);
    return __fmul_rn(__fmul_rn(side, side), per_n);
}

float exact_cap_per_n(int n)
{
    return (float)((double)kExactSpacing2 / std::cbrt((double)n * (double)n));
}

template <int IPT>
__device__ __forceinline__ WarpGeom warp_geometry(const float4 *__restrict__ box, int tile0,
                                                  int nchunks, float far2, float cap2)
{
    WarpGeom g;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        g.bmn[a] = 3.0e38f;
        g.bmx[a] = -3.0e38f;
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k)
        if (tile0 + k < nchunks) {
            const float4 a = box[2 * (tile0 + k)], b = box[2 * (tile0 + k) + 1];
            g.bmn[0] = fminf(g.bmn[0], a.x); g.bmn[1] = fminf(g.bmn[1], a.y);
            g.bmn[2] = fminf(g.bmn[2], a.z);
            g.bmx[0] = fmaxf(g.bmx[0], b.x); g.bmx[1] = fmaxf(g.bmx[1], b.y);
            g.bmx[2] = fmaxf(g.bmx[2], b.z);
        }
    float side[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        g.c[a] = __fmul_rn(0.5f, __fadd_rn(g.bmn[a], g.bmx[a]));
        side[a] = __fsub_rn(g.bmx[a], g.bmn[a]);
    }
    const float diam2 = __fmaf_rn(side[2], side[2],
                                  __fmaf_rn(side[1], side[1], __fmul_rn(side[0], side[0])));
    g.thr2 = __fmul_rn(far2, diam2);        // far: double-single not needed
    g.thr2v = __fmul_rn(kVeryFar2, diam2);  // very far: Newton step not needed
    // Pairs closer than R leave the FP32 sum and are evaluated in double-single
    // by exact_pairs_kernel (only chunks nearer than R can hold one):
    // R = min(kExact D, kExactSpacing s, the global cap), s the mean body
    // spacing of the warp's box, (V / 64)^(1/3) with every side padded by D / 16
    // so that a flat box keeps its in-plane spacing.
    const float pad = __fmul_rn(0.0625f, sqrtf(diam2));
    const float vol = __fmul_rn(__fmul_rn(__fadd_rn(side[0], pad), __fadd_rn(side[1], pad)),
                                __fadd_rn(side[2], pad));
    const float s2 = exp2f(__fmul_rn(0.6666667f, log2f(__fmul_rn(vol, 1.0f / (32.0f * IPT)))));
    g.thr2x = fminf(fminf(__fmul_rn(kExact2, diam2), __fmul_rn(kExactSpacing2, s2)), cap2);
    return g;
}

// Squared gap between the warp's box and a j-chunk's box.
__device__ __forceinline__ float chunk_gap2(const WarpGeom &g, float4 jmn, float4 jmx)
{
    const float gx = fmaxf(0.f, fmaxf(__fsub_rn(jmn.x, g.bmx[0]), __fsub_rn(g.bmn[0], jmx.x)));
    const float gy = fmaxf(0.f, fmaxf(__fsub_rn(jmn.y, g.bmx[1]), __fsub_rn(g.bmn[1], jmx.y)));
    const float gz = fmaxf(0.f, fmaxf(__fsub_rn(jmn.z, g.bmx[2]), __fsub_rn(g.bmn[2], jmx.z)));
    return __fmaf_rn(gz, gz, __fmaf_rn(gy, gy, __fmul_rn(gx, gx)));
}

// One warp = 32*IPT consecutive sorted i-bodies (chunks tile0 .. tile0+IPT-1,
// lane l of chunk k holds body (tile0 + k) * 32 + l); blockIdx.y selects the
// j-chunks [y * seg_chunks, (y + 1) * seg_chunks).  Writes per-segment Kahan
// sums and compensations (sorted order).  Warps are independent: a warp whose
// chunks are all past n returns at once.
template <int WARPS, int IPT, bool ZERO_SOFT>
__global__ void __launch_bounds__(WARPS * 32)
direct_sorted_kernel(const float4 *__restrict__ hi, const float4 *__restrict__ lo,
                     const float4 *__restrict__ box, int n, int nchunks, float eps2,
                     int seg_chunks, float *__restrict__ psum, float *__restrict__ pcomp,
                     float far2, const double *__restrict__ root, float cap_per_n)
{
    __shared__ PairTile stage[WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int tile0 = (blockIdx.x * WARPS + w) * IPT;
    if (tile0 >= nchunks) return;
    PairTile &sg = stage[w];

    const WarpGeom gm = warp_geometry<IPT>(box, tile0, nchunks, far2, exact_cap2(root, cap_per_n));
    const float cx = gm.c[0], cy = gm.c[1], cz = gm.c[2];
    const float thr2 = gm.thr2, thr2v = gm.thr2v, thr2x = gm.thr2x;
    const float thrx = __fadd_rn(thr2x, eps2);

    // i-bodies relative to c, negated and duplicated into pairs
    float2 nsx[IPT], nsy[IPT], nsz[IPT], nex[IPT], ney[IPT], nez[IPT];
    float sx[IPT], sy[IPT], sz[IPT], qx[IPT], qy[IPT], qz[IPT];
    float2 ax[IPT], ay[IPT], az[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = (tile0 + k) * kChunk + lane;
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
        if (i < n) {
            h = hi[i];
            l = lo[i];
        }
        float S, E;
        rel_ds(h.x, l.x, cx, S, E);
        nsx[k] = dup2(-S);
        nex[k] = dup2(-E);
        rel_ds(h.y, l.y, cy, S, E);
        nsy[k] = dup2(-S);
        ney[k] = dup2(-E);
        rel_ds(h.z, l.z, cz, S, E);
        nsz[k] = dup2(-S);
        nez[k] = dup2(-E);
        sx[k] = sy[k] = sz[k] = 0.f;
        qx[k] = qy[k] = qz[k] = 0.f;
        ax[k] = ay[k] = az[k] = dup2(0.f);
    }
    const float2 e2 = dup2(eps2);

    const int jc0 = blockIdx.y * seg_chunks;
    const int jc1 = min(nchunks, jc0 + seg_chunks);
    // the lane's body of the next chunk, loaded one chunk ahead
    float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
    bool valid = jc0 < jc1 && jc0 * kChunk + lane < n;
    if (valid) {
        h = hi[jc0 * kChunk + lane];
        l = lo[jc0 * kChunk + lane];
    }
    for (int jc = jc0; jc < jc1; ++jc) {
        const float gap2 = chunk_gap2(gm, box[2 * jc], box[2 * jc + 1]);
        const bool far = gap2 > 0.f && gap2 >= thr2;
        const bool vfar = far && gap2 >= thr2v;
        const bool touch = !far && gap2 < thr2x;

        // lanes past n stage a massless body far away: its terms are exactly 0
        float Sx = 1.0e18f, Sy = 1.0e18f, Sz = 1.0e18f, Ex = 0.f, Ey = 0.f, Ez = 0.f, mj = 0.f;
        if (valid) {
            if (far) {  // S alone: x - c rounded once
                Sx = rel_s(h.x, l.x, cx);
                Sy = rel_s(h.y, l.y, cy);
                Sz = rel_s(h.z, l.z, cz);
            } else {
                rel_ds(h.x, l.x, cx, Sx, Ex);
                rel_ds(h.y, l.y, cy, Sy, Ey);
                rel_ds(h.z, l.z, cz, Sz, Ez);
            }
            mj = h.w;
        }
        __syncwarp();
        if (far)
            pair_tile_put_hi(sg, lane, Sx, Sy, Sz, mj);
        else
            pair_tile_put(sg, lane, Sx, Sy, Sz, mj, Ex, Ey, Ez);
        __syncwarp();
        valid = jc + 1 < jc1 && (jc + 1) * kChunk + lane < n;
        if (valid) {
            h = hi[(jc + 1) * kChunk + lane];
            l = lo[(jc + 1) * kChunk + lane];
        }

        if (vfar) {
#pragma unroll 4
            for (int p = 0; p < kChunk / 2; ++p) {
                const JPair j = pair_tile_get(sg, p);
#pragma unroll
                for (int k = 0; k < IPT; ++k)
                    pair_term2_far<false>(j, nsx[k], nsy[k], nsz[k], e2, ax[k], ay[k], az[k]);
            }
        } else if (far) {
#pragma unroll 4
            for (int p = 0; p < kChunk / 2; ++p) {
                const JPair j = pair_tile_get(sg, p);
#pragma unroll
                for (int k = 0; k < IPT; ++k)
                    pair_term2_far<true>(j, nsx[k], nsy[k], nsz[k], e2, ax[k], ay[k], az[k]);
            }
        } else if (touch) {
            // pairs closer than R are left to exact_pairs_kernel
            bool hit = false;
#pragma unroll 4
            for (int p = 0; p < kChunk / 2; ++p) {
                const JPair j = pair_tile_get(sg, p);
#pragma unroll
                for (int k = 0; k < IPT; ++k)
                    pair_term2_excl<ZERO_SOFT>(j, nsx[k], nsy[k], nsz[k], nex[k], ney[k], nez[k],
                                               e2, thrx, ax[k], ay[k], az[k], hit);
            }
        } else {
#pragma unroll 4
            for (int p = 0; p < kChunk / 2; ++p) {
                const JPair j = pair_tile_get(sg, p);
#pragma unroll
                for (int k = 0; k < IPT; ++k)
                    pair_term2<ZERO_SOFT>(j, nsx[k], nsy[k], nsz[k], nex[k], ney[k], nez[k], e2,
                                          ax[k], ay[k], az[k]);
            }
        }
        // every accumulator lane holds 16 terms of the chunk: fold them into the
        // Kahan sums (folding after every second chunk measured no faster, and
        // raised the largest relative error at N = 65,536 from 6e-7 to 9e-7)
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            kahan_add(sx[k], qx[k], ax[k].x + ax[k].y);
            kahan_add(sy[k], qy[k], ay[k].x + ay[k].y);
            kahan_add(sz[k], qz[k], az[k].x + az[k].y);
            ax[k] = ay[k] = az[k] = dup2(0.f);
        }
    }

    const size_t plane = (size_t)n;
    const size_t base = (size_t)blockIdx.y * 3 * plane;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = (tile0 + k) * kChunk + lane;
        if (i < n) {
            psum[base + i] = sx[k];
            psum[base + plane + i] = sy[k];
            psum[base + 2 * plane + i] = sz[k];
            pcomp[base + i] = qx[k];
            pcomp[base + plane + i] = qy[k];
            pcomp[base + 2 * plane + i] = qz[k];
        }
    }
}

// The pairs direct_sorted_kernel leaves out, in double-single.  It needs
// nothing from that kernel -- it takes the same decisions from the same data
// -- so it runs beside it on a second stream.  One CTA per warp of the main
// kernel (the same i-chunks and geometry) and kExactWarps warps in it: warp w
// takes the chunks jc = w (mod kExactWarps) that the main kernel tests for
// left-out pairs (not far, nearer than R), in increasing order, skipping those
// that no lane's i-body comes within R of.  For each it stages the chunk
// exactly as the main kernel does, recomputes the same r^2 bits, and marks the
// left-out pairs of each lane (bit 2p + u of mk[k]: tile body 2p + u against
// the lane's i-body k).  The marked pairs are evaluated one per lane,
// whole-warp, in rounds of kExactRound, and every lane adds its own bodies'
// terms into their double-single sums in increasing j; the warps' sums are
// then added in warp order.  The result does not depend on timing.
// ex[c n + i] = the FP64 value of body i's sum (sorted order), 0 if none.
// At most 64 registers (four CTAs per SM): beside direct_sorted_kernel, whose
// one-warp CTAs fill the register file, a leaner CTA displaces fewer of them.
template <int IPT>
__global__ void __launch_bounds__(kExactWarps * 32, 4)
exact_pairs_kernel(const float4 *__restrict__ hi, const float4 *__restrict__ lo,
                   const float4 *__restrict__ box, int n, int nchunks, float eps2, float far2,
                   double eps2d, const double *__restrict__ root, float cap_per_n,
                   double *__restrict__ ex)
{
    __shared__ PairTile stage[kExactWarps];
    __shared__ float ibody[IPT * 32][6];                      // (S, E) of x, y, z
    __shared__ uint16_t evt[kExactWarps][kExactRound];        // (k 32 + lane) << 5 | bit
    __shared__ float term[kExactWarps][kExactRound][6];       // (hi, lo) of x, y, z
    __shared__ float red[kExactWarps][IPT * 32][6];           // the warps' sums
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int wg = blockIdx.x;
    const int tile0 = wg * IPT;
    if (tile0 >= nchunks) return;  // the whole CTA
    PairTile &sg = stage[w];
    const WarpGeom gm = warp_geometry<IPT>(box, tile0, nchunks, far2, exact_cap2(root, cap_per_n));
    const float thrx = __fadd_rn(gm.thr2x, eps2);
    const float2 e2 = dup2(eps2);
    const DS e2ds{__double2float_rn(eps2d),
                  __double2float_rn(eps2d - (double)__double2float_rn(eps2d))};

    float2 nsx[IPT], nsy[IPT], nsz[IPT], nex[IPT], ney[IPT], nez[IPT];
    DS acc[IPT][3];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = (tile0 + k) * kChunk + lane;
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
        if (i < n) {
            h = hi[i];
            l = lo[i];
        }
        float S[3], E[3];
        rel_ds(h.x, l.x, gm.c[0], S[0], E[0]);
        rel_ds(h.y, l.y, gm.c[1], S[1], E[1]);
        rel_ds(h.z, l.z, gm.c[2], S[2], E[2]);
        nsx[k] = dup2(-S[0]); nex[k] = dup2(-E[0]);
        nsy[k] = dup2(-S[1]); ney[k] = dup2(-E[1]);
        nsz[k] = dup2(-S[2]); nez[k] = dup2(-E[2]);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (w == 0) {
                ibody[k * 32 + lane][2 * a] = S[a];
                ibody[k * 32 + lane][2 * a + 1] = E[a];
            }
            acc[k][a] = DS{0.f, 0.f};
        }
    }
    __syncthreads();

    // the lane's i-bodies' box, for the per-lane test of a chunk
    float lmn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, lmx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    bool ival[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        ival[k] = (tile0 + k) * kChunk + lane < n;
        if (ival[k]) {
            const float q[3] = {-nsx[k].x, -nsy[k].x, -nsz[k].x};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                lmn[a] = fminf(lmn[a], q[a]);
                lmx[a] = fmaxf(lmx[a], q[a]);
            }
        }
    }
    // The tests below only skip work, so they must never skip a chunk (or an
    // i-chunk of it) that holds a left-out pair: R grows by a slack far above
    // the FP32 roundings that separate the boxes (hi coordinates) from the
    // staged ones and the box distance from the pair's r^2 (softening included).
    const float Rw = sqrtf(gm.thr2x);
    const float cmag = fmaxf(fabsf(gm.c[0]), fmaxf(fabsf(gm.c[1]), fabsf(gm.c[2])));
    const float e2slack = 1e-6f * (gm.thr2x + eps2);

    int scan = w;
    while (true) {
        // the next chunk jc = w (mod kExactWarps) the main kernel tests, with
        // a lane whose bodies come within R of its box
        int jc = -1;
        while (scan < nchunks) {
            const int c = scan + kExactWarps * lane;
            bool t = false;
            float4 jmn = make_float4(0.f, 0.f, 0.f, 0.f), jmx = jmn;
            if (c < nchunks) {
                jmn = box[2 * c];
                jmx = box[2 * c + 1];
                const float gap2 = chunk_gap2(gm, jmn, jmx);
                t = !(gap2 > 0.f && gap2 >= gm.thr2) && gap2 < gm.thr2x;
            }
            uint32_t cand = __ballot_sync(0xffffffffu, t);
            while (cand) {
                const int src = __ffs(cand) - 1;
                cand &= cand - 1u;
                // this lane's bodies against the candidate's box (relative to c)
                const float bx0 = __shfl_sync(0xffffffffu, jmn.x, src) - gm.c[0];
                const float by0 = __shfl_sync(0xffffffffu, jmn.y, src) - gm.c[1];
                const float bz0 = __shfl_sync(0xffffffffu, jmn.z, src) - gm.c[2];
                const float bx1 = __shfl_sync(0xffffffffu, jmx.x, src) - gm.c[0];
                const float by1 = __shfl_sync(0xffffffffu, jmx.y, src) - gm.c[1];
                const float bz1 = __shfl_sync(0xffffffffu, jmx.z, src) - gm.c[2];
                const float gx = fmaxf(0.f, fmaxf(bx0 - lmx[0], lmn[0] - bx1));
                const float gy = fmaxf(0.f, fmaxf(by0 - lmx[1], lmn[1] - by1));
                const float gz = fmaxf(0.f, fmaxf(bz0 - lmx[2], lmn[2] - bz1));
                const float mag = cmag + fmaxf(fmaxf(fabsf(bx0), fabsf(bx1)),
                                               fmaxf(fmaxf(fabsf(by0), fabsf(by1)),
                                                     fmaxf(fabsf(bz0), fabsf(bz1))));
                const float Re = Rw + 1e-6f * mag;
                if (__any_sync(0xffffffffu, gx * gx + gy * gy + gz * gz <= Re * Re + e2slack)) {
                    jc = scan + kExactWarps * src;
                    break;
                }
            }
            if (jc >= 0) {
                scan = jc + kExactWarps;
                break;
            }
            scan += 32 * kExactWarps;
        }
        if (jc < 0) break;

        // the i-chunks with a body within R of the chunk's box (a lane's own
        // body against the box, the same slack)
        bool need[IPT];
        {
            const float4 jmn = box[2 * jc], jmx = box[2 * jc + 1];
            const float bx0 = jmn.x - gm.c[0], by0 = jmn.y - gm.c[1], bz0 = jmn.z - gm.c[2];
            const float bx1 = jmx.x - gm.c[0], by1 = jmx.y - gm.c[1], bz1 = jmx.z - gm.c[2];
            const float mag = cmag + fmaxf(fmaxf(fabsf(bx0), fabsf(bx1)),
                                           fmaxf(fmaxf(fabsf(by0), fabsf(by1)),
                                                 fmaxf(fabsf(bz0), fabsf(bz1))));
            const float Re = Rw + 1e-6f * mag;
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const float px = -nsx[k].x, py = -nsy[k].x, pz = -nsz[k].x;
                const float gx = fmaxf(0.f, fmaxf(bx0 - px, px - bx1));
                const float gy = fmaxf(0.f, fmaxf(by0 - py, py - by1));
                const float gz = fmaxf(0.f, fmaxf(bz0 - pz, pz - bz1));
                need[k] = __any_sync(0xffffffffu,
                                     ival[k] && gx * gx + gy * gy + gz * gz <= Re * Re + e2slack);
            }
        }

        // stage the chunk as the main kernel's near path does
        const int b = jc * kChunk + lane;
        float Sx = 1.0e18f, Sy = 1.0e18f, Sz = 1.0e18f, Ex = 0.f, Ey = 0.f, Ez = 0.f, mj = 0.f,
              ml = 0.f;
        if (b < n) {
            const float4 h = hi[b], l = lo[b];
            rel_ds(h.x, l.x, gm.c[0], Sx, Ex);
            rel_ds(h.y, l.y, gm.c[1], Sy, Ey);
            rel_ds(h.z, l.z, gm.c[2], Sz, Ez);
            mj = h.w;
            ml = l.w;
        }
        __syncwarp();
        pair_tile_put(sg, lane, Sx, Sy, Sz, mj, Ex, Ey, Ez);
        pair_tile_put_mlo(sg, lane, ml);
        __syncwarp();

        // the left-out pairs: the main kernel's r^2 test, same operands
        uint32_t mk[IPT];
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            mk[k] = 0u;
            if (!need[k]) continue;
            const int i = (tile0 + k) * kChunk + lane;
#pragma unroll 2
            for (int p = 0; p < kChunk / 2; ++p) {
                const JPair j = pair_tile_get(sg, p);
                const int j0 = jc * kChunk + 2 * p;
                const PairGeom g = pair_geom(j, nsx[k], nsy[k], nsz[k], nex[k], ney[k], nez[k], e2);
                const uint32_t b0 = (g.r2.x < thrx && i < n && j0 != i) ? 1u : 0u;
                const uint32_t b1 = (g.r2.y < thrx && i < n && j0 + 1 != i) ? 2u : 0u;
                mk[k] |= (b0 | b1) << (2 * p);
            }
        }
        // pairs numbered by (k, lane, bit)
        int off[IPT], total = 0;
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int c = __popc(mk[k]);
            int inc = c;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, inc, d);
                if (lane >= d) inc += v;
            }
            off[k] = total + inc - c;
            total += __shfl_sync(0xffffffffu, inc, 31);
        }
        for (int r = 0; r < total; r += kExactRound) {
            const int r1 = min(total, r + kExactRound);
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                uint32_t m = mk[k];
                for (int e = off[k]; m != 0u; ++e) {
                    const int bit = __ffs(m) - 1;
                    m &= m - 1u;
                    if (e >= r && e < r1) evt[w][e - r] = (uint16_t)(((k * 32 + lane) << 5) | bit);
                }
            }
            __syncwarp();
            for (int e = lane; e < r1 - r; e += 32) {
                const int code = evt[w][e];
                const int il = code >> 5, bit = code & 31;
                const int p = bit >> 1;
                const bool u = bit & 1;
                const float4 A = sg.s[p], B = sg.t[p], C = sg.e[p];
                const float2 F = sg.f[p], M = sg.g[p];
                const float *q = ibody[il];
                DS t[3];
                pair_term_ds(DS{u ? A.y : A.x, u ? C.y : C.x}, DS{u ? A.w : A.z, u ? C.w : C.z},
                             DS{u ? B.y : B.x, u ? F.y : F.x}, DS{u ? B.w : B.z, u ? M.y : M.x},
                             DS{q[0], q[1]}, DS{q[2], q[3]}, DS{q[4], q[5]}, e2ds, t);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    term[w][e][2 * a] = t[a].hi;
                    term[w][e][2 * a + 1] = t[a].lo;
                }
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                uint32_t m = mk[k];
                for (int e = off[k]; m != 0u; ++e) {
                    m &= m - 1u;
                    if (e >= r && e < r1)
#pragma unroll
                        for (int a = 0; a < 3; ++a)
                            acc[k][a] = ds_add(acc[k][a],
                                               DS{term[w][e - r][2 * a], term[w][e - r][2 * a + 1]});
                }
            }
            __syncwarp();
        }
    }

    // the warps' sums in warp order
#pragma unroll
    for (int k = 0; k < IPT; ++k)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            red[w][k * 32 + lane][2 * a] = acc[k][a].hi;
            red[w][k * 32 + lane][2 * a + 1] = acc[k][a].lo;
        }
    __syncthreads();
    if (w != 0) return;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = (tile0 + k) * kChunk + lane;
        DS sum[3] = {DS{0.f, 0.f}, DS{0.f, 0.f}, DS{0.f, 0.f}};
        for (int v = 0; v < kExactWarps; ++v)
#pragma unroll
            for (int a = 0; a < 3; ++a)
                sum[a] = ds_add(sum[a], DS{red[v][k * 32 + lane][2 * a],
                                           red[v][k * 32 + lane][2 * a + 1]});
        if (i < n)
#pragma unroll
            for (int a = 0; a < 3; ++a)
                ex[(size_t)a * n + i] = (double)sum[a].hi + (double)sum[a].lo;
    }
}

// a[order[i]] = G * (sum_s (sum_s - comp_s) + ex_i) for sorted body i: a
// double-single sum over the segments, plus the left-out pairs (ex: none when
// NULL), scaled in FP64.
__global__ void combine_sorted_kernel(const float *__restrict__ psum,
                                      const float *__restrict__ pcomp, int n, int segments,
                                      double G, const uint32_t *__restrict__ order,
                                      const double *__restrict__ ex, double *__restrict__ ax,
                                      double *__restrict__ ay, double *__restrict__ az)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t plane = (size_t)n;
    float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
    // the loads of several segments go out before their (ordered) sums
#pragma unroll 8
    for (int s = 0; s < segments; ++s) {
        const size_t base = (size_t)s * 3 * plane;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            ds_add_kahan(hi[c], lo[c], psum[base + c * plane + i], pcomp[base + c * plane + i]);
    }
    const uint32_t o = order[i];
    if (!NB_IN_RANGE(o, n)) return;
    double a[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        a[c] = ((double)hi[c] + (double)lo[c]) + (ex ? ex[c * plane + i] : 0.0);
    ax[o] = G * a[0];
    ay[o] = G * a[1];
    az[o] = G * a[2];
}

// CTA shapes the autotuner times: warps per CTA x 32-body chunks per warp.
// Warps stage their own j-chunks, so the CTA size matters only for
// scheduling: with one- or two-warp CTAs a slow warp (many near chunks) holds
// fewer idle warp slots until its CTA retires (1.2 % faster at N = 65,536).
// Chunks per warp (the warp's box, hence its near/far decisions and origin)
// and the j-segments (sorted_plan_for_shape) are the same for every shape, so
// the timed choice never changes the bits of a result.
struct SortedShape {
    int warps, ipt;
};
constexpr SortedShape kSortedShapes[] = {{4, kIpt}, {8, kIpt}, {2, kIpt}, {1, kIpt}};
constexpr int kNumSortedShapes = sizeof(kSortedShapes) / sizeof(kSortedShapes[0]);

template <int W, int I>
int sorted_slots()
{
    static const int slots = [] {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, (const void *)direct_sorted_kernel<W, I, false>, W * 32, 0);
        return std::max(1, per_sm) * device_props().num_sms;
    }();
    return slots;
}

int sorted_slots_for(int warps, int ipt)
{
    if (warps == 4 && ipt == 2) return sorted_slots<4, 2>();
    if (warps == 8 && ipt == 2) return sorted_slots<8, 2>();
    if (warps == 2 && ipt == 2) return sorted_slots<2, 2>();
    if (warps == 1 && ipt == 2) return sorted_slots<1, 2>();
    return 0;
}

template <int W, int I>
void launch_sorted_shape(dim3 grid, cudaStream_t st, const float4 *hi, const float4 *lo,
                         const float4 *box, int n, double eps2, int seg_chunks, float *psum,
                         float *pcomp, const double *root)
{
    const int nchunks = (n + kChunk - 1) / kChunk;
    if (eps2 > 0.0)
        direct_sorted_kernel<W, I, false><<<grid, W * 32, 0, st>>>(
            hi, lo, box, n, nchunks, (float)eps2, seg_chunks, psum, pcomp, kFarFactor2, root,
            exact_cap_per_n(n));
    else
        direct_sorted_kernel<W, I, true><<<grid, W * 32, 0, st>>>(
            hi, lo, box, n, nchunks, 0.0f, seg_chunks, psum, pcomp, kFarFactor2, root,
            exact_cap_per_n(n));
}

// DirectPlan fields here: block = threads per CTA (32 * warps), ipt = chunks
// per warp, seg_tiles = j-chunks per segment.
bool launch_sorted(const DirectPlan &p, cudaStream_t st, const float4 *hi, const float4 *lo,
                   const float4 *box, int n, double eps2, float *psum, float *pcomp,
                   const double *root)
{
    const int warps = p.block / 32;
    const int nchunks = (n + kChunk - 1) / kChunk;
    const int per_cta = warps * p.ipt;
    const dim3 grid((nchunks + per_cta - 1) / per_cta, p.segments);
    if (warps == 4 && p.ipt == 2)
        launch_sorted_shape<4, 2>(grid, st, hi, lo, box, n, eps2, p.seg_tiles, psum, pcomp,
                                  root);
    else if (warps == 8 && p.ipt == 2)
        launch_sorted_shape<8, 2>(grid, st, hi, lo, box, n, eps2, p.seg_tiles, psum, pcomp,
                                  root);
    else if (warps == 2 && p.ipt == 2)
        launch_sorted_shape<2, 2>(grid, st, hi, lo, box, n, eps2, p.seg_tiles, psum, pcomp,
                                  root);
    else if (warps == 1 && p.ipt == 2)
        launch_sorted_shape<1, 2>(grid, st, hi, lo, box, n, eps2, p.seg_tiles, psum, pcomp,
                                  root);
    else
        return false;
    return true;
}

// The j-split is modelled on one-warp CTAs of two chunks for every shape
// (segments of at least 8 chunks, 256 j), so it depends on n alone.
DirectPlan sorted_plan_for_shape(int n, int warps, int ipt)
{
    DirectPlan p;
    p.block = warps * 32;
    p.ipt = ipt;
    const int nchunks = (n + kChunk - 1) / kChunk;
    const int iblocks = (nchunks + 1) / 2;
    const int units = std::max(1, nchunks / 8);
    const int s = direct_pick_segments(iblocks, units, sorted_slots_for(1, 2));
    p.seg_tiles = (nchunks + s - 1) / s;
    p.segments = (nchunks + p.seg_tiles - 1) / p.seg_tiles;
    return p;
}

std::mutex g_sorted_mutex;
std::map<int, DirectPlan> g_sorted_tuned;

} // namespace

void SortedBuffers::release()
{
    hi.release();
    lo.release();
    partials.release();
    boxes.release();
    exact.release();
    if (side) cudaStreamDestroy(side);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    side = nullptr;
    fork = join = nullptr;
    if (sorter) bh_destroy(sorter);
    sorter = nullptr;
    order = nullptr;
    centre = nullptr;
    order_n = -1;
}

bool direct_sorted_enabled(int n, int flags)
{
    if (flags & NB_FLAG_MIXED_UNSORTED) return false;
    if (flags & NB_FLAG_MIXED_SORTED) return n > 0;
    static const bool on = [] {
        const char *e = std::getenv("NB_DIRECT_SORTED");
        return !(e && std::strcmp(e, "0") == 0);
    }();
    return on && n >= kSortedMinBodies;
}

// Warps of the main kernel (one per kIpt i-chunks).
static int sorted_warps(int n) { return ((n + kChunk - 1) / kChunk + kIpt - 1) / kIpt; }

static nb_status run_sorted(const DirectPlan &p, const float4 *hi, const float4 *lo, int n,
                            double eps2, SortedBuffers &b, cudaStream_t st, float **psum_out)
{
    NB_TRY(b.partials.reserve(sizeof(float) * 6 * (size_t)n * p.segments));
    float *psum = b.partials.as<float>();
    float *pcomp = psum + 3 * (size_t)n * p.segments;
    if (!launch_sorted(p, st, hi, lo, b.boxes.as<float4>(), n, eps2, psum, pcomp, b.centre))
        return fail(NB_ERR_UNSUPPORTED, "direct_mixed_sorted: unsupported tile shape");
    NB_LAUNCH_CHECK();
    *psum_out = psum;
    return NB_OK;
}

// The left-out pairs, into b.exact (3 n doubles), on b.side: the kernel
// waits for the staging on st (fork) and st waits for it before the combine
// (join).  The side stream has the highest priority, so the exact CTAs start
// at once and their longest chains run while the main kernel fills the GPU.
static nb_status launch_exact_pairs(const float4 *hi, const float4 *lo, int n, double eps2,
                                    SortedBuffers &b, cudaStream_t st)
{
    NB_TRY(b.exact.reserve(sizeof(double) * 3 * (size_t)n));
    if (!b.side) {
        int least = 0, greatest = 0;
        NB_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        NB_CUDA_TRY(cudaStreamCreateWithPriority(&b.side, cudaStreamNonBlocking, greatest));
        NB_CUDA_TRY(cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming));
        NB_CUDA_TRY(cudaEventCreateWithFlags(&b.join, cudaEventDisableTiming));
    }
    NB_CUDA_TRY(cudaEventRecord(b.fork, st));
    NB_CUDA_TRY(cudaStreamWaitEvent(b.side, b.fork, 0));
    const int nchunks = (n + kChunk - 1) / kChunk;
    exact_pairs_kernel<kIpt><<<sorted_warps(n), kExactWarps * 32, 0, b.side>>>(
        hi, lo, b.boxes.as<float4>(), n, nchunks, eps2 > 0.0 ? (float)eps2 : 0.0f, kFarFactor2,
        eps2 > 0.0 ? eps2 : 0.0, b.centre, exact_cap_per_n(n), b.exact.as<double>());
    NB_LAUNCH_CHECK();
    NB_CUDA_TRY(cudaEventRecord(b.join, b.side));
    return NB_OK;
}

// Times every CTA shape, kernel and combine together (the combine writes the
// real outputs, which the evaluation then overwrites), and records the
// fastest plan for this n.
static nb_status autotune_sorted(const float4 *hi, const float4 *lo, int n, double eps2,
                                 double G, const uint32_t *order, double *ax, double *ay,
                                 double *az, SortedBuffers &b, cudaStream_t st, DirectPlan *best)
{
    cudaEvent_t e0, e1;
    NB_CUDA_TRY(cudaEventCreate(&e0));
    NB_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    // Above 2^18 bodies every shape is timed on all i-bodies against the first
    // 512 j-chunks only (one segment): an evaluation there takes 0.1 s and more.
    const bool probe = n > (1 << 18);
    for (int k = 0; k < kNumSortedShapes; ++k) {
        const DirectPlan p = sorted_plan_for_shape(n, kSortedShapes[k].warps, kSortedShapes[k].ipt);
        {
            DirectPlan t = p;
            if (probe) {
                t.segments = 1;
                t.seg_tiles = std::min(p.seg_tiles * p.segments, 512);
            }
            float *psum = nullptr;
            NB_TRY(run_sorted(t, hi, lo, n, eps2, b, st, &psum));
            cudaEventRecord(e0, st);
            for (int r = 0; r < 2; ++r) {
                NB_TRY(run_sorted(t, hi, lo, n, eps2, b, st, &psum));
                combine_sorted_kernel<<<(n + 255) / 256, 256, 0, st>>>(
                    psum, psum + 3 * (size_t)n * t.segments, n, t.segments, G, order, nullptr,
                    ax, ay, az);
                NB_LAUNCH_CHECK();
            }
            cudaEventRecord(e1, st);
            NB_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best_ms) {
                best_ms = ms;
                *best = p;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lock(g_sorted_mutex);
    g_sorted_tuned[n] = *best;
    return NB_OK;
}

nb_status direct_mixed_sorted(const double *x, const double *y, const double *z, const double *m,
                              int n, double G, double eps2, double *ax, double *ay, double *az,
                              SortedBuffers &b, cudaStream_t st, const KernelTimer *timer)
{
    if (n <= 0) return NB_OK;
    NvtxRange range("direct_sorted");
    if (!b.sorter) b.sorter = bh_create();
    if (b.order_n != n || b.evals_since_sort >= kResortEvals) {
        // 2^30 cells: far smaller than a 32-body chunk
        if (kHilbertOrder)
            NB_TRY(bh_hilbert_order(b.sorter, x, y, z, n, st, &b.order, &b.centre));
        else
            NB_TRY(bh_morton_order(b.sorter, x, y, z, n, 10, st, &b.order, &b.centre));
        b.order_n = n;
        b.evals_since_sort = 0;
    }
    ++b.evals_since_sort;
    const uint32_t *order = b.order;
    const double *centre = b.centre;
    const int nchunks = (n + kChunk - 1) / kChunk;
    NB_TRY(b.hi.reserve(sizeof(float4) * (size_t)n));
    NB_TRY(b.lo.reserve(sizeof(float4) * (size_t)n));
    NB_TRY(b.boxes.reserve(sizeof(float4) * 2 * (size_t)nchunks));
    float4 *hi = b.hi.as<float4>(), *lo = b.lo.as<float4>();
    split_sorted_kernel<<<(n + 255) / 256, 256, 0, st>>>(order, x, y, z, m, n, centre, hi, lo,
                                                         b.boxes.as<float4>());
    NB_LAUNCH_CHECK();
    DirectPlan p;
    bool tuned;
    {
        std::lock_guard<std::mutex> lock(g_sorted_mutex);
        auto it = g_sorted_tuned.find(n);
        tuned = it != g_sorted_tuned.end();
        if (tuned) p = it->second;
    }
    if (!tuned) {
        const char *e = std::getenv("NB_AUTOTUNE");
        if (!(e && std::strcmp(e, "0") == 0))
            NB_TRY(autotune_sorted(hi, lo, n, eps2, G, order, ax, ay, az, b, st, &p));
        else p = sorted_plan_for_shape(n, 1, 2);
    }
    NB_TRY(launch_exact_pairs(hi, lo, n, eps2, b, st));
    if (timer && timer->start) NB_CUDA_TRY(cudaEventRecord(timer->start, st));
    float *psum = nullptr;
    NB_TRY(run_sorted(p, hi, lo, n, eps2, b, st, &psum));
    if (timer && timer->stop) NB_CUDA_TRY(cudaEventRecord(timer->stop, st));
    float *pcomp = psum + 3 * (size_t)n * p.segments;
    NB_CUDA_TRY(cudaStreamWaitEvent(st, b.join, 0));
    combine_sorted_kernel<<<(n + 255) / 256, 256, 0, st>>>(psum, pcomp, n, p.segments, G, order,
                                                          b.exact.as<double>(), ax, ay, az);
    NB_LAUNCH_CHECK();
    return NB_OK;
}

} // namespace nb
