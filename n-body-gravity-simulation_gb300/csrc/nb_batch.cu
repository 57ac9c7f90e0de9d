// nb_batch.cu -- many independent systems of uneven N in one persistent launch.
//
// No reference counterpart: the reference simulates one system per process.
// A batch holds the bodies of every system in one pool of FP64 planes
// (x y z vx vy vz ax ay az m, 80 B/body) plus the float4 hi/lo mirror of the
// mixed pair term (32 B/body).  A system is a descriptor {first, n, ipt}: its
// bodies are pool slots [first, first + n).
//
// Forces.  The work queue holds one item per (system, 32*ipt i-bodies); items
// are ordered by cost, largest first.  A persistent kernel (a fixed grid of
// resident CTAs) lets every warp take the next item with one atomicAdd and
// sum its system's j-bodies in tiles of 32 staged in the warp's own slice of
// shared memory: the same double-single / folded-Newton pair term as the
// single-system kernel, evaluated on j-pairs in packed f32x2 arithmetic, and a
// Kahan-compensated add after every tile.  Each item writes only its own
// i-bodies' accelerations, after summing j in index order, so a system's
// result does not depend on what else is in the batch or on which warp ran
// which item: a system gives the same bits alone and in any mix.
//
// ipt (i-bodies per lane) is chosen per N bucket (powers of two) by an
// autotuner that times the candidates on the batch's own systems.
#include "nb_internal.h"
#include "nb_check.cuh"
#include "nb_curve.cuh"
#include "nb_pair.cuh"

#include <algorithm>
#include <cmath>

namespace nb {
namespace {

constexpr int kBatchBlock = 128;  // 4 warps
constexpr int kBatchWarps = kBatchBlock / 32;
// Systems of at least this many bodies take two i-chunks per warp item in the
// sorted variant (a fixed rule of n, so that a system's item shapes -- and its
// bits -- do not depend on the other systems of the batch).
constexpr int kSortedIpt2Min = 2048;

template <int IPT, bool ZERO_SOFT>
__device__ __forceinline__ void batch_item(const float4 *__restrict__ hi,
                                           const float4 *__restrict__ lo, const SysDesc &sd,
                                           int i0, float eps2, double G, double *__restrict__ ax,
                                           double *__restrict__ ay, double *__restrict__ az,
                                           PairTile &pt)
{
    const int lane = threadIdx.x & 31;
    // i-bodies negated and duplicated into f32x2 pairs
    float2 nxh[IPT], nyh[IPT], nzh[IPT], nxl[IPT], nyl[IPT], nzl[IPT];
    float sx[IPT], sy[IPT], sz[IPT], cx[IPT], cy[IPT], cz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = i0 + k * 32 + lane;
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
        if (i < sd.n) {
            h = hi[sd.first + i];
            l = lo[sd.first + i];
        }
        nxh[k] = dup2(-h.x); nyh[k] = dup2(-h.y); nzh[k] = dup2(-h.z);
        nxl[k] = dup2(-l.x); nyl[k] = dup2(-l.y); nzl[k] = dup2(-l.z);
        sx[k] = sy[k] = sz[k] = 0.f;
        cx[k] = cy[k] = cz[k] = 0.f;
    }
    const float2 e2 = dup2(eps2);
    for (int t0 = 0; t0 < sd.n; t0 += 32) {
        const int j = t0 + lane;
        float4 h = far_body(), l = make_float4(0.f, 0.f, 0.f, 0.f);
        if (j < sd.n) {
            h = hi[sd.first + j];
            l = lo[sd.first + j];
        }
        __syncwarp();
        pair_tile_put(pt, lane, h.x, h.y, h.z, h.w, l.x, l.y, l.z);
        __syncwarp();
        float2 ax_[IPT], ay_[IPT], az_[IPT];
#pragma unroll
        for (int k = 0; k < IPT; ++k) ax_[k] = ay_[k] = az_[k] = dup2(0.f);
#pragma unroll 2
        for (int p = 0; p < 16; ++p) {
            const JPair jp = pair_tile_get(pt, p);
#pragma unroll
            for (int k = 0; k < IPT; ++k)
                pair_term2<ZERO_SOFT>(jp, nxh[k], nyh[k], nzh[k], nxl[k], nyl[k], nzl[k], e2,
                                      ax_[k], ay_[k], az_[k]);
        }
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            kahan_add(sx[k], cx[k], ax_[k].x + ax_[k].y);
            kahan_add(sy[k], cy[k], ay_[k].x + ay_[k].y);
            kahan_add(sz[k], cz[k], az_[k].x + az_[k].y);
        }
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = i0 + k * 32 + lane;
        if (i < sd.n) {
            ax[sd.first + i] = G * ((double)sx[k] - (double)cx[k]);
            ay[sd.first + i] = G * ((double)sy[k] - (double)cy[k]);
            az[sd.first + i] = G * ((double)sz[k] - (double)cz[k]);
        }
    }
}

template <bool ZERO_SOFT>
__global__ void __launch_bounds__(kBatchBlock)
batch_force_kernel(const float4 *__restrict__ hi, const float4 *__restrict__ lo,
                   const SysDesc *__restrict__ sys, const WorkItem *__restrict__ items,
                   int num_items, int *__restrict__ counter, float eps2, double G,
                   double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az,
                   int total)
{
    __shared__ PairTile tiles[kBatchWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    while (true) {
        int item = 0;
        if (lane == 0) item = atomicAdd(counter, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= num_items) break;
        const WorkItem w = items[item];
        const SysDesc sd = sys[w.sys];
        if (!NB_IN_RANGE(sd.first, total) || !NB_IN_RANGE(sd.first + sd.n - 1, total)) continue;
        switch (sd.ipt) {
        case 1:
            batch_item<1, ZERO_SOFT>(hi, lo, sd, w.i0, eps2, G, ax, ay, az,
                                     tiles[warp]);
            break;
        case 2:
            batch_item<2, ZERO_SOFT>(hi, lo, sd, w.i0, eps2, G, ax, ay, az,
                                     tiles[warp]);
            break;
        default:
            batch_item<4, ZERO_SOFT>(hi, lo, sd, w.i0, eps2, G, ax, ay, az,
                                     tiles[warp]);
            break;
        }
    }
}

int batch_grid()
{
    // a function-local static: initialised once, thread-safe
    static const int grid = [] {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, (const void *)batch_force_kernel<false>, kBatchBlock, 0);
        return std::max(1, per_sm) * device_props().num_sms;
    }();
    return grid;
}

// ---------------------------------------------------------------- sorted
// The Hilbert-sorted variant (ensemble): every system's bodies are sorted
// along a Hilbert curve through the cube around that system alone, so a
// 32-body chunk of sorted bodies is spatially compact; a warp item is one
// i-chunk, its box centre is the origin of its staged j-chunks, and j-chunks
// far from its box take the plain FP32 term (see nb_direct_sorted.cu).  Every
// quantity a system's result depends on -- its order, its centre, its chunk
// boxes, each item's classification -- is computed from that system alone, so
// a system still gives the same bits alone and in any mix.

// body_sys[i] = s for the bodies of system s; chunk table entries (first
// body, count) of its 32-body chunks.
__global__ void batch_layout_kernel(const SysDesc *__restrict__ sys, int *__restrict__ body_sys,
                                    int2 *__restrict__ chunks)
{
    const SysDesc sd = sys[blockIdx.x];
    for (int i = threadIdx.x; i < sd.n; i += blockDim.x) body_sys[sd.first + i] = blockIdx.x;
    const int nch = (sd.n + 31) / 32;
    for (int c = threadIdx.x; c < nch; c += blockDim.x)
        chunks[sd.chunk0 + c] = make_int2(sd.first + 32 * c, min(32, sd.n - 32 * c));
}

// geom[s] = (centre x, y, z, side) of the cube around system s: one block per
// system, min/max on order-preserving integer keys.
__global__ void __launch_bounds__(256)
batch_geom_kernel(const SysDesc *__restrict__ sys, const double *__restrict__ x,
                  const double *__restrict__ y, const double *__restrict__ z,
                  double4 *__restrict__ geom)
{
    constexpr long long kMax = 0x7fffffffffffffffll, kMin = -kMax - 1;
    __shared__ long long sh[6][8];
    const SysDesc sd = sys[blockIdx.x];
    const double *ax[3] = {x, y, z};
    long long v[6] = {kMax, kMax, kMax, kMin, kMin, kMin};
    for (int i = threadIdx.x; i < sd.n; i += 256)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double q = ax[c][sd.first + i];
            v[c] = min(v[c], order_key(q, kMax));
            v[c + 3] = max(v[c + 3], order_key(q, kMin));
        }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = min(v[c], __shfl_xor_sync(0xffffffffu, v[c], o));
            v[c + 3] = max(v[c + 3], __shfl_xor_sync(0xffffffffu, v[c + 3], o));
        }
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < 6; ++c) sh[c][warp] = v[c];
    __syncthreads();
    if (threadIdx.x != 0) return;
    double lo[3], hi[3], side = 0.0;
    for (int c = 0; c < 3; ++c) {
        long long a = sh[c][0], b = sh[c + 3][0];
        for (int w = 1; w < 8; ++w) {
            a = min(a, sh[c][w]);
            b = max(b, sh[c + 3][w]);
        }
        // only NaN coordinates: a unit cube at the origin
        lo[c] = a == kMax ? 0.0 : key_value(a);
        hi[c] = b == kMin ? 0.0 : key_value(b);
        side = fmax(side, hi[c] - lo[c]);
    }
    side = fmax(side, 1e-30) * (1.0 + 1e-6);
    geom[blockIdx.x] = make_double4(0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]),
                                    0.5 * (lo[2] + hi[2]), side);
}

// keys[i] = (system, Hilbert index in its cube) in the top sys_bits + 30 bits,
// vals[i] = i: a stable sort keeps every system in its own index range.
__global__ void __launch_bounds__(256)
batch_key_kernel(const double *__restrict__ x, const double *__restrict__ y,
                 const double *__restrict__ z, const int *__restrict__ body_sys,
                 const double4 *__restrict__ geom, int n, int key_shift,
                 uint64_t *__restrict__ keys, uint32_t *__restrict__ vals)
{
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const int s = body_sys[i];
    const double4 g = geom[s];
    const double scale = 1024.0 / g.w;
    const double p[3] = {x[i], y[i], z[i]}, c[3] = {g.x, g.y, g.z};
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double f = floor((p[k] - (c[k] - 0.5 * g.w)) * scale);
        q[k] = (uint32_t)fmin(fmax(f, 0.0), 1023.0);
    }
    const uint64_t key = ((uint64_t)s << 30) | hilbert_index30(q[0], q[1], q[2]);
    keys[i] = key << key_shift;
    vals[i] = (uint32_t)i;
}

// Sorted positions relative to their system's centre, split into hi/lo
// (double-single) parts; mass in hi.w.
__global__ void __launch_bounds__(256)
batch_split_sorted_kernel(const uint32_t *__restrict__ order, const double *__restrict__ x,
                          const double *__restrict__ y, const double *__restrict__ z,
                          const double *__restrict__ m, const int *__restrict__ body_sys,
                          const double4 *__restrict__ geom, int n, float4 *__restrict__ hi,
                          float4 *__restrict__ lo)
{
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = order[i];
    if (!NB_IN_RANGE(o, n)) return;
    const double4 g = geom[body_sys[i]];
    const double X = x[o] - g.x, Y = y[o] - g.y, Z = z[o] - g.z;
    const float hx = __double2float_rn(X), hy = __double2float_rn(Y), hz = __double2float_rn(Z);
    hi[i] = make_float4(hx, hy, hz, __double2float_rn(m[o]));
    lo[i] = make_float4(__double2float_rn(X - (double)hx), __double2float_rn(Y - (double)hy),
                        __double2float_rn(Z - (double)hz), 0.0f);
}

// Bounding box of every chunk (one warp per chunk): box[2g] = min, box[2g+1] = max.
__global__ void batch_chunk_box_kernel(const float4 *__restrict__ hi,
                                       const int2 *__restrict__ chunks, int num_chunks,
                                       float4 *__restrict__ box)
{
    const int g = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (g >= num_chunks) return;
    const int2 ch = chunks[g];
    const float4 p = hi[ch.x + (lane < ch.y ? lane : 0)];
    float mn[3] = {p.x, p.y, p.z}, mx[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    if (lane == 0) {
        box[2 * g] = make_float4(mn[0], mn[1], mn[2], 0.f);
        box[2 * g + 1] = make_float4(mx[0], mx[1], mx[2], 0.f);
    }
}

// One warp item = IPT consecutive 32-body i-chunks of a system (lane l holds
// body l of each) against all its j-chunks.  The items's box (the union of its
// i-chunk boxes, diameter D) is the origin of the staged j-chunks: near chunks
// (closer than D/8) take the double-single term, far ones the plain FP32
// term, very far ones (D/4) the plain term without the Newton step; each
// chunk's 16 terms per accumulator lane are folded into Kahan sums.
template <int IPT, bool ZERO_SOFT>
__device__ __forceinline__ void batch_sorted_item(const float4 *__restrict__ hi,
                                                  const float4 *__restrict__ lo,
                                                  const float4 *__restrict__ box,
                                                  const SysDesc &sd, int i0, float eps2,
                                                  double G, const uint32_t *__restrict__ order,
                                                  double *__restrict__ ax,
                                                  double *__restrict__ ay,
                                                  double *__restrict__ az, PairTile &sg,
                                                  int total)
{
    const int lane = threadIdx.x & 31;
    const int nch = (sd.n + 31) / 32;
    const int ic0 = i0 / 32;
    float4 bmn = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f);
    float4 bmx = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.f);
#pragma unroll
    for (int k = 0; k < IPT; ++k)
        if (ic0 + k < nch) {
            const float4 a = box[2 * (sd.chunk0 + ic0 + k)], b = box[2 * (sd.chunk0 + ic0 + k) + 1];
            bmn = make_float4(fminf(bmn.x, a.x), fminf(bmn.y, a.y), fminf(bmn.z, a.z), 0.f);
            bmx = make_float4(fmaxf(bmx.x, b.x), fmaxf(bmx.y, b.y), fmaxf(bmx.z, b.z), 0.f);
        }
    const float diam2 = (bmx.x - bmn.x) * (bmx.x - bmn.x) + (bmx.y - bmn.y) * (bmx.y - bmn.y) +
                        (bmx.z - bmn.z) * (bmx.z - bmn.z);
    const float thr2 = kFarFactor2 * diam2, thr2v = kVeryFar2 * diam2;
    const float cx = 0.5f * (bmn.x + bmx.x), cy = 0.5f * (bmn.y + bmx.y),
                cz = 0.5f * (bmn.z + bmx.z);
    float2 nsx[IPT], nsy[IPT], nsz[IPT], nex[IPT], ney[IPT], nez[IPT];
    float sx[IPT], sy[IPT], sz[IPT], qx[IPT], qy[IPT], qz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = i0 + 32 * k + lane;
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
        if (i < sd.n) {
            h = hi[sd.first + i];
            l = lo[sd.first + i];
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
        sx[k] = sy[k] = sz[k] = qx[k] = qy[k] = qz[k] = 0.f;
    }
    const float2 e2 = dup2(eps2);
    float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
    bool valid = lane < sd.n;
    if (valid) {
        h = hi[sd.first + lane];
        l = lo[sd.first + lane];
    }
    for (int jc = 0; jc < nch; ++jc) {
        const float4 jmn = box[2 * (sd.chunk0 + jc)], jmx = box[2 * (sd.chunk0 + jc) + 1];
        const float gx = fmaxf(0.f, fmaxf(jmn.x - bmx.x, bmn.x - jmx.x));
        const float gy = fmaxf(0.f, fmaxf(jmn.y - bmx.y, bmn.y - jmx.y));
        const float gz = fmaxf(0.f, fmaxf(jmn.z - bmx.z, bmn.z - jmx.z));
        const float gap2 = gx * gx + gy * gy + gz * gz;
        const bool far = gap2 > 0.f && gap2 >= thr2;
        const bool vfar = far && gap2 >= thr2v;
        // lanes past the system stage a massless body far away: exactly 0
        float Sx = 1.0e18f, Sy = 1.0e18f, Sz = 1.0e18f, Ex = 0.f, Ey = 0.f, Ez = 0.f, mj = 0.f;
        if (valid) {
            if (far) {
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
        valid = (jc + 1) * 32 + lane < sd.n;
        if (valid) {
            h = hi[sd.first + (jc + 1) * 32 + lane];
            l = lo[sd.first + (jc + 1) * 32 + lane];
        }
        float2 fx[IPT], fy[IPT], fz[IPT];
#pragma unroll
        for (int k = 0; k < IPT; ++k) fx[k] = fy[k] = fz[k] = dup2(0.f);
        if (vfar) {
#pragma unroll 4
            for (int p = 0; p < 16; ++p) {
                const JPair j = pair_tile_get(sg, p);
#pragma unroll
                for (int k = 0; k < IPT; ++k)
                    pair_term2_far<false>(j, nsx[k], nsy[k], nsz[k], e2, fx[k], fy[k], fz[k]);
            }
        } else if (far) {
#pragma unroll 4
            for (int p = 0; p < 16; ++p) {
                const JPair j = pair_tile_get(sg, p);
#pragma unroll
                for (int k = 0; k < IPT; ++k)
                    pair_term2_far<true>(j, nsx[k], nsy[k], nsz[k], e2, fx[k], fy[k], fz[k]);
            }
        } else {
#pragma unroll 4
            for (int p = 0; p < 16; ++p) {
                const JPair j = pair_tile_get(sg, p);
#pragma unroll
                for (int k = 0; k < IPT; ++k)
                    pair_term2<ZERO_SOFT>(j, nsx[k], nsy[k], nsz[k], nex[k], ney[k], nez[k], e2,
                                          fx[k], fy[k], fz[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            kahan_add(sx[k], qx[k], fx[k].x + fx[k].y);
            kahan_add(sy[k], qy[k], fy[k].x + fy[k].y);
            kahan_add(sz[k], qz[k], fz[k].x + fz[k].y);
        }
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = i0 + 32 * k + lane;
        if (i < sd.n) {
            const uint32_t o = order[sd.first + i];
            if (!NB_IN_RANGE(o, total)) continue;
            ax[o] = G * ((double)sx[k] - (double)qx[k]);
            ay[o] = G * ((double)sy[k] - (double)qy[k]);
            az[o] = G * ((double)sz[k] - (double)qz[k]);
        }
    }
}

template <bool ZERO_SOFT>
__global__ void __launch_bounds__(kBatchBlock)
batch_sorted_kernel(const float4 *__restrict__ hi, const float4 *__restrict__ lo,
                    const float4 *__restrict__ box, const SysDesc *__restrict__ sys,
                    const WorkItem *__restrict__ items, int num_items, int *__restrict__ counter,
                    float eps2, double G, const uint32_t *__restrict__ order,
                    double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az,
                    int total, int num_chunks)
{
    __shared__ PairTile tiles[kBatchWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    while (true) {
        int item = 0;
        if (lane == 0) item = atomicAdd(counter, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= num_items) break;
        const WorkItem w = items[item];
        const SysDesc sd = sys[w.sys];
        if (!NB_IN_RANGE(sd.first, total) || !NB_IN_RANGE(sd.first + sd.n - 1, total) ||
            !NB_IN_RANGE(sd.chunk0 + (sd.n - 1) / 32, num_chunks))
            continue;
        if (sd.ipt == 2)
            batch_sorted_item<2, ZERO_SOFT>(hi, lo, box, sd, w.i0, eps2, G, order, ax, ay, az,
                                            tiles[warp], total);
        else
            batch_sorted_item<1, ZERO_SOFT>(hi, lo, box, sd, w.i0, eps2, G, order, ax, ay, az,
                                            tiles[warp], total);
    }
}

int batch_sorted_grid()
{
    static const int grid = [] {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, (const void *)batch_sorted_kernel<false>, kBatchBlock, 0);
        return std::max(1, per_sm) * device_props().num_sms;
    }();
    return grid;
}

} // namespace

int bucket_of(int n)
{
    int b = 0;
    while ((2 << b) <= n && b < 30) ++b;
    return b;  // floor(log2(n))
}

void build_work_items(const std::vector<SysDesc> &sys, std::vector<WorkItem> &items)
{
    // largest cost first: an item costs ~ n_j * 32 ipt, the same for every
    // full item of a system, so the systems are ordered (stably) by that cost
    // and each contributes its items in order -- O(items), no per-item sort
    std::vector<int> by_cost(sys.size());
    for (int s = 0; s < (int)sys.size(); ++s) by_cost[s] = s;
    std::stable_sort(by_cost.begin(), by_cost.end(), [&](int a, int b) {
        return (long)sys[a].n * std::min(32 * sys[a].ipt, sys[a].n) >
               (long)sys[b].n * std::min(32 * sys[b].ipt, sys[b].n);
    });
    items.clear();
    for (int s : by_cost) {
        const int per = 32 * sys[s].ipt;
        for (int i0 = 0; i0 < sys[s].n; i0 += per) items.push_back(WorkItem{s, i0});
    }
}

nb_status batch_forces(const float4 *hi, const float4 *lo, const SysDesc *d_sys,
                       const WorkItem *d_items, int num_items, int *d_counter, double G,
                       double eps2, double *ax, double *ay, double *az, int total,
                       cudaStream_t st, const KernelTimer *timer)
{
    if (num_items <= 0) return NB_OK;
    NB_CUDA_TRY(cudaMemsetAsync(d_counter, 0, sizeof(int), st));
    if (timer && timer->start) NB_CUDA_TRY(cudaEventRecord(timer->start, st));
    if (eps2 > 0.0)
        batch_force_kernel<false><<<batch_grid(), kBatchBlock, 0, st>>>(
            hi, lo, d_sys, d_items, num_items, d_counter, (float)eps2, G, ax, ay, az, total);
    else
        batch_force_kernel<true><<<batch_grid(), kBatchBlock, 0, st>>>(
            hi, lo, d_sys, d_items, num_items, d_counter, 0.0f, G, ax, ay, az, total);
    NB_LAUNCH_CHECK();
    if (timer && timer->stop) NB_CUDA_TRY(cudaEventRecord(timer->stop, st));
    return NB_OK;
}


void BatchSorted::release()
{
    if (sorter) bh_destroy(sorter);
    sorter = nullptr;
    order = nullptr;
    DevBuf *bufs[] = {&body_sys, &chunks, &geom, &boxes};
    for (DevBuf *b : bufs) b->release();
}

int batch_sorted_ipt(int n) { return n >= kSortedIpt2Min ? 2 : 1; }

int batch_sorted_chunks(std::vector<SysDesc> &sys)
{
    int c = 0;
    for (SysDesc &s : sys) {
        s.ipt = batch_sorted_ipt(s.n);
        s.chunk0 = c;
        c += (s.n + 31) / 32;
    }
    return c;
}

nb_status batch_sorted_setup(BatchSorted &b, const SysDesc *d_sys, int num_sys, int num_chunks,
                             int total, cudaStream_t st)
{
    b.num_sys = num_sys;
    b.num_chunks = num_chunks;
    b.total = total;
    int sys_bits = 1;
    while ((1 << sys_bits) < num_sys) ++sys_bits;
    const int key_bits = sys_bits + 30;
    b.key_shift = 64 - key_bits;
    b.first_shift = b.key_shift / 8 * 8;
    NB_TRY(b.body_sys.reserve(sizeof(int) * (size_t)std::max(total, 1)));
    NB_TRY(b.chunks.reserve(sizeof(int2) * (size_t)std::max(num_chunks, 1)));
    NB_TRY(b.geom.reserve(sizeof(double4) * (size_t)std::max(num_sys, 1)));
    NB_TRY(b.boxes.reserve(sizeof(float4) * 2 * (size_t)std::max(num_chunks, 1)));
    if (!b.sorter) b.sorter = bh_create();
    batch_layout_kernel<<<num_sys, 128, 0, st>>>(d_sys, b.body_sys.as<int>(), b.chunks.as<int2>());
    NB_LAUNCH_CHECK();
    return NB_OK;
}

nb_status batch_sorted_sort(BatchSorted &b, const SysDesc *d_sys, const double *x,
                            const double *y, const double *z, cudaStream_t st)
{
    if (b.total <= 0) return NB_OK;
    uint64_t *keys = nullptr;
    uint32_t *vals = nullptr;
    NB_TRY(bh_sort_buffers(b.sorter, b.total, &keys, &vals));
    batch_geom_kernel<<<b.num_sys, 256, 0, st>>>(d_sys, x, y, z, b.geom.as<double4>());
    NB_LAUNCH_CHECK();
    batch_key_kernel<<<(b.total + 255) / 256, 256, 0, st>>>(
        x, y, z, b.body_sys.as<int>(), b.geom.as<double4>(), b.total, b.key_shift, keys, vals);
    NB_LAUNCH_CHECK();
    return bh_sort_keys(b.sorter, b.total, b.first_shift, st, &b.order);
}

nb_status batch_sorted_forces(BatchSorted &b, const double *x, const double *y, const double *z,
                              const double *m, const SysDesc *d_sys, const WorkItem *d_items,
                              int num_items, int *d_counter, double G, double eps2, float4 *hi,
                              float4 *lo, double *ax, double *ay, double *az, cudaStream_t st,
                              const KernelTimer *timer)
{
    if (num_items <= 0) return NB_OK;
    if (!b.order) return fail(NB_ERR_NOT_LOADED, "sorted batch: no order (sort first)");
    batch_split_sorted_kernel<<<(b.total + 255) / 256, 256, 0, st>>>(
        b.order, x, y, z, m, b.body_sys.as<int>(), b.geom.as<double4>(), b.total, hi, lo);
    NB_LAUNCH_CHECK();
    batch_chunk_box_kernel<<<(b.num_chunks + 7) / 8, 256, 0, st>>>(
        hi, b.chunks.as<int2>(), b.num_chunks, b.boxes.as<float4>());
    NB_LAUNCH_CHECK();
    NB_CUDA_TRY(cudaMemsetAsync(d_counter, 0, sizeof(int), st));
    if (timer && timer->start) NB_CUDA_TRY(cudaEventRecord(timer->start, st));
    if (eps2 > 0.0)
        batch_sorted_kernel<false><<<batch_sorted_grid(), kBatchBlock, 0, st>>>(
            hi, lo, b.boxes.as<float4>(), d_sys, d_items, num_items, d_counter, (float)eps2, G,
            b.order, ax, ay, az, b.total, b.num_chunks);
    else
        batch_sorted_kernel<true><<<batch_sorted_grid(), kBatchBlock, 0, st>>>(
            hi, lo, b.boxes.as<float4>(), d_sys, d_items, num_items, d_counter, 0.0f, G,
            b.order, ax, ay, az, b.total, b.num_chunks);
    NB_LAUNCH_CHECK();
    if (timer && timer->stop) NB_CUDA_TRY(cudaEventRecord(timer->stop, st));
    return NB_OK;
}
} // namespace nb
