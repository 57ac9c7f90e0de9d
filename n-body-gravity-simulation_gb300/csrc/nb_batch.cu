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
#include "nb_pair.cuh"

#include <algorithm>
#include <cmath>

namespace nb {
namespace {

constexpr int kBatchBlock = 128;  // 4 warps
constexpr int kBatchWarps = kBatchBlock / 32;

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
                   double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az)
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
    static int grid = 0;
    if (!grid) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, (const void *)batch_force_kernel<false>, kBatchBlock, 0);
        grid = std::max(1, per_sm) * device_props().num_sms;
    }
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
                       double eps2, double *ax, double *ay, double *az, cudaStream_t st,
                       const KernelTimer *timer)
{
    if (num_items <= 0) return NB_OK;
    NB_CUDA_TRY(cudaMemsetAsync(d_counter, 0, sizeof(int), st));
    if (timer && timer->start) NB_CUDA_TRY(cudaEventRecord(timer->start, st));
    if (eps2 > 0.0)
        batch_force_kernel<false><<<batch_grid(), kBatchBlock, 0, st>>>(
            hi, lo, d_sys, d_items, num_items, d_counter, (float)eps2, G, ax, ay, az);
    else
        batch_force_kernel<true><<<batch_grid(), kBatchBlock, 0, st>>>(
            hi, lo, d_sys, d_items, num_items, d_counter, 0.0f, G, ax, ay, az);
    NB_LAUNCH_CHECK();
    if (timer && timer->stop) NB_CUDA_TRY(cudaEventRecord(timer->stop, st));
    return NB_OK;
}

} // namespace nb
