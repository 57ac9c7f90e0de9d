// nb_direct.cu -- all-pairs gravity on sm_103a.
//
// Replaces computeAccelerationNaiveKernel (CUDA/src/force_calculator_naive.cu:4-59,
// one FP64 thread per body, 256-body tiles, ceil(N/256) CTAs).  Two kernels:
//
//  * direct_mixed_kernel -- the production path.  Each body is held as a float4
//    "hi" (x, y, z, m) plus a float4 "lo" (x - hi, ...): a double-single copy of
//    its FP64 position.  The pair displacement is formed as
//    (xj_hi - xi_hi) + (xj_lo - xi_lo), which is exact to FP32 rounding for close
//    pairs, so close encounters keep a relative force error near 1e-7 however far
//    the pair is from the origin.  The rest of the pair term is plain FP32 on the
//    FMA pipe with one MUFU rsqrt (rsqrt.approx.ftz.f32) whose ~1.3e-7 error is
//    removed by a Newton step folded into r^-3 (3 extra FP32 ops: 21 FP32-pipe
//    operations + 1 MUFU per pair against the 12 of the bare pair term).  The
//    FP32 work runs as packed f32x2 operations on j-pairs (two j per
//    instruction, nb_pair.cuh), which halves its issue slots.  Every thread
//    owns IPT i-bodies, so one broadcast shared-memory read of a j-pair feeds
//    IPT pair terms.  Every 32 j the FP32 partial sum is added into a Kahan-compensated
//    (sum, compensation) pair; the CTA's partial over its j-segment is written
//    as FP32 (sum, comp) and the segments are combined as a double-single,
//    scaled by G in FP64.
//    The tensor cores stay idle: a softened 1/r^3 sum is not a contraction.
//
//  * direct_fp64_kernel -- the 1e-12 path: the same tiling in FP64.
//
// Grid: x = i-blocks of BLOCK*IPT bodies, y = j-segments.  The j-split keeps
// all 152 SMs busy at small N (the reference runs 4 CTAs at N = 1024) and the
// segment count is chosen to fill whole waves.
#include "nb_internal.h"
#include "nb_pair.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

namespace nb {
namespace {

template <int BLOCK, int IPT, bool ZERO_SOFT>
__global__ void __launch_bounds__(BLOCK)
direct_mixed_kernel(const float4 *__restrict__ hi, const float4 *__restrict__ lo, int n,
                    float eps2, int seg_len, float *__restrict__ psum,
                    float *__restrict__ pcomp)
{
    __shared__ PairTile tiles[BLOCK / 32];

    const int tid = threadIdx.x;
    const int ibase = blockIdx.x * (BLOCK * IPT);

    // i-bodies negated and duplicated into f32x2 pairs
    float2 nxh[IPT], nyh[IPT], nzh[IPT], nxl[IPT], nyl[IPT], nzl[IPT];
    float sx[IPT], sy[IPT], sz[IPT], cx[IPT], cy[IPT], cz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + k * BLOCK + tid;
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
        if (i < n) {
            h = hi[i];
            l = lo[i];
        }
        nxh[k] = dup2(-h.x); nyh[k] = dup2(-h.y); nzh[k] = dup2(-h.z);
        nxl[k] = dup2(-l.x); nyl[k] = dup2(-l.y); nzl[k] = dup2(-l.z);
        sx[k] = sy[k] = sz[k] = 0.f;
        cx[k] = cy[k] = cz[k] = 0.f;
    }
    const float2 e2 = dup2(eps2);

    const int j0 = blockIdx.y * seg_len;
    const int j1 = min(n, j0 + seg_len);
    for (int t0 = j0; t0 < j1; t0 += BLOCK) {
        const int j = t0 + tid;
        float4 h = far_body(), l = make_float4(0.f, 0.f, 0.f, 0.f);
        if (j < j1) {
            h = hi[j];
            l = lo[j];
        }
        __syncthreads();
        pair_tile_put(tiles[tid >> 5], tid & 31, h.x, h.y, h.z, h.w, l.x, l.y, l.z);
        __syncthreads();

        // FP32 partial sums over each 32-body tile (16 terms per f32x2 lane),
        // Kahan-added into (s, c): the rounding of a running FP32 sum grows
        // with its length, and short runs keep it below the per-term error of
        // the pair arithmetic.
#pragma unroll 1
        for (int t = 0; t < BLOCK / 32; ++t) {
            float2 ax[IPT], ay[IPT], az[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k) ax[k] = ay[k] = az[k] = dup2(0.f);
#pragma unroll 2
            for (int p = 0; p < 16; ++p) {
                const JPair jp = pair_tile_get(tiles[t], p);
#pragma unroll
                for (int k = 0; k < IPT; ++k)
                    pair_term2<ZERO_SOFT>(jp, nxh[k], nyh[k], nzh[k], nxl[k], nyl[k], nzl[k], e2,
                                          ax[k], ay[k], az[k]);
            }
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                kahan_add(sx[k], cx[k], ax[k].x + ax[k].y);
                kahan_add(sy[k], cy[k], ay[k].x + ay[k].y);
                kahan_add(sz[k], cz[k], az[k].x + az[k].y);
            }
        }
    }

    const size_t plane = (size_t)n;
    const size_t base = (size_t)blockIdx.y * 3 * plane;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + k * BLOCK + tid;
        if (i < n) {
            psum[base + i] = sx[k];
            psum[base + plane + i] = sy[k];
            psum[base + 2 * plane + i] = sz[k];
            pcomp[base + i] = cx[k];
            pcomp[base + plane + i] = cy[k];
            pcomp[base + 2 * plane + i] = cz[k];
        }
    }
}

// a_i = G * sum_s (sum_s - comp_s), segments in index order, accumulated as a
// double-single and scaled in FP64.
__global__ void combine_mixed_kernel(const float *__restrict__ psum,
                                     const float *__restrict__ pcomp, int n, int segments,
                                     double G, double *__restrict__ ax,
                                     double *__restrict__ ay, double *__restrict__ az)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t plane = (size_t)n;
    float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
    for (int s = 0; s < segments; ++s) {
        const size_t base = (size_t)s * 3 * plane;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            ds_add_kahan(hi[c], lo[c], psum[base + c * plane + i], pcomp[base + c * plane + i]);
    }
    ax[i] = G * ((double)hi[0] + (double)lo[0]);
    ay[i] = G * ((double)hi[1] + (double)lo[1]);
    az[i] = G * ((double)hi[2] + (double)lo[2]);
}

template <int BLOCK, int IPT, bool ZERO_SOFT>
__global__ void __launch_bounds__(BLOCK)
direct_fp64_kernel(const double *__restrict__ x, const double *__restrict__ y,
                   const double *__restrict__ z, const double *__restrict__ m, int n,
                   double eps2, int seg_len, double *__restrict__ part)
{
    __shared__ double4_32a sh[BLOCK];
    const int tid = threadIdx.x;
    const int ibase = blockIdx.x * (BLOCK * IPT);
    double xi[IPT], yi[IPT], zi[IPT], ax[IPT], ay[IPT], az[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + k * BLOCK + tid;
        xi[k] = (i < n) ? x[i] : 0.0;
        yi[k] = (i < n) ? y[i] : 0.0;
        zi[k] = (i < n) ? z[i] : 0.0;
        ax[k] = ay[k] = az[k] = 0.0;
    }
    const int j0 = blockIdx.y * seg_len;
    const int j1 = min(n, j0 + seg_len);
    for (int t0 = j0; t0 < j1; t0 += BLOCK) {
        const int j = t0 + tid;
        double4_32a b = make_double4_32a(1.0e150, 1.0e150, 1.0e150, 0.0);
        if (j < j1) b = make_double4_32a(x[j], y[j], z[j], m[j]);
        __syncthreads();
        sh[tid] = b;
        __syncthreads();
#pragma unroll 2
        for (int jj = 0; jj < BLOCK; ++jj) {
            const double4_32a B = sh[jj];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const double dx = B.x - xi[k];
                const double dy = B.y - yi[k];
                const double dz = B.z - zi[k];
                const double r2 = fma(dz, dz, fma(dy, dy, fma(dx, dx, eps2)));
                double inv = rsqrt(r2);
                if (ZERO_SOFT) inv = (r2 > 0.0) ? inv : 0.0;
                const double s = B.w * inv * inv * inv;
                ax[k] = fma(dx, s, ax[k]);
                ay[k] = fma(dy, s, ay[k]);
                az[k] = fma(dz, s, az[k]);
            }
        }
    }
    const size_t plane = (size_t)n;
    const size_t base = (size_t)blockIdx.y * 3 * plane;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + k * BLOCK + tid;
        if (i < n) {
            part[base + i] = ax[k];
            part[base + plane + i] = ay[k];
            part[base + 2 * plane + i] = az[k];
        }
    }
}

__global__ void combine_fp64_kernel(const double *__restrict__ part, int n, int segments,
                                    double G, double *__restrict__ ax, double *__restrict__ ay,
                                    double *__restrict__ az)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t plane = (size_t)n;
    double a[3] = {0.0, 0.0, 0.0};
    for (int s = 0; s < segments; ++s) {
        const size_t base = (size_t)s * 3 * plane;
#pragma unroll
        for (int c = 0; c < 3; ++c) a[c] += part[base + c * plane + i];
    }
    ax[i] = G * a[0];
    ay[i] = G * a[1];
    az[i] = G * a[2];
}

__global__ void split_kernel(const double *__restrict__ x, const double *__restrict__ y,
                             const double *__restrict__ z, const double *__restrict__ m, int n,
                             float4 *__restrict__ hi, float4 *__restrict__ lo)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double X = x[i], Y = y[i], Z = z[i];
    const float hx = __double2float_rn(X), hy = __double2float_rn(Y), hz = __double2float_rn(Z);
    hi[i] = make_float4(hx, hy, hz, __double2float_rn(m[i]));
    lo[i] = make_float4(__double2float_rn(X - (double)hx), __double2float_rn(Y - (double)hy),
                        __double2float_rn(Z - (double)hz), 0.0f);
}

// Picks the j-split so that i-blocks x segments fills whole waves of
// `slots` resident CTAs; longer segments are preferred on ties.
int pick_segments(int iblocks, int tiles, int slots)
{
    int best = 1;
    double best_eff = -1.0;
    const int smax = std::max(1, std::min(tiles, 64));
    for (int s = 1; s <= smax; ++s) {
        const int seg_tiles = (tiles + s - 1) / s;
        const int s_eff = (tiles + seg_tiles - 1) / seg_tiles;
        const long ctas = (long)iblocks * s_eff;
        const long waves = (ctas + slots - 1) / slots;
        // useful work / (waves * slots * longest segment): tail and
        // quantisation losses; a small penalty per extra segment.
        const double eff = (double)tiles * iblocks / ((double)waves * slots * seg_tiles) -
                           0.002 * s_eff;
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = s_eff;
        }
    }
    return best;
}

template <int BLOCK, int IPT>
int resident_ctas(const void *fn)
{
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, BLOCK, 0);
    return std::max(1, per_sm) * device_props().num_sms;
}

constexpr int kMixBlock = 256;
constexpr int kMixIpt = 4;
constexpr int kF64Block = 128;
constexpr int kF64Ipt = 2;
constexpr int kF64SmallMax = 8192;  // largest N of the one-warp FP64 shape

// Tile shapes of the mixed kernel the autotuner chooses from: threads per CTA
// x i-bodies per thread.  More i-bodies per thread amortise the two
// broadcast shared-memory loads of a j-body and add independent work per
// warp; fewer keep more warps resident.
struct MixShape {
    int block, ipt;
};
constexpr MixShape kMixShapes[] = {{256, 4}, {128, 2}, {128, 4}, {256, 2}, {64, 4},
                                    {32, 1}, {32, 2}};
constexpr int kNumMixShapes = sizeof(kMixShapes) / sizeof(kMixShapes[0]);

template <int B, int I>
int mix_slots()
{
    static const int slots = resident_ctas<B, I>((const void *)direct_mixed_kernel<B, I, false>);
    return slots;
}

int mix_slots_for(int block, int ipt)
{
    if (block == 256 && ipt == 4) return mix_slots<256, 4>();
    if (block == 128 && ipt == 2) return mix_slots<128, 2>();
    if (block == 128 && ipt == 4) return mix_slots<128, 4>();
    if (block == 256 && ipt == 2) return mix_slots<256, 2>();
    if (block == 64 && ipt == 4) return mix_slots<64, 4>();
    if (block == 32 && ipt == 1) return mix_slots<32, 1>();
    if (block == 32 && ipt == 2) return mix_slots<32, 2>();
    return 0;
}

template <int B, int I>
void launch_mixed_shape(dim3 grid, cudaStream_t st, const float4 *hi, const float4 *lo, int n,
                        double eps2, int seg_len, float *psum, float *pcomp)
{
    if (eps2 > 0.0)
        direct_mixed_kernel<B, I, false>
            <<<grid, B, 0, st>>>(hi, lo, n, (float)eps2, seg_len, psum, pcomp);
    else
        direct_mixed_kernel<B, I, true><<<grid, B, 0, st>>>(hi, lo, n, 0.0f, seg_len, psum, pcomp);
}

// Launches the all-pairs kernel of plan p (partials psum/pcomp sized for
// p.segments); returns false for a shape that is not compiled in.
bool launch_mixed(const DirectPlan &p, cudaStream_t st, const float4 *hi, const float4 *lo,
                  int n, double eps2, float *psum, float *pcomp)
{
    const int per_cta = p.block * p.ipt;
    dim3 grid((n + per_cta - 1) / per_cta, p.segments);
    const int seg_len = p.seg_tiles * p.block;
    if (p.block == 256 && p.ipt == 4)
        launch_mixed_shape<256, 4>(grid, st, hi, lo, n, eps2, seg_len, psum, pcomp);
    else if (p.block == 128 && p.ipt == 2)
        launch_mixed_shape<128, 2>(grid, st, hi, lo, n, eps2, seg_len, psum, pcomp);
    else if (p.block == 128 && p.ipt == 4)
        launch_mixed_shape<128, 4>(grid, st, hi, lo, n, eps2, seg_len, psum, pcomp);
    else if (p.block == 256 && p.ipt == 2)
        launch_mixed_shape<256, 2>(grid, st, hi, lo, n, eps2, seg_len, psum, pcomp);
    else if (p.block == 64 && p.ipt == 4)
        launch_mixed_shape<64, 4>(grid, st, hi, lo, n, eps2, seg_len, psum, pcomp);
    else if (p.block == 32 && p.ipt == 1)
        launch_mixed_shape<32, 1>(grid, st, hi, lo, n, eps2, seg_len, psum, pcomp);
    else if (p.block == 32 && p.ipt == 2)
        launch_mixed_shape<32, 2>(grid, st, hi, lo, n, eps2, seg_len, psum, pcomp);
    else
        return false;
    return true;
}

DirectPlan plan_for_shape_model(int n, int block, int ipt)
{
    DirectPlan p;
    p.block = block;
    p.ipt = ipt;
    const int per_cta = block * ipt;
    const int iblocks = (n + per_cta - 1) / per_cta;
    const int tiles = (n + block - 1) / block;
    p.segments = pick_segments(iblocks, tiles, mix_slots_for(block, ipt));
    p.seg_tiles = (tiles + p.segments - 1) / p.segments;
    p.segments = (tiles + p.seg_tiles - 1) / p.seg_tiles;
    return p;
}

// The j-segment length of n bodies: that of the default shape (one-warp CTAs
// below 4096 bodies, kMixBlock x kMixIpt above).  A body's summation order
// depends only on the segment boundaries (every shape sums each segment in
// 32-body tiles from its start), so fixing them per n makes every tile shape
// give the same bits and the autotuner's timed choice cannot change a result.
int mixed_segment_length(int n)
{
    const DirectPlan d = n < 4096 ? plan_for_shape_model(n, 32, n < 2048 ? 1 : 2)
                                  : plan_for_shape_model(n, kMixBlock, kMixIpt);
    return d.seg_tiles * d.block;
}

DirectPlan plan_for_shape(int n, int block, int ipt)
{
    DirectPlan p;
    p.block = block;
    p.ipt = ipt;
    const int seg_len = mixed_segment_length(n);  // a multiple of every block size below it
    p.seg_tiles = std::max(1, seg_len / block);
    p.segments = std::max(1, (n + seg_len - 1) / seg_len);
    return p;
}

// Autotuned plans by body count (the tuner times every shape on the caller's
// own bodies at the first evaluation of each N; NB_AUTOTUNE=0 disables it).
std::mutex g_tune_mutex;
std::map<int, DirectPlan> g_tuned;

bool autotune_enabled()
{
    static const bool on = [] {
        const char *e = std::getenv("NB_AUTOTUNE");
        return !(e && std::strcmp(e, "0") == 0);
    }();
    return on;
}

} // namespace

int direct_pick_segments(int iblocks, int tiles, int slots)
{
    return pick_segments(iblocks, tiles, slots);
}

DirectPlan direct_mixed_plan(int n)
{
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tuned.find(n);
        if (it != g_tuned.end()) return it->second;
    }
    // small systems (not tuned): one-warp CTAs, as many as the j-split allows
    if (n < 4096) return plan_for_shape(n, 32, n < 2048 ? 1 : 2);
    return plan_for_shape(n, kMixBlock, kMixIpt);
}

// Times every tile shape on the given bodies (two launches each after one
// warm-up, CUDA events on `st`) and records the fastest for this n.
static nb_status autotune_mixed(const float4 *hi, const float4 *lo, int n, double eps2,
                                DevBuf &partials, cudaStream_t st, DirectPlan *best)
{
    DirectPlan plans[kNumMixShapes];
    size_t need = 0;
    for (int k = 0; k < kNumMixShapes; ++k) {
        plans[k] = plan_for_shape(n, kMixShapes[k].block, kMixShapes[k].ipt);
        need = std::max(need, sizeof(float) * 6 * (size_t)n * plans[k].segments);
    }
    NB_TRY(partials.reserve(need));
    cudaEvent_t e0, e1;
    NB_CUDA_TRY(cudaEventCreate(&e0));
    NB_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    *best = plans[0];
    for (int k = 0; k < kNumMixShapes; ++k) {
        float *psum = partials.as<float>();
        float *pcomp = psum + 3 * (size_t)n * plans[k].segments;
        launch_mixed(plans[k], st, hi, lo, n, eps2, psum, pcomp);
        NB_LAUNCH_CHECK();
        cudaEventRecord(e0, st);
        for (int r = 0; r < 2; ++r) launch_mixed(plans[k], st, hi, lo, n, eps2, psum, pcomp);
        cudaEventRecord(e1, st);
        NB_LAUNCH_CHECK();
        NB_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
            best_ms = ms;
            *best = plans[k];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tuned[n] = *best;
    return NB_OK;
}

nb_status split_positions(const double *x, const double *y, const double *z, const double *m,
                          int n, float4 *hi, float4 *lo, cudaStream_t st)
{
    if (n <= 0) return NB_OK;
    split_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, y, z, m, n, hi, lo);
    NB_LAUNCH_CHECK();
    return NB_OK;
}

nb_status direct_mixed(const float4 *hi, const float4 *lo, int n, double G, double eps2,
                       double *ax, double *ay, double *az, DevBuf &partials, cudaStream_t st,
                       const KernelTimer *timer, const DirectPlan *plan_override)
{
    if (n <= 0) return NB_OK;
    DirectPlan p;
    if (plan_override) {
        p = *plan_override;
    } else {
        bool tuned;
        {
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            tuned = g_tuned.count(n) != 0;
        }
        if (!tuned && autotune_enabled() && n >= 4096)
            NB_TRY(autotune_mixed(hi, lo, n, eps2, partials, st, &p));
        else
            p = direct_mixed_plan(n);
    }
    NB_TRY(partials.reserve(sizeof(float) * 6 * (size_t)n * p.segments));
    float *psum = partials.as<float>();
    float *pcomp = psum + 3 * (size_t)n * p.segments;
    if (timer && timer->start) NB_CUDA_TRY(cudaEventRecord(timer->start, st));
    if (!launch_mixed(p, st, hi, lo, n, eps2, psum, pcomp))
        return fail(NB_ERR_UNSUPPORTED, "direct_mixed: unsupported tile shape");
    NB_LAUNCH_CHECK();
    if (timer && timer->stop) NB_CUDA_TRY(cudaEventRecord(timer->stop, st));
    combine_mixed_kernel<<<(n + 255) / 256, 256, 0, st>>>(psum, pcomp, n, p.segments, G, ax, ay,
                                                         az);
    NB_LAUNCH_CHECK();
    return NB_OK;
}

template <int B, int I>
static nb_status direct_fp64_shape(const double *x, const double *y, const double *z,
                                   const double *m, int n, double G, double eps2, double *ax,
                                   double *ay, double *az, DevBuf &partials, cudaStream_t st,
                                   const KernelTimer *timer)
{
    const int per_cta = B * I;
    const int iblocks = (n + per_cta - 1) / per_cta;
    const int tiles = (n + B - 1) / B;
    static const int slots = resident_ctas<B, I>((const void *)direct_fp64_kernel<B, I, false>);
    int segs = pick_segments(iblocks, tiles, slots);
    const int seg_tiles = (tiles + segs - 1) / segs;
    segs = (tiles + seg_tiles - 1) / seg_tiles;
    NB_TRY(partials.reserve(sizeof(double) * 3 * (size_t)n * segs));
    double *part = partials.as<double>();
    dim3 grid(iblocks, segs);
    const int seg_len = seg_tiles * B;
    if (timer && timer->start) NB_CUDA_TRY(cudaEventRecord(timer->start, st));
    if (eps2 > 0.0)
        direct_fp64_kernel<B, I, false><<<grid, B, 0, st>>>(x, y, z, m, n, eps2, seg_len, part);
    else
        direct_fp64_kernel<B, I, true><<<grid, B, 0, st>>>(x, y, z, m, n, 0.0, seg_len, part);
    NB_LAUNCH_CHECK();
    if (timer && timer->stop) NB_CUDA_TRY(cudaEventRecord(timer->stop, st));
    combine_fp64_kernel<<<(n + 255) / 256, 256, 0, st>>>(part, n, segs, G, ax, ay, az);
    NB_LAUNCH_CHECK();
    return NB_OK;
}

// Small systems take one-warp CTAs with 32-body j-tiles, so that up to
// (N/32)^2 CTAs share the FP64 work (N = 1024 with the large shape fills only
// 32 CTAs); large systems take 128 x 2.
nb_status direct_fp64(const double *x, const double *y, const double *z, const double *m, int n,
                      double G, double eps2, double *ax, double *ay, double *az,
                      DevBuf &partials, cudaStream_t st, const KernelTimer *timer)
{
    if (n <= 0) return NB_OK;
    if (n <= kF64SmallMax)
        return direct_fp64_shape<32, 1>(x, y, z, m, n, G, eps2, ax, ay, az, partials, st, timer);
    return direct_fp64_shape<kF64Block, kF64Ipt>(x, y, z, m, n, G, eps2, ax, ay, az, partials,
                                                 st, timer);
}

} // namespace nb

// ---------------------------------------------------------------------------
// All-pairs forces for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc/cudaFree on their hot
// path: a host application whose device memory is entirely owned by its own
// pool allocator, a plugin that is given a fixed device-memory budget at
// start-up, or a real-time loop that cannot afford the implicit device-wide
// synchronisation an allocation or free can cause.  For them,
// nb_direct_mixed_forces_noalloc runs the same split / all-pairs / combine
// kernels as the NB_DIRECT_MIXED method, but keeps its scratch (the float4
// hi/lo mirror of the bodies and the per-segment Kahan partial sums) in the
// file-scope device array below instead of memory it allocates.
//
// The array is kNoAllocScratchBytes (16 MiB) on every device that loads this
// library, held until the process exits, and limits n to kNoAllocMaxBodies.
// Its name is only a host-side stand-in in host code: the device address is
// fetched once per device with cudaGetSymbolAddress, by the first call made
// while that device is current (make that first call before any stream
// capture).  Every call shares the one array and leaves its contents behind;
// no part of it has to start at zero, because each call writes every element
// it later reads.  Calls whose kernels overlap on the GPU (different streams,
// or another thread) race on the array and must be serialised by the caller.
// ---------------------------------------------------------------------------
static constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace nb {
namespace {

constexpr size_t kNoAllocMaxBodies = 262144;  // hi/lo (32 B) + one segment (24 B) per body
constexpr int kNoAllocMaxDevices = 64;

std::mutex g_noalloc_mutex;
void *g_noalloc_address[kNoAllocMaxDevices] = {};

size_t round_up_256(size_t b) { return (b + 255) / 256 * 256; }

} // namespace
} // namespace nb

extern "C" nb_status nb_direct_mixed_forces_noalloc(size_t n, const double *x, const double *y,
                                                   const double *z, const double *m, double G,
                                                   double softening, double *ax, double *ay,
                                                   double *az, void *stream)
{
    using namespace nb;
    if (n > kNoAllocMaxBodies)
        return fail(NB_ERR_CAPACITY,
                    "nb_direct_mixed_forces_noalloc: n = " + std::to_string(n) +
                        " exceeds its fixed scratch limit of " +
                        std::to_string(kNoAllocMaxBodies) + " bodies");
    if (n == 0) return NB_OK;
    if (!x || !y || !z || !m || !ax || !ay || !az)
        return fail(NB_ERR_INVALID_ARGUMENT, "nb_direct_mixed_forces_noalloc: NULL array");
    if (!(softening >= 0.0))
        return fail(NB_ERR_INVALID_ARGUMENT, "nb_direct_mixed_forces_noalloc: softening < 0");
    int dev = 0;
    NB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return fail(NB_ERR_UNSUPPORTED, "nb_direct_mixed_forces_noalloc: device ordinal >= 64");
    void *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_address[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
            g_noalloc_address[dev] = p;
        }
        base = g_noalloc_address[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int ni = (int)n;
    const size_t mirror = round_up_256(sizeof(float4) * n);
    float4 *hi = static_cast<float4 *>(base);
    float4 *lo = reinterpret_cast<float4 *>(static_cast<unsigned char *>(base) + mirror);
    float *psum = reinterpret_cast<float *>(static_cast<unsigned char *>(base) + 2 * mirror);

    // Same plan as the allocating path, with the j-split capped so that the
    // partial sums fit the remaining scratch.
    DirectPlan p = direct_mixed_plan(ni);
    const int tiles = (ni + p.block - 1) / p.block;
    const size_t per_segment = sizeof(float) * 6 * n;
    const int max_segments = (int)std::max<size_t>(1, (kNoAllocScratchBytes - 2 * mirror) /
                                                          per_segment);
    if (p.segments > max_segments) {
        p.seg_tiles = (tiles + max_segments - 1) / max_segments;
        p.segments = (tiles + p.seg_tiles - 1) / p.seg_tiles;
    }
    float *pcomp = psum + 3 * n * (size_t)p.segments;

    split_kernel<<<(ni + 255) / 256, 256, 0, st>>>(x, y, z, m, ni, hi, lo);
    NB_LAUNCH_CHECK();
    const double eps2 = softening * softening;
    if (!launch_mixed(p, st, hi, lo, ni, eps2, psum, pcomp))
        return fail(NB_ERR_UNSUPPORTED, "nb_direct_mixed_forces_noalloc: tile shape");
    NB_LAUNCH_CHECK();
    combine_mixed_kernel<<<(ni + 255) / 256, 256, 0, st>>>(psum, pcomp, ni, p.segments, G, ax,
                                                          ay, az);
    NB_LAUNCH_CHECK();
    return NB_OK;
}
