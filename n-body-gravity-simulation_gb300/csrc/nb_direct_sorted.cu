// nb_direct_sorted.cu -- the mixed-precision all-pairs sum over Morton-sorted
// bodies with a near/far split of the j-tiles.
//
// The double-single displacement of the mixed pair term (nb_pair.cuh) costs 6
// of its 21 FP32 operations and is needed only when a pair is close compared
// with the pair's distance from the coordinate origin.  Here the origin is
// moved to each i-block: bodies are sorted along a Morton curve (the
// Barnes-Hut encode and radix sort), so the BLOCK*IPT consecutive bodies a CTA
// owns are spatially compact; the CTA takes the centre c of its i-block's
// bounding box as origin, and for a j-tile whose bounding box is at least the
// i-block's diameter D away, forms single-precision coordinates relative to c
// once per j (when staging the tile) and runs the plain FP32 pair term.
//
// Error of the far term: |xi - c| <= D/2 and |xj - c| <= r + D/2, so the
// rounding of the relative coordinates is at most 2^-24 (r + D) <= 2^-23 r
// for r >= D -- a displacement good to ~1.2e-7 relative, like the FP32
// arithmetic that follows.  The folded Newton step on the MUFU rsqrt is kept.
// Near tiles (including the i-block's own) take the full double-single term.
// Every tile decision is uniform over the CTA, so there is no divergence.
#include "nb_internal.h"
#include "nb_pair.cuh"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

namespace nb {
namespace {

// Positions in Morton order relative to the root centre, split into
// double-single hi/lo parts; mass in hi.w.
__global__ void split_sorted_kernel(const uint32_t *__restrict__ order,
                                    const double *__restrict__ x, const double *__restrict__ y,
                                    const double *__restrict__ z, const double *__restrict__ m,
                                    int n, const double *__restrict__ centre,
                                    float4 *__restrict__ hi, float4 *__restrict__ lo)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = order[i];
    const double X = x[o] - centre[0], Y = y[o] - centre[1], Z = z[o] - centre[2];
    const float hx = __double2float_rn(X), hy = __double2float_rn(Y), hz = __double2float_rn(Z);
    hi[i] = make_float4(hx, hy, hz, __double2float_rn(m[o]));
    lo[i] = make_float4(__double2float_rn(X - (double)hx), __double2float_rn(Y - (double)hy),
                        __double2float_rn(Z - (double)hz), 0.0f);
}

// Bounding box of every tile of `tile` consecutive sorted bodies (one block
// of `tile` threads per tile): box[2t] = min, box[2t+1] = max.
__global__ void tile_box_kernel(const float4 *__restrict__ hi, int n, float4 *__restrict__ box)
{
    __shared__ float mn[3][256], mx[3][256];
    const int t = threadIdx.x, tile = blockDim.x;
    const int i = blockIdx.x * tile + t;
    float4 p = i < n ? hi[i] : hi[blockIdx.x * tile];  // the tile's first body is valid
    mn[0][t] = mx[0][t] = p.x;
    mn[1][t] = mx[1][t] = p.y;
    mn[2][t] = mx[2][t] = p.z;
    __syncthreads();
    for (int w = tile / 2; w > 0; w >>= 1) {
        if (t < w)
            for (int k = 0; k < 3; ++k) {
                mn[k][t] = fminf(mn[k][t], mn[k][t + w]);
                mx[k][t] = fmaxf(mx[k][t], mx[k][t + w]);
            }
        __syncthreads();
    }
    if (t == 0) {
        box[2 * blockIdx.x] = make_float4(mn[0][0], mn[1][0], mn[2][0], 0.f);
        box[2 * blockIdx.x + 1] = make_float4(mx[0][0], mx[1][0], mx[2][0], 0.f);
    }
}

// Plain FP32 pair term on coordinates relative to the i-block centre.
template <bool ZERO_SOFT>
__device__ __forceinline__ void pair_term_far(const float4 &A, float xr, float yr, float zr,
                                              float eps2, float &ax, float &ay, float &az)
{
    const float dx = A.x - xr;
    const float dy = A.y - yr;
    const float dz = A.z - zr;
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
    float inv = rsqrt_mufu(r2);
    if (ZERO_SOFT) inv = (r2 > 0.f) ? inv : 0.f;
    const float inv2 = inv * inv;
    const float corr = fmaf(-1.5f, r2 * inv2, 2.5f);
    const float s = ((A.w * inv) * inv2) * corr;
    ax = fmaf(dx, s, ax);
    ay = fmaf(dy, s, ay);
    az = fmaf(dz, s, az);
}

template <int BLOCK, int IPT, bool ZERO_SOFT>
__global__ void __launch_bounds__(BLOCK)
direct_sorted_kernel(const float4 *__restrict__ hi, const float4 *__restrict__ lo,
                     const float4 *__restrict__ box, int n, int ntiles, float eps2,
                     int seg_len, float *__restrict__ psum, float *__restrict__ pcomp,
                     unsigned long long *__restrict__ far_tiles)
{
    __shared__ float4 sh_a[BLOCK];
    __shared__ float4 sh_b[BLOCK];
    __shared__ float s_geo[10];  // i-box min xyz, max xyz, centre xyz, diameter^2

    const int tid = threadIdx.x;
    const int ibase = blockIdx.x * (BLOCK * IPT);
    if (tid == 0) {
        float mn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, mx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        const int t0 = ibase / BLOCK;
        for (int k = 0; k < IPT && t0 + k < ntiles; ++k) {
            const float4 a = box[2 * (t0 + k)], b = box[2 * (t0 + k) + 1];
            mn[0] = fminf(mn[0], a.x); mn[1] = fminf(mn[1], a.y); mn[2] = fminf(mn[2], a.z);
            mx[0] = fmaxf(mx[0], b.x); mx[1] = fmaxf(mx[1], b.y); mx[2] = fmaxf(mx[2], b.z);
        }
        float d2 = 0.f;
        for (int k = 0; k < 3; ++k) {
            s_geo[k] = mn[k];
            s_geo[3 + k] = mx[k];
            s_geo[6 + k] = 0.5f * (mn[k] + mx[k]);
            d2 += (mx[k] - mn[k]) * (mx[k] - mn[k]);
        }
        s_geo[9] = d2;
    }
    __syncthreads();
    const float cx = s_geo[6], cy = s_geo[7], cz = s_geo[8], diam2 = s_geo[9];

    float xh[IPT], yh[IPT], zh[IPT], xl[IPT], yl[IPT], zl[IPT], xr[IPT], yr[IPT], zr[IPT];
    float sx[IPT], sy[IPT], sz[IPT], qx[IPT], qy[IPT], qz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + k * BLOCK + tid;
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
        if (i < n) {
            h = hi[i];
            l = lo[i];
        }
        xh[k] = h.x; yh[k] = h.y; zh[k] = h.z;
        xl[k] = l.x; yl[k] = l.y; zl[k] = l.z;
        xr[k] = (h.x - cx) + l.x;
        yr[k] = (h.y - cy) + l.y;
        zr[k] = (h.z - cz) + l.z;
        sx[k] = sy[k] = sz[k] = 0.f;
        qx[k] = qy[k] = qz[k] = 0.f;
    }

    unsigned nfar = 0;
    const int j0 = blockIdx.y * seg_len;
    const int j1 = min(n, j0 + seg_len);
    for (int t0 = j0; t0 < j1; t0 += BLOCK) {
        // tile gap to the i-block box: far when at least the i-block diameter
        const float4 bmin = box[2 * (t0 / BLOCK)], bmax = box[2 * (t0 / BLOCK) + 1];
        const float gx = fmaxf(0.f, fmaxf(bmin.x - s_geo[3], s_geo[0] - bmax.x));
        const float gy = fmaxf(0.f, fmaxf(bmin.y - s_geo[4], s_geo[1] - bmax.y));
        const float gz = fmaxf(0.f, fmaxf(bmin.z - s_geo[5], s_geo[2] - bmax.z));
        const float gap2 = gx * gx + gy * gy + gz * gz;
        const bool far = gap2 > 0.f && gap2 >= diam2;
        nfar += far;

        const int j = t0 + tid;
        float4 h = far_body(), l = make_float4(0.f, 0.f, 0.f, 0.f);
        if (j < j1) {
            h = hi[j];
            l = lo[j];
        }
        __syncthreads();
        if (far) sh_a[tid] = make_float4((h.x - cx) + l.x, (h.y - cy) + l.y, (h.z - cz) + l.z, h.w);
        else {
            sh_a[tid] = h;
            sh_b[tid] = l;
        }
        __syncthreads();

        constexpr int kSub = 32;
#pragma unroll 1
        for (int s0 = 0; s0 < BLOCK; s0 += kSub) {
            float ax[IPT], ay[IPT], az[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k) ax[k] = ay[k] = az[k] = 0.f;
            if (far) {
#pragma unroll 4
                for (int jj = s0; jj < s0 + kSub; ++jj) {
                    const float4 A = sh_a[jj];
#pragma unroll
                    for (int k = 0; k < IPT; ++k)
                        pair_term_far<ZERO_SOFT>(A, xr[k], yr[k], zr[k], eps2, ax[k], ay[k],
                                                 az[k]);
                }
            } else {
#pragma unroll 4
                for (int jj = s0; jj < s0 + kSub; ++jj) {
                    const float4 H = sh_a[jj];
                    const float4 L = sh_b[jj];
#pragma unroll
                    for (int k = 0; k < IPT; ++k)
                        pair_term<ZERO_SOFT>(H, L, xh[k], yh[k], zh[k], xl[k], yl[k], zl[k], eps2,
                                             ax[k], ay[k], az[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                kahan_add(sx[k], qx[k], ax[k]);
                kahan_add(sy[k], qy[k], ay[k]);
                kahan_add(sz[k], qz[k], az[k]);
            }
        }
    }
    if (far_tiles && tid == 0 && nfar) atomicAdd(far_tiles, (unsigned long long)nfar);

    const size_t plane = (size_t)n;
    const size_t base = (size_t)blockIdx.y * 3 * plane;
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + k * BLOCK + tid;
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

// a[order[i]] = G * sum_s (sum_s - comp_s) for sorted body i, in FP64.
__global__ void combine_sorted_kernel(const float *__restrict__ psum,
                                      const float *__restrict__ pcomp, int n, int segments,
                                      double G, const uint32_t *__restrict__ order,
                                      double *__restrict__ ax, double *__restrict__ ay,
                                      double *__restrict__ az)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t plane = (size_t)n;
    double a[3] = {0.0, 0.0, 0.0};
    for (int s = 0; s < segments; ++s) {
        const size_t base = (size_t)s * 3 * plane;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            a[c] += (double)psum[base + c * plane + i] - (double)pcomp[base + c * plane + i];
    }
    const uint32_t o = order[i];
    ax[o] = G * a[0];
    ay[o] = G * a[1];
    az[o] = G * a[2];
}

struct SortedShape {
    int block, ipt;
};
constexpr SortedShape kSortedShapes[] = {{256, 4}, {128, 8}, {128, 4}};
constexpr int kNumSortedShapes = sizeof(kSortedShapes) / sizeof(kSortedShapes[0]);

template <int B, int I>
int sorted_slots()
{
    static int slots = 0;
    if (!slots) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, (const void *)direct_sorted_kernel<B, I, false>, B, 0);
        slots = std::max(1, per_sm) * device_props().num_sms;
    }
    return slots;
}

int sorted_slots_for(int block, int ipt)
{
    if (block == 256 && ipt == 4) return sorted_slots<256, 4>();
    if (block == 128 && ipt == 8) return sorted_slots<128, 8>();
    if (block == 128 && ipt == 4) return sorted_slots<128, 4>();
    return 0;
}

template <int B, int I>
void launch_sorted_shape(dim3 grid, cudaStream_t st, const float4 *hi, const float4 *lo,
                         const float4 *box, int n, double eps2, int seg_len, float *psum,
                         float *pcomp, unsigned long long *far_tiles)
{
    const int ntiles = (n + B - 1) / B;
    if (eps2 > 0.0)
        direct_sorted_kernel<B, I, false><<<grid, B, 0, st>>>(hi, lo, box, n, ntiles, (float)eps2,
                                                              seg_len, psum, pcomp, far_tiles);
    else
        direct_sorted_kernel<B, I, true><<<grid, B, 0, st>>>(hi, lo, box, n, ntiles, 0.0f,
                                                             seg_len, psum, pcomp, far_tiles);
}

bool launch_sorted(const DirectPlan &p, cudaStream_t st, const float4 *hi, const float4 *lo,
                   const float4 *box, int n, double eps2, float *psum, float *pcomp,
                   unsigned long long *far_tiles)
{
    const int per_cta = p.block * p.ipt;
    dim3 grid((n + per_cta - 1) / per_cta, p.segments);
    const int seg_len = p.seg_tiles * p.block;
    if (p.block == 256 && p.ipt == 4)
        launch_sorted_shape<256, 4>(grid, st, hi, lo, box, n, eps2, seg_len, psum, pcomp,
                                    far_tiles);
    else if (p.block == 128 && p.ipt == 8)
        launch_sorted_shape<128, 8>(grid, st, hi, lo, box, n, eps2, seg_len, psum, pcomp,
                                    far_tiles);
    else if (p.block == 128 && p.ipt == 4)
        launch_sorted_shape<128, 4>(grid, st, hi, lo, box, n, eps2, seg_len, psum, pcomp,
                                    far_tiles);
    else
        return false;
    return true;
}

DirectPlan sorted_plan_for_shape(int n, int block, int ipt)
{
    DirectPlan p;
    p.block = block;
    p.ipt = ipt;
    const int per_cta = block * ipt;
    const int iblocks = (n + per_cta - 1) / per_cta;
    const int tiles = (n + block - 1) / block;
    p.segments = direct_pick_segments(iblocks, tiles, sorted_slots_for(block, ipt));
    p.seg_tiles = (tiles + p.segments - 1) / p.segments;
    p.segments = (tiles + p.seg_tiles - 1) / p.seg_tiles;
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
    if (sorter) bh_destroy(sorter);
    sorter = nullptr;
}

bool direct_sorted_enabled(int n)
{
    static const bool on = [] {
        const char *e = std::getenv("NB_DIRECT_SORTED");
        return !(e && std::strcmp(e, "0") == 0);
    }();
    return on && n >= 8192;
}

// Boxes of tiles of the plan's block size, then the kernel.
static nb_status run_sorted(const DirectPlan &p, const float4 *hi, const float4 *lo, int n,
                            double eps2, SortedBuffers &b, cudaStream_t st, float **psum_out)
{
    const int ntiles = (n + p.block - 1) / p.block;
    NB_TRY(b.boxes.reserve(sizeof(float4) * 2 * (size_t)ntiles));
    NB_TRY(b.partials.reserve(sizeof(float) * 6 * (size_t)n * p.segments));
    tile_box_kernel<<<ntiles, p.block, 0, st>>>(hi, n, b.boxes.as<float4>());
    NB_LAUNCH_CHECK();
    float *psum = b.partials.as<float>();
    float *pcomp = psum + 3 * (size_t)n * p.segments;
    if (!launch_sorted(p, st, hi, lo, b.boxes.as<float4>(), n, eps2, psum, pcomp, nullptr))
        return fail(NB_ERR_UNSUPPORTED, "direct_mixed_sorted: unsupported tile shape");
    NB_LAUNCH_CHECK();
    *psum_out = psum;
    return NB_OK;
}

static nb_status autotune_sorted(const float4 *hi, const float4 *lo, int n, double eps2,
                                 SortedBuffers &b, cudaStream_t st, DirectPlan *best)
{
    cudaEvent_t e0, e1;
    NB_CUDA_TRY(cudaEventCreate(&e0));
    NB_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    for (int k = 0; k < kNumSortedShapes; ++k) {
        const DirectPlan p = sorted_plan_for_shape(n, kSortedShapes[k].block, kSortedShapes[k].ipt);
        float *psum = nullptr;
        NB_TRY(run_sorted(p, hi, lo, n, eps2, b, st, &psum));
        cudaEventRecord(e0, st);
        for (int r = 0; r < 2; ++r) NB_TRY(run_sorted(p, hi, lo, n, eps2, b, st, &psum));
        cudaEventRecord(e1, st);
        NB_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
            best_ms = ms;
            *best = p;
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
    if (!b.sorter) b.sorter = bh_create();
    const uint32_t *order = nullptr;
    const double *centre = nullptr;
    // 10 levels of the Morton curve: cells far smaller than an i-block
    NB_TRY(bh_morton_order(b.sorter, x, y, z, n, 10, st, &order, &centre));
    NB_TRY(b.hi.reserve(sizeof(float4) * (size_t)n));
    NB_TRY(b.lo.reserve(sizeof(float4) * (size_t)n));
    float4 *hi = b.hi.as<float4>(), *lo = b.lo.as<float4>();
    split_sorted_kernel<<<(n + 255) / 256, 256, 0, st>>>(order, x, y, z, m, n, centre, hi, lo);
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
        if (!(e && std::strcmp(e, "0") == 0)) NB_TRY(autotune_sorted(hi, lo, n, eps2, b, st, &p));
        else p = sorted_plan_for_shape(n, 256, 4);
    }
    if (timer && timer->start) NB_CUDA_TRY(cudaEventRecord(timer->start, st));
    float *psum = nullptr;
    NB_TRY(run_sorted(p, hi, lo, n, eps2, b, st, &psum));
    if (timer && timer->stop) NB_CUDA_TRY(cudaEventRecord(timer->stop, st));
    float *pcomp = psum + 3 * (size_t)n * p.segments;
    combine_sorted_kernel<<<(n + 255) / 256, 256, 0, st>>>(psum, pcomp, n, p.segments, G, order,
                                                          ax, ay, az);
    NB_LAUNCH_CHECK();
    return NB_OK;
}

} // namespace nb
