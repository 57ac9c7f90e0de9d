// nb_bh.cu -- Barnes-Hut on sm_103a: 63-bit Morton encode, LSD radix sort,
// a parallel octree build read off the sorted codes, monopoles from FP64 prefix
// sums, and a warp-cooperative walk over child groups.
//
// Replaces BarnesHutForceCalculator (CUDA/src/force_calculator_barnes_hut.cu):
// six CUB min/max passes (:108-173), a 30-bit Morton code (:217-251), a CUB pair
// sort (:254-273), a level-by-level octree build with a host round trip and a
// cudaMalloc/cudaFree set per level (:294-492), ten per-level COM launches
// (:494-578) and a per-thread 50-entry stack walk that silently falls back to a
// monopole when the stack is full (:15-91).
//
// Tree rule.  The octree is the reference CPU tree's set of non-empty cells
// (CPU/src/force_calculator_barnes_hut_optimized.cpp): root cube centred on the
// bounding box with side max extent + 1e-9 (:105-124); a cell splits while it
// holds more than leaf_capacity bodies and its half side is >= 1e-9 (:138-173,
// :206-211), here also at most 21 levels (63-bit codes).  A body's code is the
// sequence of octants it falls into, computed with the CPU tree's own FP64
// comparisons and child-centre additions, so codes, sort order and topology
// equal the CPU restatement bit for bit.  Digits are x-high (x=4, y=2, z=1),
// the Morton order of force_calculator_barnes_hut.cu:243-248.
//
// Build.  After the sort, body i starts a node at depth d exactly when its
// depth-d cell begins at i and that cell's parent holds more than
// leaf_capacity bodies.  The nodes starting at i form a chain of consecutive
// depths that ends at the first leaf; one thread per body finds its chain by
// galloping over the sorted codes, an exclusive scan of the chain lengths
// numbers every node in preorder (depth-first, children in Morton order), and
// the node after a cell's subtree -- its skip pointer -- is simply the first
// node of the body that follows the cell.  Masses and centres of mass come
// from FP64 prefix sums of (m, m x, m y, m z) over the sorted bodies (positions
// relative to the root centre), so no level-by-level pass is needed.
//
// Walk.  One warp walks for 64 consecutive sorted bodies, two per lane.  At
// each node every body applies the reference's opening test (open when size^2
// >= theta^2 d^2 to the COM, or when the node holds the body); the warp opens
// the node if any body does (so each body gets a refinement of its own walk,
// never a coarser one).  The children of every node are stored together (a
// group): the warp reads a group in one round trip, adds the monopoles of the
// children no body opens and the bodies of opened leaves, and pushes the
// groups of opened internal children on its stack, which holds the deepest
// tree's groups.  The stackless preorder walk over skip pointers finds the
// same interactions (NB_BH_WALK=preorder).  Accelerations are scattered back
// to the original order in FP64, multiplied by G.
#include "nb_internal.h"
#include "nb_check.cuh"
#include "nb_curve.cuh"
#include "nb_pair.cuh"

#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace nb {

namespace {

constexpr int kMaxLevels = 21;

struct alignas(32) D4 {
    double x, y, z, w;
};

__host__ __device__ __forceinline__ D4 d4_add(const D4 &a, const D4 &b)
{
    return D4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w};
}

struct BHRoot {
    double cx, cy, cz, size;        // root cube (bh_*_order hand out &cx: centre, then side)
    double off[kMaxLevels];         // child-centre offset below depth l: size * 2^-(l+2)
    float size2[kMaxLevels + 1];    // squared side of a depth-d cell (opening test)
    int levels;                     // depths the root may split into (<= 21)
    int pad;
};

// A leaf is the node whose skip pointer is the next node (no subtree).
struct alignas(32) BHNode {
    float4 com_mass;  // centre of mass relative to the root centre, mass
    int first;        // first sorted body
    int count;        // bodies in the cell
    int skip;         // next node (preorder) outside this subtree
    float size2;      // squared side of the cell (the opening test's size^2)
};
static_assert(sizeof(BHNode) == 32, "node layout");

struct BHStats {
    unsigned long long m2p, p2p;  // terms of the last walk (reset by every build/refit)
    int leaves, max_depth;
    unsigned long long total;     // terms of every walk of this tree object (never reset)
};

// ------------------------------------------------------------ bounding box
__global__ void __launch_bounds__(256)
bbox_partial_kernel(const double *__restrict__ x, const double *__restrict__ y,
                    const double *__restrict__ z, int n, double *__restrict__ part)
{
    constexpr long long kMax = 0x7fffffffffffffffll, kMin = -kMax - 1;
    __shared__ long long sh[6][8];
    long long v[6] = {kMax, kMax, kMax, kMin, kMin, kMin};
    const double *ax[3] = {x, y, z};
    // four grid strides per iteration: twelve loads in flight per thread
    const int stride = gridDim.x * 256;
    int i = blockIdx.x * 256 + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        double p[3][4];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int u = 0; u < 4; ++u) p[c][u] = ax[c][i + u * stride];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                v[c] = min(v[c], order_key(p[c][u], kMax));
                v[c + 3] = max(v[c + 3], order_key(p[c][u], kMin));
            }
    }
    for (; i < n; i += stride)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double q = ax[c][i];
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
    if (threadIdx.x < 6) {
        const int c = threadIdx.x;
        long long r = sh[c][0];
        for (int w = 1; w < 8; ++w) r = c < 3 ? min(r, sh[c][w]) : max(r, sh[c][w]);
        // a block that saw only NaN (or nothing) reports the neutral value
        const bool empty = r == (c < 3 ? kMax : kMin);
        part[blockIdx.x * 6 + c] = empty ? (c < 3 ? 1e308 : -1e308) : key_value(r);
    }
}

// One block: reduce the partials, then thread 0 derives the root cube by the
// CPU tree's rule (force_calculator_barnes_hut_optimized.cpp:112-124,
// std::max(a,b) = a<b?b:a).  Min and max are exact, so the order of the
// reduction does not matter.
__global__ void __launch_bounds__(256)
bbox_final_kernel(const double *__restrict__ part, int nparts, BHRoot *root)
{
    __shared__ double sh[6][256];
    double v[6] = {1e308, 1e308, 1e308, -1e308, -1e308, -1e308};
    for (int b = threadIdx.x; b < nparts; b += 256) {
        for (int k = 0; k < 3; ++k) v[k] = fmin(v[k], part[b * 6 + k]);
        for (int k = 3; k < 6; ++k) v[k] = fmax(v[k], part[b * 6 + k]);
    }
    for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            for (int k = 0; k < 3; ++k)
                sh[k][threadIdx.x] = fmin(sh[k][threadIdx.x], sh[k][threadIdx.x + w]);
            for (int k = 3; k < 6; ++k)
                sh[k][threadIdx.x] = fmax(sh[k][threadIdx.x], sh[k][threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    for (int k = 0; k < 6; ++k) v[k] = sh[k][0];
    const double ex = v[3] - v[0], ey = v[4] - v[1], ez = v[5] - v[2];
    const double eyz = (ey < ez) ? ez : ey;
    double size = ((ex < eyz) ? eyz : ex) + 1e-9;
    root->cx = (v[0] + v[3]) / 2;
    root->cy = (v[1] + v[4]) / 2;
    root->cz = (v[2] + v[5]) / 2;
    root->size = size;
    int lv = 0;
    double s = size;
    while (lv < kMaxLevels) {
        const double half = s / 2.0;
        if (half < 1e-9) break;
        s = half;
        ++lv;
    }
    root->levels = lv;
    s = size;
    for (int l = 0; l < kMaxLevels; ++l) {
        root->size2[l] = (float)(s * s);
        const double half = s / 2.0;
        root->off[l] = half / 2.0;
        s = half;
    }
    root->size2[kMaxLevels] = (float)(s * s);
}

// ------------------------------------------------------------ Morton encode
// Fast path of one axis: the cell index on the ideal 2^21 grid of the root
// cube and whether the position is far enough from every grid line that the
// CPU tree's rounded running centres cannot compare differently.  f carries a
// few roundings of ~2^-31 grid cells; the margin (>= 1e-6 cells) covers them.
// Five FP64 operations (the FP64 pipe bounds this kernel): f, its floor as an
// integer, back to FP64, the fraction, and the fraction in FP32 (an error of
// ~2^-24, far below the margin) for the two comparisons.
__device__ __forceinline__ bool grid_index(double p, double lo_scaled, double scale,
                                           float margin, uint64_t *q)
{
    const double f = fma(p, scale, -lo_scaled);
    const long long fl = min(max(__double2ll_rd(f), 0ll), 2097151ll);
    *q = (uint64_t)fl;
    const float frac = __double2float_rn(f - (double)fl);  // in [0, 1) unless clamped
    return frac > margin && frac < 1.0f - margin;
}

__global__ void __launch_bounds__(256)
encode_kernel(const double *__restrict__ x, const double *__restrict__ y,
              const double *__restrict__ z, int n, const BHRoot *__restrict__ root,
              uint64_t *__restrict__ keys, uint32_t *__restrict__ vals)
{
    __shared__ double off[kMaxLevels];
    __shared__ double c0[3], lo_scaled[3], scale;
    __shared__ float margin;
    __shared__ int levels;
    if (threadIdx.x < kMaxLevels) off[threadIdx.x] = root->off[threadIdx.x];
    if (threadIdx.x == 0) {
        c0[0] = root->cx; c0[1] = root->cy; c0[2] = root->cz;
        levels = root->levels;
        const double size = root->size;
        scale = 2097152.0 / size;
        double cmax = 0.0;
        for (int k = 0; k < 3; ++k) {
            lo_scaled[k] = (c0[k] - size / 2) * scale;
            cmax = fmax(cmax, fabs(c0[k]));
        }
        // Running centres accumulate at most 21 roundings of half an ulp of
        // |centre| <= cmax + size; the fast index adds a few more roundings
        // (of |p| * scale and of lo * scale: 2^-52 (cmax + size) scale each).
        // Positions farther than this from every grid line index exactly.
        const double u_c = ldexp(1.0, ilogb(cmax + size) - 52);
        const double u_s = ldexp(1.0, ilogb(size) - 52);
        margin = (float)((32.0 * u_c + 4.0 * u_s) * scale + 1e-6);
    }
    __syncthreads();
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const double px = x[i], py = y[i], pz = z[i];
    uint64_t qx, qy, qz;
    const bool okx = grid_index(px, lo_scaled[0], scale, margin, &qx);
    const bool oky = grid_index(py, lo_scaled[1], scale, margin, &qy);
    const bool okz = grid_index(pz, lo_scaled[2], scale, margin, &qz);
    if (okx && oky && okz) {
        uint64_t code = (spread21(qx) << 2) | (spread21(qy) << 1) | spread21(qz);
        const int drop = 3 * (kMaxLevels - levels);  // digits below the split limit are 0
        if (drop >= 63) code = 0;
        else code = (code >> drop) << drop;
        keys[i] = code;
        vals[i] = (uint32_t)i;
        return;
    }
    // Exact path: the CPU tree's own comparisons and child-centre additions.
    double cx = c0[0], cy = c0[1], cz = c0[2];
    uint64_t code = 0;
    for (int l = 0; l < kMaxLevels; ++l) {
        uint64_t d = 0;
        if (l < levels) {
            const bool bx = px >= cx, by = py >= cy, bz = pz >= cz;
            d = ((uint64_t)bx << 2) | ((uint64_t)by << 1) | (uint64_t)bz;
            const double o = off[l];
            cx = __dadd_rn(cx, bx ? o : -o);
            cy = __dadd_rn(cy, by ? o : -o);
            cz = __dadd_rn(cz, bz ? o : -o);
        }
        code = (code << 3) | d;
    }
    keys[i] = code;
    vals[i] = (uint32_t)i;
}

// ------------------------------------------------------------ Hilbert encode
// keys[i] = the 30-bit Hilbert index of body i in bits 33..62 (the bits a
// 10-level Morton sort orders by), vals[i] = i.
__global__ void __launch_bounds__(256)
hilbert_kernel(const double *__restrict__ x, const double *__restrict__ y,
               const double *__restrict__ z, int n, const BHRoot *__restrict__ root,
               uint64_t *__restrict__ keys, uint32_t *__restrict__ vals)
{
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const double size = root->size, scale = 1024.0 / size;
    const double p[3] = {x[i], y[i], z[i]}, c[3] = {root->cx, root->cy, root->cz};
    uint32_t g[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double f = floor((p[k] - (c[k] - size / 2)) * scale);
        g[k] = (uint32_t)fmin(fmax(f, 0.0), 1023.0);
    }
    keys[i] = (uint64_t)hilbert_index30(g[0], g[1], g[2]) << 33;
    vals[i] = (uint32_t)i;
}

// ------------------------------------------------------------ scans (fixed order)
template <class T> struct Add;
template <> struct Add<int> {
    __device__ static int zero() { return 0; }
    __device__ static int op(int a, int b) { return a + b; }
};
template <> struct Add<D4> {
    __device__ static D4 zero() { return D4{0.0, 0.0, 0.0, 0.0}; }
    __device__ static D4 op(const D4 &a, const D4 &b) { return d4_add(a, b); }
};

// Elements per thread of the scans: more for the FP64 moments, whose warp
// and block steps run on GB300's narrow FP64 pipe, so fewer of them per
// element pays.
template <class T> struct ScanItems { static constexpr int n = 4; };
template <> struct ScanItems<D4> { static constexpr int n = 8; };
template <class T> __host__ __device__ constexpr int scan_tile() { return 256 * ScanItems<T>::n; }

__device__ __forceinline__ int shfl_up(int v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ D4 shfl_up(const D4 &v, int d)
{
    return D4{__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
              __shfl_up_sync(0xffffffffu, v.z, d), __shfl_up_sync(0xffffffffu, v.w, d)};
}

// Inclusive scan of one value per lane over a warp (shuffles).
template <class T>
__device__ __forceinline__ T warp_inclusive(T v, int lane)
{
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const T u = shfl_up(v, off);
        if (lane >= off) v = Add<T>::op(u, v);
    }
    return v;
}

// Exclusive scan of one value per thread over a block of NW warps: each warp
// scans its lanes, warp 0 scans the warp totals (the FP64 pipe is narrow, so
// no thread adds up all of them itself), and *total receives the block's
// sum.  Every thread of the block must call it; warp_sums holds NW + 1.
template <class T, int NW>
__device__ __forceinline__ T block_exclusive(T s, T *warp_sums, T *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const T inc = warp_inclusive(s, lane);
    if (lane == 31) warp_sums[warp] = inc;
    T excl = shfl_up(inc, 1);
    if (lane == 0) excl = Add<T>::zero();
    __syncthreads();
    if (warp == 0) {
        const T w = lane < NW ? warp_sums[lane] : Add<T>::zero();
        const T wi = warp_inclusive(w, lane);
        T we = shfl_up(wi, 1);
        if (lane == 0) we = Add<T>::zero();
        __syncwarp();
        if (lane < NW) warp_sums[lane] = we;
        if (lane == NW - 1) warp_sums[NW] = wi;
    }
    __syncthreads();
    *total = warp_sums[NW];
    return Add<T>::op(warp_sums[warp], excl);
}

// sums[b] = the sum of tile b (scan_tile<T>() elements): a tree in shared memory,
// whose idle warps skip their steps (fewer FP64 adds than a shuffle
// reduction, in which every lane adds at every step).
template <class T>
__global__ void __launch_bounds__(256)
scan_reduce_kernel(const T *__restrict__ in, int n, T *__restrict__ sums)
{
    constexpr int kItems = ScanItems<T>::n;
    __shared__ T sh[256];
    const int base = blockIdx.x * scan_tile<T>() + threadIdx.x * kItems;
    T s = Add<T>::zero();
#pragma unroll
    for (int k = 0; k < kItems; ++k)
        if (base + k < n) s = Add<T>::op(s, in[base + k]);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = Add<T>::op(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = sh[0];
}

// Exclusive scan of the tile sums in place, one block of up to 1024 threads
// (a warp per 32 sums: the FP64 steps of a block scan run on one SM's narrow
// FP64 pipe, so idle warps would only cost time).
template <class T>
__global__ void __launch_bounds__(1024) scan_top_kernel(T *__restrict__ a, int len)
{
    __shared__ T warp_sums[33];
    const int t = threadIdx.x;
    if (t < 33) warp_sums[t] = Add<T>::zero();  // the warps the block lacks add nothing
    __syncthreads();
    const int chunk = (len + (int)blockDim.x - 1) / (int)blockDim.x;
    const int b = t * chunk, e = min(len, b + chunk);
    T s = Add<T>::zero();
    for (int k = b; k < e; ++k) s = Add<T>::op(s, a[k]);
    T total;
    T run = block_exclusive<T, 32>(s, warp_sums, &total);
    for (int k = b; k < e; ++k) {
        const T v = a[k];
        a[k] = run;
        run = Add<T>::op(run, v);
    }
}

// out[i] = sum_{k<i} in[k] for i in [0, n], out has n+1 entries.
template <class T>
__global__ void __launch_bounds__(256)
scan_apply_kernel(const T *__restrict__ in, int n, const T *__restrict__ block_off,
                  T *__restrict__ out)
{
    constexpr int kItems = ScanItems<T>::n;
    __shared__ T warp_sums[9];
    const int base = blockIdx.x * scan_tile<T>() + threadIdx.x * kItems;
    T s = Add<T>::zero();
#pragma unroll
    for (int k = 0; k < kItems; ++k)
        if (base + k < n) s = Add<T>::op(s, in[base + k]);
    T total;
    T run = Add<T>::op(block_off[blockIdx.x], block_exclusive<T, 8>(s, warp_sums, &total));
#pragma unroll
    for (int k = 0; k < kItems; ++k) {  // the thread's elements again (L1)
        if (base + k < n) {
            const T v = in[base + k];
            out[base + k] = run;
            run = Add<T>::op(run, v);
        }
        if (base + k == n - 1) out[n] = run;
    }
}

// ------------------------------------------------------------ radix sort
constexpr int kSortWarps = 8;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortWarps * 32 * kSortRounds;  // 2048 keys
// Up to this many tiles (n <= 262,144) a scatter block sums the per-tile digit
// counts itself instead of a separate scan pass.
constexpr int kSortDirectTiles = 128;
// Up to this many tiles (n <= 131,072) the scatter also counts the next pass's
// digits (a global atomic per key), so passes after the first need no
// histogram launch; above it the atomics cost more than the launch saves.
constexpr int kSortFusedTiles = 64;

__global__ void __launch_bounds__(256)
radix_hist_kernel(const uint64_t *__restrict__ keys, int n, int shift, int *__restrict__ counts,
                  int num_tiles)
{
    __shared__ int h[kSortWarps][256];
    const int warp = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < kSortWarps * 256; k += 256) (&h[0][0])[k] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int k = threadIdx.x; k < kSortTile; k += 256) {
        const int idx = base + k;
        if (idx < n) atomicAdd(&h[warp][(int)((keys[idx] >> shift) & 0xFF)], 1);
    }
    __syncthreads();
    int c = 0;
    for (int w = 0; w < kSortWarps; ++w) c += h[w][threadIdx.x];
    counts[threadIdx.x * num_tiles + blockIdx.x] = c;
}

// Stable scatter of one 8-bit digit.  Warp w of the block ranks keys
// [tile + w*256, +256) in rounds of 32 (lane order), so ranks follow the input
// order; per-warp digit counts are turned into per-warp offsets.  The tile is
// then put in digit order in shared memory and written out by consecutive
// threads, so each digit's run of the tile goes to consecutive addresses.  The
// tile's global offset per digit comes from the scanned histogram (offsets),
// or, when offsets is null (few tiles), from the per-tile counts directly:
// the digit's count in the earlier tiles plus all keys of smaller digits.
// next_counts (not for the last pass) receives the next pass's per-tile
// histogram, counted as the keys land (integer adds: any order gives the same
// counts), so that pass needs no histogram launch; each block also clears its
// column of zero_counts, the buffer the pass after next counts into.
__global__ void __launch_bounds__(256)
radix_scatter_kernel(const uint64_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                     uint64_t *__restrict__ kout, uint32_t *__restrict__ vout, int n, int shift,
                     const int *__restrict__ offsets, const int *__restrict__ counts,
                     int *__restrict__ next_counts, int *__restrict__ zero_counts, int num_tiles)
{
    __shared__ int wh[kSortWarps][256];
    __shared__ int toff[256];    // global position of the tile's first key of digit d
    __shared__ int tstart[256];  // position in the tile of its first key of digit d
    __shared__ int wsum[kSortWarps];
    __shared__ int dsum[kSortWarps + 1];
    __shared__ uint64_t skey[kSortTile];
    __shared__ uint32_t sval[kSortTile];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < kSortWarps * 256; k += 256) (&wh[0][0])[k] = 0;
    if (offsets) {
        toff[threadIdx.x] = offsets[threadIdx.x * num_tiles + blockIdx.x];
    } else {
        const int *row = counts + threadIdx.x * num_tiles;
        int before = 0, all = 0;
        for (int tl = 0; tl < num_tiles; ++tl) {
            const int c = row[tl];
            all += c;
            if (tl < (int)blockIdx.x) before += c;
        }
        int keys;
        toff[threadIdx.x] = block_exclusive<int, kSortWarps>(all, dsum, &keys) + before;
    }
    __syncthreads();
    const int tile0 = blockIdx.x * kSortTile;
    const int base = tile0 + warp * 32 * kSortRounds;
    uint64_t key[kSortRounds];
    uint32_t val[kSortRounds];
    int rank[kSortRounds], dig[kSortRounds];
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        const int idx = base + r * 32 + lane;
        const bool valid = idx < n;
        key[r] = valid ? kin[idx] : 0ull;
        val[r] = valid ? vin[idx] : 0u;
        const int d = valid ? (int)((key[r] >> shift) & 0xFF) : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int before = __popc(peers & ((1u << lane) - 1u));
        const int leader = 31 - __clz(peers);
        const int b = valid ? wh[warp][d] : 0;
        __syncwarp();
        if (valid && lane == leader) wh[warp][d] = b + __popc(peers);
        __syncwarp();
        rank[r] = b + before;
        dig[r] = d;
    }
    __syncthreads();
    {
        // per-warp offsets within the digit, and the tile's digit starts
        // (exclusive scan of the digit totals: warp shuffles, then warp sums)
        const int d = threadIdx.x;
        int run = 0;
        for (int w = 0; w < kSortWarps; ++w) {
            const int c = wh[w][d];
            wh[w][d] = run;
            run += c;
        }
        int inc = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += u;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        int before = 0;
        for (int w = 0; w < warp; ++w) before += wsum[w];
        tstart[d] = before + inc - run;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        const int d = dig[r];
        if (d >= 0) {
            const int lpos = tstart[d] + wh[warp][d] + rank[r];
            skey[lpos] = key[r];
            sval[lpos] = val[r];
        }
    }
    __syncthreads();
    const int count = min(kSortTile, n - tile0);
    for (int j = threadIdx.x; j < count; j += 256) {
        const uint64_t k = skey[j];
        const int d = (int)((k >> shift) & 0xFF);
        const int pos = toff[d] + (j - tstart[d]);
        if (!NB_IN_RANGE(pos, n)) continue;
        kout[pos] = k;
        vout[pos] = sval[j];
        if (next_counts)
            atomicAdd(&next_counts[(int)((k >> (shift + 8)) & 0xFF) * num_tiles + pos / kSortTile], 1);
    }
    if (zero_counts) zero_counts[threadIdx.x * num_tiles + blockIdx.x] = 0;
}

// ------------------------------------------------------------ gather
__global__ void __launch_bounds__(256)
gather_kernel(const uint32_t *__restrict__ order, const double *__restrict__ x,
              const double *__restrict__ y, const double *__restrict__ z,
              const double *__restrict__ m, int n, const BHRoot *__restrict__ root,
              float4 *__restrict__ body, D4 *__restrict__ moments)
{
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = order[i];
    if (!NB_IN_RANGE(o, n)) return;
    const double rx = x[o] - root->cx, ry = y[o] - root->cy, rz = z[o] - root->cz;
    const double mm = m[o];
    body[i] = make_float4((float)rx, (float)ry, (float)rz, (float)mm);
    moments[i] = D4{mm, mm * rx, mm * ry, mm * rz};
}

// Second moments m x x^T (relative to the root centre) of every sorted body,
// for the quadrupoles: a = (m x x, m y y, m z z, m x y), b = (m x z, m y z, 0, 0).
__global__ void __launch_bounds__(256)
gather2_kernel(const uint32_t *__restrict__ order, const double *__restrict__ x,
               const double *__restrict__ y, const double *__restrict__ z,
               const double *__restrict__ m, int n, const BHRoot *__restrict__ root,
               D4 *__restrict__ ma, D4 *__restrict__ mb)
{
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = order[i];
    const double rx = x[o] - root->cx, ry = y[o] - root->cy, rz = z[o] - root->cz;
    const double mm = m[o];
    ma[i] = D4{mm * rx * rx, mm * ry * ry, mm * rz * rz, mm * rx * ry};
    mb[i] = D4{mm * rx * rz, mm * ry * rz, 0.0, 0.0};
}

// ------------------------------------------------------------ tree build
// First index after i whose depth-d prefix differs from code[i]'s (galloping).
__device__ __forceinline__ int cell_end(const uint64_t *__restrict__ c, int n, int i, int d)
{
    if (d == 0) return n;
    const int sh = 63 - 3 * d;
    const uint64_t p = c[i] >> sh;
    int lo = i, hi, step = 1;
    while (true) {
        hi = lo + step;
        if (hi >= n) {
            hi = n;
            break;
        }
        if ((c[hi] >> sh) != p) break;
        lo = hi;
        step <<= 1;
    }
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if ((c[mid] >> sh) == p) lo = mid;
        else hi = mid;
    }
    return hi;
}

// First index of the depth-d cell that contains body i.
__device__ __forceinline__ int cell_start(const uint64_t *__restrict__ c, int i, int d)
{
    if (d == 0) return 0;
    const int sh = 63 - 3 * d;
    const uint64_t p = c[i] >> sh;
    int hi = i, lo, step = 1;
    while (true) {
        lo = hi - step;
        if (lo < 0) {
            lo = -1;
            break;
        }
        if ((c[lo] >> sh) != p) break;
        hi = lo;
        step <<= 1;
    }
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if ((c[mid] >> sh) == p) hi = mid;
        else lo = mid;
    }
    return hi;
}

// Depth of the first node starting at body i and the length of its chain
// (0 when no node starts at i); pstart[i]: the first body of that node's
// parent cell (when i starts a chain below the root).
__global__ void __launch_bounds__(256)
chain_kernel(const uint64_t *__restrict__ c, int n, int cap, const BHRoot *__restrict__ root,
             int *__restrict__ chain_len, int *__restrict__ chain_depth, int *__restrict__ pstart)
{
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const int levels = root->levels;
    int a = 0, L = 0;
    bool starts = true;
    if (i > 0) {
        const uint64_t x = c[i] ^ c[i - 1];
        const int common = x == 0 ? 63 : (__clzll((long long)x) - 1);
        const int s = min(common / 3, levels);
        if (s >= levels) {
            starts = false;
        } else {
            a = s + 1;
            const int ps = cell_start(c, i, s);
            const int pc = cell_end(c, n, i, s) - ps;
            starts = pc > cap;
            pstart[i] = ps;
        }
    }
    if (starts) {
        int d = a;
        while (true) {
            const int cnt = cell_end(c, n, i, d) - i;
            ++L;
            if (cnt > cap && d < levels) ++d;
            else break;
        }
    }
    chain_len[i] = L;
    chain_depth[i] = a;
}

// (centre of mass, mass) of the bodies between two prefix sums of
// (m, m x, m y, m z): the differences in FP64 (exact enough: the sums are
// FP64), the division in FP32 (two roundings more than an FP64 division
// rounded to FP32, ~1e-7 of the position; the FP64 pipe is a small fraction
// of the FP32 one and three FP64 divisions per node dominated this kernel).
__device__ __forceinline__ float4 monopole(const D4 &lo, const D4 &hi)
{
    const double mass = hi.x - lo.x;
    if (!(mass > 0.0)) return make_float4(0.f, 0.f, 0.f, 0.f);
    const float m = (float)mass;
    if (m > 1e-30f && m < 1e30f) {
        const float r = 1.0f / m;
        return make_float4((float)(hi.y - lo.y) * r, (float)(hi.z - lo.z) * r,
                           (float)(hi.w - lo.w) * r, m);
    }
    return make_float4((float)((hi.y - lo.y) / mass), (float)((hi.z - lo.z) / mass),
                       (float)((hi.w - lo.w) / mass), m);  // outside FP32's comfortable range
}

// The centre of a depth-d cell's parent, relative to the root centre (the
// frame of the walk's bodies), and the cell's octant in that parent (bit 0 x,
// bit 1 y, bit 2 z: the high side), in .w as an int; the root (d = 0), which
// has no parent, gets 8.  The cell is read off the Morton code of any of its
// bodies: digit k (x high) of the 3d-bit prefix halves the cube along each axis.
__device__ __forceinline__ float4 parent_centre(uint64_t code, int d, const BHRoot *root)
{
    if (d == 0) return make_float4(0.f, 0.f, 0.f, __int_as_float(8));
    const uint64_t pfx = code >> (63 - 3 * d);
    const int dig = (int)(pfx & 7u);
    uint32_t ix = 0, iy = 0, iz = 0;
    for (int k = 0; k < d - 1; ++k) {
        const int g = (int)((pfx >> (3 * (d - 1 - k))) & 7u);
        ix = 2 * ix + ((g >> 2) & 1);
        iy = 2 * iy + ((g >> 1) & 1);
        iz = 2 * iz + (g & 1);
    }
    const double side = ldexp(root->size, -(d - 1));  // the parent's side
    const double h = 0.5 * root->size;
    const int oct = ((dig >> 2) & 1) | (((dig >> 1) & 1) << 1) | ((dig & 1) << 2);
    return make_float4((float)(((double)ix + 0.5) * side - h), (float)(((double)iy + 0.5) * side - h),
                       (float)(((double)iz + 0.5) * side - h), __int_as_float(oct));
}

__global__ void __launch_bounds__(256)
node_kernel(const uint64_t *__restrict__ c, int n, int cap, const BHRoot *__restrict__ root,
            const int *__restrict__ chain_len, const int *__restrict__ chain_depth,
            const int *__restrict__ offsets, const D4 *__restrict__ P,
            BHNode *__restrict__ nodes, unsigned char *__restrict__ node_depth,
            const int *__restrict__ pstart, int *__restrict__ parent,
            unsigned char *__restrict__ octant, unsigned char *__restrict__ kidflag,
            BHStats *__restrict__ stats, int node_cap)
{
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i >= n) return;
    const int L = chain_len[i];
    if (L == 0) return;
    const int levels = root->levels;
    const int a = chain_depth[i];
    const int id0 = offsets[i];
    int leaves = 0, maxd = 0;
    for (int k = 0; k < L; ++k) {
        const int d = a + k;
        const int cnt = cell_end(c, n, i, d) - i;
        const bool leaf = !(cnt > cap && d < levels);
        if (!NB_IN_RANGE(id0 + k, node_cap) || !NB_IN_RANGE(i + cnt, n + 1)) break;
        BHNode nd;
        nd.com_mass = monopole(P[i], P[i + cnt]);
        nd.first = i;
        nd.count = cnt;
        nd.skip = offsets[i + cnt];
        nd.size2 = root->size2[d];
        nodes[id0 + k] = nd;
        node_depth[id0 + k] = (unsigned char)d;
        if (d > 0) {  // the parent: the previous node of the chain, or the one holding it
            int par = id0 + k - 1;
            if (k == 0) {
                const int j = pstart[i];
                par = offsets[j] + (d - 1 - chain_depth[j]);
            }
            const int oct = (int)((c[i] >> (63 - 3 * d)) & 7u);
            parent[id0 + k] = par;
            octant[id0 + k] = (unsigned char)oct;
            if (NB_IN_RANGE(par, node_cap)) kidflag[(size_t)par * 8 + oct] = 1;
        }
        leaves += leaf;
        maxd = max(maxd, d);
    }
    if (leaves) atomicAdd(&stats->leaves, leaves);
    atomicMax(&stats->max_depth, maxd);
}

// Parent centres and octants of every node (parent_centre), for the walk
// under the reference's opening rule only: read off the Morton code of the
// node's first body and its depth.
__global__ void __launch_bounds__(256)
pcen_kernel(const uint64_t *__restrict__ c, const BHNode *__restrict__ nodes,
            const unsigned char *__restrict__ node_depth, const int *__restrict__ total,
            const BHRoot *__restrict__ root, float4 *__restrict__ pcen)
{
    const int num = *total;
    for (int k = blockIdx.x * 256 + threadIdx.x; k < num; k += gridDim.x * 256)
        pcen[k] = parent_centre(c[nodes[k].first], node_depth[k], root);
}

// ------------------------------------------------------------ refit
// Tree reuse: the topology and body order of the last build are kept while
// the bodies move; every evaluation in between recomputes the monopoles from
// the bodies' current positions and replaces each cell's side by the larger of
// its cube side and the extent of its bodies' bounding box, so a drifted cell
// is opened at least as readily as a freshly built one would be.
__device__ __forceinline__ float box_ext2(float4 lo, float4 hi)
{
    const float e = fmaxf(hi.x - lo.x, fmaxf(hi.y - lo.y, hi.z - lo.z));
    return e * e;
}

// Monopoles of every node; bounding boxes and sides of the leaves.
__global__ void __launch_bounds__(256)
refit_kernel(BHNode *__restrict__ nodes, const int *__restrict__ total,
             const unsigned char *__restrict__ node_depth, const D4 *__restrict__ P,
             const BHRoot *__restrict__ root, const float4 *__restrict__ body,
             float4 *__restrict__ boxes)
{
    const int k = blockIdx.x * 256 + threadIdx.x;
    if (k >= *total) return;
    BHNode nd = nodes[k];
    nd.com_mass = monopole(P[nd.first], P[nd.first + nd.count]);
    if (nd.skip == k + 1) {  // leaf
        float4 mn = body[nd.first], mx = mn;
        for (int b = nd.first + 1; b < nd.first + nd.count; ++b) {
            const float4 q = body[b];
            mn = make_float4(fminf(mn.x, q.x), fminf(mn.y, q.y), fminf(mn.z, q.z), 0.f);
            mx = make_float4(fmaxf(mx.x, q.x), fmaxf(mx.y, q.y), fmaxf(mx.z, q.z), 0.f);
        }
        boxes[2 * k] = mn;
        boxes[2 * k + 1] = mx;
        nd.size2 = fmaxf(root->size2[node_depth[k]], box_ext2(mn, mx));
    }
    nodes[k] = nd;
}

// Internal nodes of depth d: box = union of the children's boxes (children:
// node + 1, then each child's skip pointer up to the node's own).
__global__ void __launch_bounds__(256)
refit_level_kernel(BHNode *__restrict__ nodes, const int *__restrict__ total,
                   const unsigned char *__restrict__ node_depth, int d,
                   const BHRoot *__restrict__ root, float4 *__restrict__ boxes)
{
    const int k = blockIdx.x * 256 + threadIdx.x;
    if (k >= *total || node_depth[k] != d) return;
    const int skip = nodes[k].skip;
    if (skip == k + 1) return;  // leaf: done by refit_kernel
    float4 mn = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f);
    float4 mx = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.f);
    for (int c = k + 1; c < skip; c = nodes[c].skip) {
        const float4 a = boxes[2 * c], b = boxes[2 * c + 1];
        mn = make_float4(fminf(mn.x, a.x), fminf(mn.y, a.y), fminf(mn.z, a.z), 0.f);
        mx = make_float4(fmaxf(mx.x, b.x), fmaxf(mx.y, b.y), fmaxf(mx.z, b.z), 0.f);
    }
    boxes[2 * k] = mn;
    boxes[2 * k + 1] = mx;
    nodes[k].size2 = fmaxf(root->size2[d], box_ext2(mn, mx));
}

// ------------------------------------------------------------ quadrupoles
// Traceless quadrupole of every node about its centre of mass, from the FP64
// prefix sums of the moments: with S = sum m x x^T - M c c^T (positions
// relative to the root centre, c the centre of mass),
// Q = 3 S - tr(S) I; stored as (Qxx, Qyy, Qzz, Qxy), (Qxz, Qyz, 0, 0).
__global__ void __launch_bounds__(256)
quad_kernel(const BHNode *__restrict__ nodes, const int *__restrict__ total, const D4 *__restrict__ P,
            const D4 *__restrict__ PA, const D4 *__restrict__ PB, float4 *__restrict__ quad)
{
    const int k = blockIdx.x * 256 + threadIdx.x;
    if (k >= *total) return;
    const int a = nodes[k].first, b = a + nodes[k].count;
    const double M = P[b].x - P[a].x;
    float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0;
    if (M > 0.0) {
        const double cx = (P[b].y - P[a].y) / M, cy = (P[b].z - P[a].z) / M,
                     cz = (P[b].w - P[a].w) / M;
        const double sxx = (PA[b].x - PA[a].x) - M * cx * cx;
        const double syy = (PA[b].y - PA[a].y) - M * cy * cy;
        const double szz = (PA[b].z - PA[a].z) - M * cz * cz;
        const double sxy = (PA[b].w - PA[a].w) - M * cx * cy;
        const double sxz = (PB[b].x - PB[a].x) - M * cx * cz;
        const double syz = (PB[b].y - PB[a].y) - M * cy * cz;
        const double tr = sxx + syy + szz;
        q0 = make_float4((float)(3.0 * sxx - tr), (float)(3.0 * syy - tr),
                         (float)(3.0 * szz - tr), (float)(3.0 * sxy));
        q1 = make_float4((float)(3.0 * sxz), (float)(3.0 * syz), 0.f, 0.f);
    }
    quad[2 * k] = q0;
    quad[2 * k + 1] = q1;
}

// ------------------------------------------------------------ walk
constexpr int kWalkBlock = 128;

// ZERO_SOFT: eps2 == 0, where the lane's own body (r2 == 0) contributes 0.
// QUAD: accepted cells act as monopole + quadrupole, a = G M r / |r|^3 +
// G (5/2 (r.Q r) r / |r|^2 - Q r) / |r|^5 with r from the body to the centre
// of mass (softened |r| throughout).
// The reference's opening rule (NB_FLAG_BH_REFERENCE_OPENING;
// CPU/src/force_calculator_barnes_hut_optimized.cpp and
// CUDA/src/force_calculator_barnes_hut.cu:60-73): of every node a walk opens,
// the child in the body's octant (relative to the node's centre) is opened
// too, whether or not it holds the body; the opening test applies to the
// other children.  A node is reached only after its parent was opened, so
// the walk asks, per node, whether the body lies on the node's side of its
// parent's centre on all three axes (pc from parent_centre).
__device__ __forceinline__ bool toward_body(float4 pc, float x, float y, float z)
{
    const int oct = __float_as_int(pc.w);
    return oct < 8 && ((x >= pc.x) == ((oct & 1) != 0)) && ((y >= pc.y) == ((oct & 2) != 0)) &&
           ((z >= pc.z) == ((oct & 4) != 0));
}

template <bool ZERO_SOFT, bool QUAD, bool DIR>
__global__ void __launch_bounds__(kWalkBlock)
walk_kernel(const BHNode *__restrict__ nodes, const int *__restrict__ total,
            const float4 *__restrict__ body, const uint32_t *__restrict__ order, int n,
            float theta2, float eps2, double G, double *__restrict__ ax,
            double *__restrict__ ay, double *__restrict__ az, BHStats *__restrict__ stats,
            const float4 *__restrict__ quad, const float4 *__restrict__ pcen)
{
    const int num_nodes = *total;
    const int lane = threadIdx.x & 31;
    const int warp0 = (blockIdx.x * kWalkBlock + threadIdx.x) - lane;
    if (warp0 >= n) return;  // whole warp past the end
    const int i = warp0 + lane;
    const bool valid = i < n;
    const float4 p = body[valid ? i : n - 1];
    const float2 npx = dup2(-p.x), npy = dup2(-p.y), npz = dup2(-p.z), e2 = dup2(eps2);
    float fx = 0.f, fy = 0.f, fz = 0.f;                         // monopoles, odd bodies
    float2 gx = dup2(0.f), gy = dup2(0.f), gz = dup2(0.f);     // leaf bodies in pairs
    unsigned m2p = 0, p2p = 0;
    int node = 0;
    while (node < num_nodes) {
        const BHNode nd = nodes[node];
        const float dx = nd.com_mass.x - p.x;
        const float dy = nd.com_mass.y - p.y;
        const float dz = nd.com_mass.z - p.z;
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const bool mine = (unsigned)(i - nd.first) < (unsigned)nd.count;
        bool open = valid && (mine || nd.size2 >= theta2 * d2);
        if (DIR) open = open || (valid && toward_body(pcen[node], p.x, p.y, p.z));
        if (__any_sync(0xffffffffu, open)) {
            if (nd.skip != node + 1) {  // internal: descend
                ++node;
                continue;
            }
            // leaf: its bodies, two per f32x2 instruction
            const int e = NB_IN_RANGE(nd.first, n) && NB_IN_RANGE(nd.first + nd.count - 1, n)
                              ? nd.first + nd.count
                              : nd.first;
            int b = nd.first;
            for (; b + 1 < e; b += 2) {
                const float4 q0 = body[b], q1 = body[b + 1];
                const float2 rx = add2(make_float2(q0.x, q1.x), npx);
                const float2 ry = add2(make_float2(q0.y, q1.y), npy);
                const float2 rz = add2(make_float2(q0.z, q1.z), npz);
                const float2 r2 = fma2(rz, rz, fma2(ry, ry, fma2(rx, rx, e2)));
                float2 inv = make_float2(rsqrt_mufu(r2.x), rsqrt_mufu(r2.y));
                if (ZERO_SOFT) {
                    inv.x = r2.x > 0.f ? inv.x : 0.f;
                    inv.y = r2.y > 0.f ? inv.y : 0.f;
                }
                const float2 s = mul2(mul2(make_float2(q0.w, q1.w), inv), mul2(inv, inv));
                gx = fma2(rx, s, gx);
                gy = fma2(ry, s, gy);
                gz = fma2(rz, s, gz);
            }
            if (b < e) {
                const float4 q = body[b];
                const float rx = q.x - p.x, ry = q.y - p.y, rz = q.z - p.z;
                const float r2 = fmaf(rz, rz, fmaf(ry, ry, fmaf(rx, rx, eps2)));
                float inv = rsqrt_mufu(r2);
                if (ZERO_SOFT) inv = r2 > 0.f ? inv : 0.f;
                const float s = (q.w * inv) * (inv * inv);
                fx = fmaf(rx, s, fx);
                fy = fmaf(ry, s, fy);
                fz = fmaf(rz, s, fz);
            }
            p2p += nd.count;
        } else {
            const float inv = rsqrt_mufu(d2 + eps2);
            const float inv2 = inv * inv;
            const float s = (nd.com_mass.w * inv) * inv2;
            fx = fmaf(dx, s, fx);
            fy = fmaf(dy, s, fy);
            fz = fmaf(dz, s, fz);
            if (QUAD) {
                const float4 q0 = quad[2 * node], q1 = quad[2 * node + 1];
                const float qx = fmaf(q0.x, dx, fmaf(q0.w, dy, q1.x * dz));
                const float qy = fmaf(q0.w, dx, fmaf(q0.y, dy, q1.y * dz));
                const float qz = fmaf(q1.x, dx, fmaf(q1.y, dy, q0.z * dz));
                const float rqr = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
                const float inv5 = (inv * inv2) * inv2;  // |r|^-5
                const float f = 2.5f * rqr * inv2;
                fx = fmaf(inv5, fmaf(f, dx, -qx), fx);
                fy = fmaf(inv5, fmaf(f, dy, -qy), fy);
                fz = fmaf(inv5, fmaf(f, dz, -qz), fz);
            }
            ++m2p;
        }
        if (!NB_IN_RANGE(nd.skip - node - 1, num_nodes)) break;  // skips only go forward
        node = nd.skip;
    }
    if (valid) {
        const uint32_t o = order[i];
        ax[o] = G * ((double)fx + ((double)gx.x + (double)gx.y));
        ay[o] = G * ((double)fy + ((double)gy.x + (double)gy.y));
        az[o] = G * ((double)fz + ((double)gz.x + (double)gz.y));
    }
    // every lane ran the same interactions: count once per valid lane
    const unsigned nv = __popc(__ballot_sync(0xffffffffu, valid));
    if (lane == 0) {
        atomicAdd(&stats->m2p, (unsigned long long)m2p * nv);
        atomicAdd(&stats->p2p, (unsigned long long)p2p * nv);
        atomicAdd(&stats->total, (unsigned long long)(m2p + p2p) * nv);
    }
}

// The same walk for 64 * NP consecutive sorted bodies per warp, 2 * NP per
// lane (body w0 + 32 k + lane for k < 2 NP, held as NP packed pairs): one node
// load, vote and branch serve them all, and their MAC, monopole and leaf terms
// run as f32x2 pairs.  The warp opens a node if any of its bodies does --
// never a coarser walk than any body's own.
template <bool ZERO_SOFT, bool QUAD, int NP, bool DIR>
__global__ void __launch_bounds__(kWalkBlock)
walk2_kernel(const BHNode *__restrict__ nodes, const int *__restrict__ total,
             const float4 *__restrict__ body, const uint32_t *__restrict__ order, int n,
             float theta2, float eps2, double G, double *__restrict__ ax,
             double *__restrict__ ay, double *__restrict__ az, BHStats *__restrict__ stats,
             const float4 *__restrict__ quad, const float4 *__restrict__ pcen)
{
    const int num_nodes = *total;
    constexpr int kPer = 64 * NP;  // bodies per warp
    const int lane = threadIdx.x & 31;
    const int w0 = ((blockIdx.x * kWalkBlock + threadIdx.x) >> 5) * kPer;
    if (w0 >= n) return;  // whole warp past the end
    int ia[NP], ib[NP];
    bool va[NP], vb[NP];
    float2 npx[NP], npy[NP], npz[NP], fx[NP], fy[NP], fz[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        ia[k] = w0 + 64 * k + lane;
        ib[k] = ia[k] + 32;
        va[k] = ia[k] < n;
        vb[k] = ib[k] < n;
        const float4 pa = body[va[k] ? ia[k] : n - 1], pb = body[vb[k] ? ib[k] : n - 1];
        npx[k] = make_float2(-pa.x, -pb.x);
        npy[k] = make_float2(-pa.y, -pb.y);
        npz[k] = make_float2(-pa.z, -pb.z);
        fx[k] = fy[k] = fz[k] = dup2(0.f);
    }
    const float2 e2 = dup2(eps2), t2 = dup2(theta2);
    unsigned m2p = 0, p2p = 0;
    int node = 0;
    while (node < num_nodes) {
        const BHNode nd = nodes[node];
        const float4 pc = DIR ? pcen[node] : make_float4(0.f, 0.f, 0.f, 0.f);
        float2 dx[NP], dy[NP], dz[NP], d2[NP];
        bool open = false;
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            dx[k] = add2(dup2(nd.com_mass.x), npx[k]);
            dy[k] = add2(dup2(nd.com_mass.y), npy[k]);
            dz[k] = add2(dup2(nd.com_mass.z), npz[k]);
            d2[k] = fma2(dz[k], dz[k], fma2(dy[k], dy[k], mul2(dx[k], dx[k])));
            const float2 td2 = mul2(t2, d2[k]);
            const bool oa = va[k] & (((unsigned)(ia[k] - nd.first) < (unsigned)nd.count) |
                                     (nd.size2 >= td2.x));
            const bool ob = vb[k] & (((unsigned)(ib[k] - nd.first) < (unsigned)nd.count) |
                                     (nd.size2 >= td2.y));
            open = open | oa | ob;
            if (DIR)
                open = open | (va[k] & toward_body(pc, -npx[k].x, -npy[k].x, -npz[k].x)) |
                       (vb[k] & toward_body(pc, -npx[k].y, -npy[k].y, -npz[k].y));
        }
        if (__any_sync(0xffffffffu, open)) {
            if (nd.skip != node + 1) {  // internal: descend
                ++node;
                continue;
            }
            const int e = NB_IN_RANGE(nd.first, n) && NB_IN_RANGE(nd.first + nd.count - 1, n)
                              ? nd.first + nd.count
                              : nd.first;
            for (int b = nd.first; b < e; ++b) {
                const float4 q = body[b];
#pragma unroll
                for (int k = 0; k < NP; ++k) {
                    const float2 rx = add2(dup2(q.x), npx[k]);
                    const float2 ry = add2(dup2(q.y), npy[k]);
                    const float2 rz = add2(dup2(q.z), npz[k]);
                    const float2 r2 = fma2(rz, rz, fma2(ry, ry, fma2(rx, rx, e2)));
                    float2 inv = make_float2(rsqrt_mufu(r2.x), rsqrt_mufu(r2.y));
                    if (ZERO_SOFT) {
                        inv.x = r2.x > 0.f ? inv.x : 0.f;
                        inv.y = r2.y > 0.f ? inv.y : 0.f;
                    }
                    const float2 s = mul2(mul2(dup2(q.w), inv), mul2(inv, inv));
                    fx[k] = fma2(rx, s, fx[k]);
                    fy[k] = fma2(ry, s, fy[k]);
                    fz[k] = fma2(rz, s, fz[k]);
                }
            }
            p2p += nd.count;
        } else {
            float4 q0, q1;
            if (QUAD) {
                q0 = quad[2 * node];
                q1 = quad[2 * node + 1];
            }
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                const float2 r2 = add2(d2[k], e2);
                const float2 inv = make_float2(rsqrt_mufu(r2.x), rsqrt_mufu(r2.y));
                const float2 inv2 = mul2(inv, inv);
                const float2 s = mul2(mul2(dup2(nd.com_mass.w), inv), inv2);
                fx[k] = fma2(dx[k], s, fx[k]);
                fy[k] = fma2(dy[k], s, fy[k]);
                fz[k] = fma2(dz[k], s, fz[k]);
                if (QUAD) {
                    const float2 qx = fma2(dup2(q0.x), dx[k],
                                           fma2(dup2(q0.w), dy[k], mul2(dup2(q1.x), dz[k])));
                    const float2 qy = fma2(dup2(q0.w), dx[k],
                                           fma2(dup2(q0.y), dy[k], mul2(dup2(q1.y), dz[k])));
                    const float2 qz = fma2(dup2(q1.x), dx[k],
                                           fma2(dup2(q1.y), dy[k], mul2(dup2(q0.z), dz[k])));
                    const float2 rqr = fma2(dx[k], qx, fma2(dy[k], qy, mul2(dz[k], qz)));
                    const float2 inv5 = mul2(mul2(inv, inv2), inv2);
                    const float2 f = mul2(mul2(dup2(2.5f), rqr), inv2);
                    fx[k] = fma2(inv5, fma2(f, dx[k], make_float2(-qx.x, -qx.y)), fx[k]);
                    fy[k] = fma2(inv5, fma2(f, dy[k], make_float2(-qy.x, -qy.y)), fy[k]);
                    fz[k] = fma2(inv5, fma2(f, dz[k], make_float2(-qz.x, -qz.y)), fz[k]);
                }
            }
            ++m2p;
        }
        if (!NB_IN_RANGE(nd.skip - node - 1, num_nodes)) break;  // skips only go forward
        node = nd.skip;
    }
    unsigned nv = 0;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        if (va[k]) {
            const uint32_t o = order[ia[k]];
            ax[o] = G * (double)fx[k].x;
            ay[o] = G * (double)fy[k].x;
            az[o] = G * (double)fz[k].x;
        }
        if (vb[k]) {
            const uint32_t o = order[ib[k]];
            ax[o] = G * (double)fx[k].y;
            ay[o] = G * (double)fy[k].y;
            az[o] = G * (double)fz[k].y;
        }
        nv += __popc(__ballot_sync(0xffffffffu, va[k])) + __popc(__ballot_sync(0xffffffffu, vb[k]));
    }
    if (lane == 0) {
        atomicAdd(&stats->m2p, (unsigned long long)m2p * nv);
        atomicAdd(&stats->p2p, (unsigned long long)p2p * nv);
        atomicAdd(&stats->total, (unsigned long long)(m2p + p2p) * nv);
    }
}

// ------------------------------------------------------------ child groups
// The group walk reads the children of a node together: gnodes holds, for
// every internal node, its children's records contiguously and in Morton order
// (a group), and group 0 is the root alone.  node_kernel records every node's
// parent and octant and marks byte (parent, octant) of an 8-byte row per node
// (each child its own byte: no atomics); alloc_groups_kernel packs a row into
// the node's octant mask and claims a place for each group from a counter (every node
// but the root is the child of exactly one node, so there are as many records
// as nodes; where a group lands changes no result, since the walk's arithmetic
// follows the groups' contents), and group_kernel writes each record with its
// children count, its parent centre and, for the quadrupole walk, its
// quadrupole beside it.  Both run over the node count read on the device.
struct alignas(32) BHGNode {
    float4 com_mass;  // as BHNode
    float size2;
    int first, count;
    int kids;         // the record of the node's first child (-1: a leaf)
};
static_assert(sizeof(BHGNode) == 32, "group record layout");

// A place for the group of every node with children (occ: the mask of its
// non-empty octants, packed from its row of kidflag): a block numbers its
// nodes' groups by a scan and claims their span from the counter with one
// atomic.
__global__ void __launch_bounds__(256)
alloc_groups_kernel(const unsigned char *__restrict__ kidflag, const int *__restrict__ total,
                    unsigned *__restrict__ occ, int *__restrict__ base, int *__restrict__ next)
{
    __shared__ int warp_sums[9];
    __shared__ int span0;
    const int num = *total;
    for (int k0 = blockIdx.x * 256; k0 < num; k0 += gridDim.x * 256) {
        const int k = k0 + threadIdx.x;
        unsigned o = 0;
        if (k < num) {
            const uint2 f = reinterpret_cast<const uint2 *>(kidflag)[k];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                o |= ((f.x >> (8 * b)) & 0xFFu) ? 1u << b : 0u;
                o |= ((f.y >> (8 * b)) & 0xFFu) ? 1u << (b + 4) : 0u;
            }
            occ[k] = o;
        }
        const int nk = __popc(o);
        int span;
        const int off = block_exclusive<int, 8>(nk, warp_sums, &span);
        if (threadIdx.x == 0) span0 = atomicAdd(next, span);
        __syncthreads();
        if (nk > 0) base[k] = span0 + off;
        __syncthreads();  // span0 and warp_sums are reused by the next round
    }
}

// Every node's record: the root at 0, a child at its parent's group place
// plus its rank among the parent's non-empty octants (Morton order).
__global__ void __launch_bounds__(256)
group_kernel(const BHNode *__restrict__ nodes, const int *__restrict__ total,
             const unsigned *__restrict__ occ, const int *__restrict__ base,
             const int *__restrict__ parent, const unsigned char *__restrict__ octant,
             const float4 *__restrict__ pcen, const float4 *__restrict__ quad,
             BHGNode *__restrict__ gnodes, unsigned char *__restrict__ gnk,
             float4 *__restrict__ gpcen, float4 *__restrict__ gquad)
{
    const int num = *total;
    for (int k = blockIdx.x * 256 + threadIdx.x; k < num; k += gridDim.x * 256) {
        int pos = 0;
        if (k > 0) {
            const int par = parent[k];
            if (!NB_IN_RANGE(par, num)) continue;
            pos = 1 + base[par] + __popc(occ[par] & ((1u << octant[k]) - 1u));
        }
        if (!NB_IN_RANGE(pos, num)) continue;
        const BHNode nd = nodes[k];
        const unsigned o = occ[k];
        BHGNode g;
        g.com_mass = nd.com_mass;
        g.size2 = nd.size2;
        g.first = nd.first;
        g.count = nd.count;
        g.kids = o ? 1 + base[k] : -1;
        gnodes[pos] = g;
        gnk[pos] = (unsigned char)__popc(o);
        if (pcen) gpcen[pos] = pcen[k];
        if (quad) {
            gquad[2 * pos] = quad[2 * k];
            gquad[2 * pos + 1] = quad[2 * k + 1];
        }
    }
}

// A depth-first walk over groups keeps, per level of its current path, at most
// 7 groups of unvisited siblings, plus the at most 8 groups the last group
// pushed; groups lie at levels 0 .. kMaxLevels.
constexpr int kGroupBlock = 32;  // threads of a group-walk CTA
constexpr int kWalkWarps = kGroupBlock / 32;
constexpr int kGroupStack = 8 * (kMaxLevels + 1);

// The walk of walk2_kernel (64 NP bodies per warp, 2 NP per lane as packed
// pairs; the same opening rule, decided for the whole warp) over child groups:
// one round trip to memory brings a group's records into the warp's shared
// memory, and the warp then tests the children one after the other, adding
// the monopoles of the children no body opens, summing opened leaves' bodies,
// and pushing the groups of opened internal children onto its stack.  The
// interactions are those of walk2_kernel; only their order differs.
template <bool ZERO_SOFT, bool QUAD, int NP, bool DIR>
__global__ void __launch_bounds__(kGroupBlock)
group_walk_kernel(const BHGNode *__restrict__ gnodes, const unsigned char *__restrict__ gnk,
                  const int *__restrict__ total, const float4 *__restrict__ body,
                  const uint32_t *__restrict__ order, int n, float theta2, float eps2, double G,
                  double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az,
                  BHStats *__restrict__ stats, const float4 *__restrict__ gquad,
                  const float4 *__restrict__ gpcen)
{
    __shared__ BHGNode s_rec[kWalkWarps][8];
    __shared__ float4 s_quad[kWalkWarps][QUAD ? 16 : 1];
    __shared__ float4 s_pc[kWalkWarps][DIR ? 8 : 1];
    __shared__ int2 s_stack[kWalkWarps][kGroupStack];
    constexpr int kPer = 64 * NP;  // bodies per warp
    const int num_nodes = *total;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int w0 = ((blockIdx.x * kGroupBlock + threadIdx.x) >> 5) * kPer;
    if (w0 >= n) return;  // whole warp past the end
    const int wend = min(n, w0 + kPer);  // the warp's bodies: [w0, wend)
    int ia[NP], ib[NP];
    bool va[NP], vb[NP];
    float2 npx[NP], npy[NP], npz[NP], fx[NP], fy[NP], fz[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        ia[k] = w0 + 64 * k + lane;
        ib[k] = ia[k] + 32;
        va[k] = ia[k] < n;
        vb[k] = ib[k] < n;
        // a slot past n walks with body w0: its tests repeat that body's
        const float4 pa = body[va[k] ? ia[k] : w0], pb = body[vb[k] ? ib[k] : w0];
        npx[k] = make_float2(-pa.x, -pb.x);
        npy[k] = make_float2(-pa.y, -pb.y);
        npz[k] = make_float2(-pa.z, -pb.z);
        fx[k] = fy[k] = fz[k] = dup2(0.f);
    }
    const float2 e2 = dup2(eps2), t2 = dup2(theta2);
    unsigned m2p = 0, p2p = 0;
    int sp = 1;
    if (lane == 0) s_stack[w][0] = make_int2(0, 1);
    while (sp > 0) {
        __syncwarp();
        const int2 g = s_stack[w][--sp];
        if (!NB_IN_RANGE(g.x + g.y - 1, num_nodes)) break;
        int mynk = 0;
        if (lane < g.y) {
            s_rec[w][lane] = gnodes[g.x + lane];
            mynk = gnk[g.x + lane];
            if (DIR) s_pc[w][lane] = gpcen[g.x + lane];
        }
        if (QUAD && lane < 2 * g.y) s_quad[w][lane] = gquad[2 * g.x + lane];
        __syncwarp();
        for (int c = 0; c < g.y; ++c) {
            const BHGNode nd = s_rec[w][c];
            const float4 pc = DIR ? s_pc[w][c] : make_float4(0.f, 0.f, 0.f, 0.f);
            float2 dx[NP], dy[NP], dz[NP], d2[NP];
            // a node that holds one of the warp's bodies is opened (each body's
            // own cell); the others by the opening test of any body
            bool open = nd.first < wend && nd.first + nd.count > w0;
#pragma unroll
            for (int k = 0; k < NP; ++k) {
                dx[k] = add2(dup2(nd.com_mass.x), npx[k]);
                dy[k] = add2(dup2(nd.com_mass.y), npy[k]);
                dz[k] = add2(dup2(nd.com_mass.z), npz[k]);
                d2[k] = fma2(dz[k], dz[k], fma2(dy[k], dy[k], mul2(dx[k], dx[k])));
                const float2 td2 = mul2(t2, d2[k]);
                open = open | (nd.size2 >= td2.x) | (nd.size2 >= td2.y);
                if (DIR)
                    open = open | toward_body(pc, -npx[k].x, -npy[k].x, -npz[k].x) |
                           toward_body(pc, -npx[k].y, -npy[k].y, -npz[k].y);
            }
            if (__any_sync(0xffffffffu, open)) {
                if (nd.kids >= 0) {  // internal: its children's group, later
                    const int nk = __shfl_sync(0xffffffffu, mynk, c);
                    if (NB_IN_RANGE(sp, kGroupStack) && sp < kGroupStack) {
                        if (lane == 0) s_stack[w][sp] = make_int2(nd.kids, nk);
                        ++sp;
                    }
                    continue;
                }
                const int e = NB_IN_RANGE(nd.first, n) && NB_IN_RANGE(nd.first + nd.count - 1, n)
                                  ? nd.first + nd.count
                                  : nd.first;
#pragma unroll 2
                for (int b = nd.first; b < e; ++b) {
                    const float4 q = body[b];
#pragma unroll
                    for (int k = 0; k < NP; ++k) {
                        const float2 rx = add2(dup2(q.x), npx[k]);
                        const float2 ry = add2(dup2(q.y), npy[k]);
                        const float2 rz = add2(dup2(q.z), npz[k]);
                        const float2 r2 = fma2(rz, rz, fma2(ry, ry, fma2(rx, rx, e2)));
                        float2 inv = make_float2(rsqrt_mufu(r2.x), rsqrt_mufu(r2.y));
                        if (ZERO_SOFT) {
                            inv.x = r2.x > 0.f ? inv.x : 0.f;
                            inv.y = r2.y > 0.f ? inv.y : 0.f;
                        }
                        const float2 s = mul2(mul2(dup2(q.w), inv), mul2(inv, inv));
                        fx[k] = fma2(rx, s, fx[k]);
                        fy[k] = fma2(ry, s, fy[k]);
                        fz[k] = fma2(rz, s, fz[k]);
                    }
                }
                p2p += nd.count;
            } else {
                float4 q0, q1;
                if (QUAD) {
                    q0 = s_quad[w][2 * c];
                    q1 = s_quad[w][2 * c + 1];
                }
#pragma unroll
                for (int k = 0; k < NP; ++k) {
                    const float2 r2 = add2(d2[k], e2);
                    const float2 inv = make_float2(rsqrt_mufu(r2.x), rsqrt_mufu(r2.y));
                    const float2 inv2 = mul2(inv, inv);
                    const float2 s = mul2(mul2(dup2(nd.com_mass.w), inv), inv2);
                    fx[k] = fma2(dx[k], s, fx[k]);
                    fy[k] = fma2(dy[k], s, fy[k]);
                    fz[k] = fma2(dz[k], s, fz[k]);
                    if (QUAD) {
                        const float2 qx = fma2(dup2(q0.x), dx[k],
                                               fma2(dup2(q0.w), dy[k], mul2(dup2(q1.x), dz[k])));
                        const float2 qy = fma2(dup2(q0.w), dx[k],
                                               fma2(dup2(q0.y), dy[k], mul2(dup2(q1.y), dz[k])));
                        const float2 qz = fma2(dup2(q1.x), dx[k],
                                               fma2(dup2(q1.y), dy[k], mul2(dup2(q0.z), dz[k])));
                        const float2 rqr = fma2(dx[k], qx, fma2(dy[k], qy, mul2(dz[k], qz)));
                        const float2 inv5 = mul2(mul2(inv, inv2), inv2);
                        const float2 f = mul2(mul2(dup2(2.5f), rqr), inv2);
                        fx[k] = fma2(inv5, fma2(f, dx[k], make_float2(-qx.x, -qx.y)), fx[k]);
                        fy[k] = fma2(inv5, fma2(f, dy[k], make_float2(-qy.x, -qy.y)), fy[k]);
                        fz[k] = fma2(inv5, fma2(f, dz[k], make_float2(-qz.x, -qz.y)), fz[k]);
                    }
                }
                ++m2p;
            }
        }
    }
    unsigned nv = 0;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        if (va[k]) {
            const uint32_t o = order[ia[k]];
            ax[o] = G * (double)fx[k].x;
            ay[o] = G * (double)fy[k].x;
            az[o] = G * (double)fz[k].x;
        }
        if (vb[k]) {
            const uint32_t o = order[ib[k]];
            ax[o] = G * (double)fx[k].y;
            ay[o] = G * (double)fy[k].y;
            az[o] = G * (double)fz[k].y;
        }
        nv += __popc(__ballot_sync(0xffffffffu, va[k])) + __popc(__ballot_sync(0xffffffffu, vb[k]));
    }
    if (lane == 0) {
        atomicAdd(&stats->m2p, (unsigned long long)m2p * nv);
        atomicAdd(&stats->p2p, (unsigned long long)p2p * nv);
        atomicAdd(&stats->total, (unsigned long long)(m2p + p2p) * nv);
    }
}

int div_up(long a, long b) { return (int)((a + b - 1) / b); }

template <class T>
nb_status scan_exclusive(const T *in, int n, T *out, DevBuf &tmp, cudaStream_t st)
{
    const int nb = div_up(n, scan_tile<T>());
    NB_TRY(tmp.reserve(sizeof(T) * (size_t)std::max(nb, 1)));
    T *sums = tmp.as<T>();
    scan_reduce_kernel<T><<<nb, 256, 0, st>>>(in, n, sums);
    NB_LAUNCH_CHECK();
    scan_top_kernel<T><<<1, std::min(1024, 32 * div_up(nb, 32)), 0, st>>>(sums, nb);
    NB_LAUNCH_CHECK();
    scan_apply_kernel<T><<<nb, 256, 0, st>>>(in, n, sums, out);
    NB_LAUNCH_CHECK();
    return NB_OK;
}

} // namespace

struct BHTree {
    int n = 0;
    int num_nodes = -1;         // host copy of the node count (-1: not read back yet)
    int node_cap = 0;           // node slots reserved (an upper bound of the count)
    int *h_total = nullptr;     // pinned host copy of the count, filled asynchronously
    cudaEvent_t total_ready = nullptr;
    DevBuf part, root, keys0, keys1, vals0, vals1, hist, body, moments, prefix, chain_len,
        chain_depth, offsets, scan_tmp, nodes, node_depth, boxes, stats, moments2a, moments2b,
        prefix2a, prefix2b, quad, pcen, pstart, parent, octant, occ, kidflag, kbase, gnodes, gnk,
        gpcen, gquad;
    bool with_quad = false;     // the nodes carry quadrupoles (quad, 2 float4 per node)
    bool ref_open = false;      // the reference's opening rule (the child toward the body too)
    bool pcen_valid = false;    // pcen holds the parent centres of the current topology
    const uint64_t *sorted_codes = nullptr;
    const uint32_t *order = nullptr;
    bool tree_valid = false;    // nodes/order describe a build of these bodies' count
    int evals_since_build = 0;  // walks on the current topology
};

void bh_invalidate(BHTree *t)
{
    if (t) t->tree_valid = false;
}

void bh_mark_count_stale(BHTree *t)
{
    if (t) t->num_nodes = -1;
}

BHTree *bh_create() { return new BHTree(); }

void bh_destroy(BHTree *t)
{
    if (!t) return;
    DevBuf *bufs[] = {&t->part, &t->root, &t->keys0, &t->keys1, &t->vals0, &t->vals1,
                      &t->hist, &t->body, &t->moments, &t->prefix, &t->chain_len,
                      &t->chain_depth, &t->offsets, &t->scan_tmp, &t->nodes, &t->node_depth,
                      &t->boxes, &t->stats, &t->moments2a, &t->moments2b, &t->prefix2a,
                      &t->prefix2b, &t->quad, &t->pcen, &t->pstart, &t->parent, &t->octant,
                      &t->occ, &t->kidflag, &t->kbase, &t->gnodes,
                      &t->gnk, &t->gpcen, &t->gquad};
    for (DevBuf *b : bufs) b->release();
    if (t->h_total) cudaFreeHost(t->h_total);
    if (t->total_ready) cudaEventDestroy(t->total_ready);
    delete t;
}

// The device copy of the node count of the last build (scan total).
static const int *d_total(const BHTree *t) { return t->offsets.as<int>() + t->n; }

// Nodes to launch over: the count if it has been read back, else the bound.
static int launch_nodes(const BHTree *t) { return t->num_nodes >= 0 ? t->num_nodes : t->node_cap; }

// The node count on the host (waits for its asynchronous read-back).
static nb_status known_nodes(BHTree *t, int *count)
{
    if (t->num_nodes < 0) {
        NB_CUDA_TRY(cudaEventSynchronize(t->total_ready));
        t->num_nodes = *t->h_total;
    }
    *count = t->num_nodes;
    return NB_OK;
}

// An upper bound of the node count of n bodies: the cells of one depth that
// split are disjoint and hold more than leaf_capacity bodies each (and there
// are at most 8^d of them); every leaf holds a body.
static size_t node_bound(int n, int leaf_capacity)
{
    const size_t per_level = (size_t)n / (size_t)(std::max(leaf_capacity, 0) + 1);
    size_t total = (size_t)n, cells = 1;
    for (int d = 0; d < kMaxLevels; ++d) {
        total += std::min(cells, per_level);
        cells = std::min(cells * 8, (size_t)1 << 40);
    }
    return total;
}

// Root cube, 63-bit codes and the stable LSD sort of the code bits
// [first_shift, 64) (first_shift 0: the full code).  Leaves the sorted codes
// and the permutation (sorted index -> original index) in t.
// Key/value ping-pong buffers and digit histograms for n entries.
static nb_status reserve_sort(BHTree *t, int n)
{
    const size_t N = (size_t)n;
    const int num_tiles = div_up(n, kSortTile);
    NB_TRY(t->keys0.reserve(sizeof(uint64_t) * N));
    NB_TRY(t->keys1.reserve(sizeof(uint64_t) * N));
    NB_TRY(t->vals0.reserve(sizeof(uint32_t) * N));
    NB_TRY(t->vals1.reserve(sizeof(uint32_t) * N));
    // three rotating digit-count buffers per tile, then their exclusive scan
    // (256 * tiles + 1 each)
    NB_TRY(t->hist.reserve(sizeof(int) * 4 * (256 * (size_t)num_tiles + 1)));
    return NB_OK;
}

// Stable LSD radix sort of (keys0, vals0) by the key bits [first_shift, 64),
// 8 bits per pass; leaves the sorted keys and values in t.
static nb_status radix_passes(BHTree *t, int n, int first_shift, cudaStream_t st)
{
    const int num_tiles = div_up(n, kSortTile);
    uint64_t *kin = t->keys0.as<uint64_t>(), *kout = t->keys1.as<uint64_t>();
    uint32_t *vin = t->vals0.as<uint32_t>(), *vout = t->vals1.as<uint32_t>();
    // pass p reads counts cnt[p % 3], counts the next digit into cnt[(p + 1) % 3]
    // and clears cnt[(p + 2) % 3] (read by pass p - 1) for pass p + 1
    const size_t stride = 256 * (size_t)num_tiles + 1;
    int *cnt[3] = {t->hist.as<int>(), t->hist.as<int>() + stride, t->hist.as<int>() + 2 * stride};
    int *digit_off = t->hist.as<int>() + 3 * stride;
    const bool direct = num_tiles <= kSortDirectTiles;  // offsets from the counts
    const bool fused = num_tiles <= kSortFusedTiles;    // next histogram in the scatter
    if (fused) NB_CUDA_TRY(cudaMemsetAsync(cnt[1], 0, sizeof(int) * 256 * (size_t)num_tiles, st));
    int p = 0;
    for (int shift = first_shift; shift < 64; shift += 8, ++p) {
        const bool last = shift + 8 >= 64;
        int *cur = fused ? cnt[p % 3] : cnt[0];
        if (!fused || p == 0) {
            radix_hist_kernel<<<num_tiles, 256, 0, st>>>(kin, n, shift, cur, num_tiles);
            NB_LAUNCH_CHECK();
        }
        if (!direct) NB_TRY(scan_exclusive<int>(cur, 256 * num_tiles, digit_off, t->scan_tmp, st));
        const bool next = fused && !last;
        radix_scatter_kernel<<<num_tiles, 256, 0, st>>>(
            kin, vin, kout, vout, n, shift, direct ? nullptr : digit_off, cur,
            next ? cnt[(p + 1) % 3] : nullptr, next ? cnt[(p + 2) % 3] : nullptr, num_tiles);
        NB_LAUNCH_CHECK();
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    t->sorted_codes = kin;
    t->order = vin;
    return NB_OK;
}

// Root cube, 63-bit codes and the stable LSD sort of the code bits
// [first_shift, 64) (first_shift 0: the full code).  Leaves the sorted codes
// and the permutation (sorted index -> original index) in t.
static nb_status morton_sort(BHTree *t, const double *x, const double *y, const double *z,
                             int n, int first_shift, cudaStream_t st, bool hilbert = false)
{
    const int nparts = std::min(div_up(n, 1024), 4 * device_props().num_sms);
    NB_TRY(t->part.reserve(sizeof(double) * 6 * nparts));
    NB_TRY(t->root.reserve(sizeof(BHRoot)));
    NB_TRY(reserve_sort(t, n));
    BHRoot *root = t->root.as<BHRoot>();

    bbox_partial_kernel<<<nparts, 256, 0, st>>>(x, y, z, n, t->part.as<double>());
    NB_LAUNCH_CHECK();
    bbox_final_kernel<<<1, 256, 0, st>>>(t->part.as<double>(), nparts, root);
    NB_LAUNCH_CHECK();
    if (hilbert)
        hilbert_kernel<<<div_up(n, 256), 256, 0, st>>>(x, y, z, n, root, t->keys0.as<uint64_t>(),
                                                        t->vals0.as<uint32_t>());
    else
        encode_kernel<<<div_up(n, 256), 256, 0, st>>>(x, y, z, n, root,
                                                       t->keys0.as<uint64_t>(),
                                                       t->vals0.as<uint32_t>());
    NB_LAUNCH_CHECK();
    return radix_passes(t, n, first_shift, st);
}

nb_status bh_sort_buffers(BHTree *t, int n, uint64_t **keys, uint32_t **vals)
{
    NB_TRY(reserve_sort(t, std::max(n, 1)));
    *keys = t->keys0.as<uint64_t>();
    *vals = t->vals0.as<uint32_t>();
    return NB_OK;
}

nb_status bh_sort_keys(BHTree *t, int n, int first_shift, cudaStream_t st,
                       const uint32_t **order)
{
    if (n > 0) NB_TRY(radix_passes(t, n, first_shift, st));
    *order = t->order;
    t->tree_valid = false;
    return NB_OK;
}

nb_status bh_morton_order(BHTree *t, const double *x, const double *y, const double *z, int n,
                          int levels, cudaStream_t st, const uint32_t **order,
                          const double **root_centre)
{
    if (n <= 0) return NB_OK;
    levels = std::max(1, std::min(levels, kMaxLevels));
    // LSD passes over the top 3*levels bits: start at the lowest of them,
    // rounded down to a digit boundary.
    const int first_shift = std::max(0, (63 - 3 * levels) / 8 * 8);
    NB_TRY(morton_sort(t, x, y, z, n, first_shift, st));
    *order = t->order;
    *root_centre = &t->root.as<BHRoot>()->cx;
    t->tree_valid = false;  // the sort replaced the tree's codes
    return NB_OK;
}

nb_status bh_hilbert_order(BHTree *t, const double *x, const double *y, const double *z, int n,
                           cudaStream_t st, const uint32_t **order, const double **root_centre)
{
    if (n <= 0) return NB_OK;
    NB_TRY(morton_sort(t, x, y, z, n, 32, st, true));  // key bits 32..63
    *order = t->order;
    *root_centre = &t->root.as<BHRoot>()->cx;
    t->tree_valid = false;
    return NB_OK;
}

// Packed body pairs per lane of the walk (0: the one-body-per-lane walk);
// NB_BH_WALK_PAIRS overrides the default.
int walk_pairs()
{
    static const int np = [] {
        const char *e = std::getenv("NB_BH_WALK_PAIRS");
        const int v = e ? std::atoi(e) : 1;
        return v < 0 ? 0 : (v > 2 ? 2 : v);
    }();
    return np;
}

// The walk over child groups (default) or the stackless preorder walk
// (NB_BH_WALK=preorder, read at every walk; both find the same interactions).
bool group_walk()
{
    const char *e = std::getenv("NB_BH_WALK");
    return !(e && std::strcmp(e, "preorder") == 0);
}

template <bool ZS, bool Q, bool D>
void walk_launch(BHTree *t, int n, float theta2, float eps2, double G, double *ax, double *ay,
                 double *az, cudaStream_t st)
{
    const int np = walk_pairs();
    const float4 *pc = t->pcen.as<float4>();
    if (group_walk() && np >= 1) {
        const BHGNode *gn = t->gnodes.as<BHGNode>();
        const unsigned char *gk = t->gnk.as<unsigned char>();
        const float4 *gq = t->gquad.as<float4>(), *gp = t->gpcen.as<float4>();
        if (np == 2)
            group_walk_kernel<ZS, Q, 2, D><<<div_up(n, 4 * kGroupBlock), kGroupBlock, 0, st>>>(
                gn, gk, d_total(t), t->body.as<float4>(), t->order, n, theta2, eps2, G, ax, ay,
                az, t->stats.as<BHStats>(), gq, gp);
        else
            group_walk_kernel<ZS, Q, 1, D><<<div_up(n, 2 * kGroupBlock), kGroupBlock, 0, st>>>(
                gn, gk, d_total(t), t->body.as<float4>(), t->order, n, theta2, eps2, G, ax, ay,
                az, t->stats.as<BHStats>(), gq, gp);
    } else if (np == 2)
        walk2_kernel<ZS, Q, 2, D><<<div_up(n, 4 * kWalkBlock), kWalkBlock, 0, st>>>(
            t->nodes.as<BHNode>(), d_total(t), t->body.as<float4>(), t->order, n, theta2,
            eps2, G, ax, ay, az, t->stats.as<BHStats>(), t->quad.as<float4>(), pc);
    else if (np == 1)
        walk2_kernel<ZS, Q, 1, D><<<div_up(n, 2 * kWalkBlock), kWalkBlock, 0, st>>>(
            t->nodes.as<BHNode>(), d_total(t), t->body.as<float4>(), t->order, n, theta2,
            eps2, G, ax, ay, az, t->stats.as<BHStats>(), t->quad.as<float4>(), pc);
    else
        walk_kernel<ZS, Q, D><<<div_up(n, kWalkBlock), kWalkBlock, 0, st>>>(
            t->nodes.as<BHNode>(), d_total(t), t->body.as<float4>(), t->order, n, theta2,
            eps2, G, ax, ay, az, t->stats.as<BHStats>(), t->quad.as<float4>(), pc);
}

template <bool ZS, bool Q>
void walk_launch_rule(BHTree *t, int n, float theta2, float eps2, double G, double *ax,
                      double *ay, double *az, cudaStream_t st)
{
    if (t->ref_open) walk_launch<ZS, Q, true>(t, n, theta2, eps2, G, ax, ay, az, st);
    else walk_launch<ZS, Q, false>(t, n, theta2, eps2, G, ax, ay, az, st);
}

static nb_status launch_walk(BHTree *t, int n, double G, double eps2, double theta, double *ax,
                             double *ay, double *az, cudaStream_t st, const KernelTimer *timer)
{
    NvtxRange range("bh_walk");
    const float th2 = (float)(theta * theta), e2 = (float)eps2;
    if (timer && timer->start) NB_CUDA_TRY(cudaEventRecord(timer->start, st));
    if (t->with_quad) {
        if (eps2 > 0.0) walk_launch_rule<false, true>(t, n, th2, e2, G, ax, ay, az, st);
        else walk_launch_rule<true, true>(t, n, th2, 0.0f, G, ax, ay, az, st);
    } else {
        if (eps2 > 0.0) walk_launch_rule<false, false>(t, n, th2, e2, G, ax, ay, az, st);
        else walk_launch_rule<true, false>(t, n, th2, 0.0f, G, ax, ay, az, st);
    }
    NB_LAUNCH_CHECK();
    if (timer && timer->stop) NB_CUDA_TRY(cudaEventRecord(timer->stop, st));
    return NB_OK;
}

// Quadrupoles of every node of the current tree (after its monopole pass).
static nb_status compute_quads(BHTree *t, const double *x, const double *y, const double *z,
                               const double *m, int n, cudaStream_t st)
{
    const size_t N = (size_t)n;
    const int nn = launch_nodes(t);
    NB_TRY(t->moments2a.reserve(sizeof(D4) * N));
    NB_TRY(t->moments2b.reserve(sizeof(D4) * N));
    NB_TRY(t->prefix2a.reserve(sizeof(D4) * (N + 1)));
    NB_TRY(t->prefix2b.reserve(sizeof(D4) * (N + 1)));
    NB_TRY(t->quad.reserve(sizeof(float4) * 2 * (size_t)nn));
    gather2_kernel<<<div_up(n, 256), 256, 0, st>>>(t->order, x, y, z, m, n,
                                                   t->root.as<BHRoot>(), t->moments2a.as<D4>(),
                                                   t->moments2b.as<D4>());
    NB_LAUNCH_CHECK();
    NB_TRY(scan_exclusive<D4>(t->moments2a.as<D4>(), n, t->prefix2a.as<D4>(), t->scan_tmp, st));
    NB_TRY(scan_exclusive<D4>(t->moments2b.as<D4>(), n, t->prefix2b.as<D4>(), t->scan_tmp, st));
    quad_kernel<<<div_up(nn, 256), 256, 0, st>>>(t->nodes.as<BHNode>(), d_total(t), t->prefix.as<D4>(),
                                                 t->prefix2a.as<D4>(), t->prefix2b.as<D4>(),
                                                 t->quad.as<float4>());
    NB_LAUNCH_CHECK();
    return NB_OK;
}

// The parent centres the reference's opening rule needs, once per topology.
static nb_status ensure_pcen(BHTree *t, cudaStream_t st)
{
    if (!t->ref_open || t->pcen_valid) return NB_OK;
    const int slots = launch_nodes(t);
    NB_TRY(t->pcen.reserve(sizeof(float4) * (size_t)slots));
    const int grid = std::max(1, std::min(div_up(slots, 256), 8 * device_props().num_sms));
    pcen_kernel<<<grid, 256, 0, st>>>(t->sorted_codes, t->nodes.as<BHNode>(),
                                      t->node_depth.as<unsigned char>(), d_total(t),
                                      t->root.as<BHRoot>(), t->pcen.as<float4>());
    NB_LAUNCH_CHECK();
    t->pcen_valid = true;
    return NB_OK;
}

// The child-group records of the current tree (after its monopoles, sides
// and quadrupoles); recount: a new topology (children counts and group
// places), else only the records are rewritten.
static nb_status group_nodes(BHTree *t, cudaStream_t st, bool recount)
{
    const int slots = launch_nodes(t);
    const int grid = std::max(1, std::min(div_up(slots, 256), 8 * device_props().num_sms));
    if (recount) {
        NB_TRY(t->kbase.reserve(sizeof(int) * ((size_t)slots + 1)));
        int *next = t->kbase.as<int>() + slots;  // the group counter (group 0: the root)
        NB_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(int), st));
        alloc_groups_kernel<<<grid, 256, 0, st>>>(t->kidflag.as<unsigned char>(), d_total(t),
                                                  t->occ.as<unsigned>(), t->kbase.as<int>(), next);
        NB_LAUNCH_CHECK();
    }
    NB_TRY(t->gnodes.reserve(sizeof(BHGNode) * (size_t)slots));
    NB_TRY(t->gnk.reserve((size_t)slots));
    if (t->ref_open) NB_TRY(t->gpcen.reserve(sizeof(float4) * (size_t)slots));
    if (t->with_quad) NB_TRY(t->gquad.reserve(sizeof(float4) * 2 * (size_t)slots));
    group_kernel<<<grid, 256, 0, st>>>(
        t->nodes.as<BHNode>(), d_total(t), t->occ.as<unsigned>(), t->kbase.as<int>(),
        t->parent.as<int>(), t->octant.as<unsigned char>(),
        t->ref_open ? t->pcen.as<float4>() : nullptr,
        t->with_quad ? t->quad.as<float4>() : nullptr, t->gnodes.as<BHGNode>(),
        t->gnk.as<unsigned char>(), t->gpcen.as<float4>(),
        t->with_quad ? t->gquad.as<float4>() : nullptr);
    NB_LAUNCH_CHECK();
    return NB_OK;
}

// Monopoles and cell sides of the kept topology for the current positions.
static nb_status refit(BHTree *t, const double *x, const double *y, const double *z,
                       const double *m, int n, cudaStream_t st)
{
    const BHRoot *root = t->root.as<BHRoot>();
    int nn = 0;
    NB_TRY(known_nodes(t, &nn));  // read back during an earlier evaluation
    NB_TRY(t->boxes.reserve(sizeof(float4) * 2 * (size_t)nn));
    gather_kernel<<<div_up(n, 256), 256, 0, st>>>(t->order, x, y, z, m, n, root,
                                                  t->body.as<float4>(), t->moments.as<D4>());
    NB_LAUNCH_CHECK();
    NB_TRY(scan_exclusive<D4>(t->moments.as<D4>(), n, t->prefix.as<D4>(), t->scan_tmp, st));
    refit_kernel<<<div_up(nn, 256), 256, 0, st>>>(t->nodes.as<BHNode>(), d_total(t),
                                                  t->node_depth.as<unsigned char>(),
                                                  t->prefix.as<D4>(), root, t->body.as<float4>(),
                                                  t->boxes.as<float4>());
    NB_LAUNCH_CHECK();
    // internal nodes, deepest first (an internal node is shallower than the
    // deepest possible level)
    for (int d = kMaxLevels - 1; d >= 0; --d) {
        refit_level_kernel<<<div_up(nn, 256), 256, 0, st>>>(
            t->nodes.as<BHNode>(), d_total(t), t->node_depth.as<unsigned char>(), d, root,
            t->boxes.as<float4>());
        NB_LAUNCH_CHECK();
    }
    // this walk's interaction counts (the tree's leaf and depth figures stay)
    NB_CUDA_TRY(cudaMemsetAsync(t->stats.ptr, 0, 2 * sizeof(unsigned long long), st));
    return NB_OK;
}

nb_status bh_compute(BHTree *t, const double *x, const double *y, const double *z,
                     const double *m, int n, double G, double eps2, double theta,
                     int leaf_capacity, double *ax, double *ay, double *az, cudaStream_t st,
                     const KernelTimer *timer, int reuse, bool quad, bool ref_open)
{
    if (n <= 0) return NB_OK;
    t->with_quad = quad;
    t->ref_open = ref_open;
    if (ax && reuse > 1 && t->tree_valid && t->n == n && t->evals_since_build < reuse) {
        NB_TRY(refit(t, x, y, z, m, n, st));
        if (quad) NB_TRY(compute_quads(t, x, y, z, m, n, st));
        NB_TRY(ensure_pcen(t, st));
        NB_TRY(group_nodes(t, st, false));
        ++t->evals_since_build;
        return launch_walk(t, n, G, eps2, theta, ax, ay, az, st, timer);
    }
    t->tree_valid = false;
    NvtxRange range("bh_build");
    const size_t N = (size_t)n;
    NB_TRY(t->body.reserve(sizeof(float4) * N));
    NB_TRY(t->moments.reserve(sizeof(D4) * N));
    NB_TRY(t->prefix.reserve(sizeof(D4) * (N + 1)));
    NB_TRY(t->chain_len.reserve(sizeof(int) * N));
    NB_TRY(t->chain_depth.reserve(sizeof(int) * N));
    NB_TRY(t->offsets.reserve(sizeof(int) * (N + 1)));
    NB_TRY(t->pstart.reserve(sizeof(int) * N));
    if (!t->stats.ptr) {
        NB_TRY(t->stats.reserve(sizeof(BHStats)));
        NB_CUDA_TRY(cudaMemsetAsync(t->stats.ptr, 0, sizeof(BHStats), st));
    }
    NB_TRY(morton_sort(t, x, y, z, n, 0, st));
    BHRoot *root = t->root.as<BHRoot>();
    BHStats *stats = t->stats.as<BHStats>();
    uint64_t *kin = const_cast<uint64_t *>(t->sorted_codes);
    uint32_t *vin = const_cast<uint32_t *>(t->order);

    gather_kernel<<<div_up(n, 256), 256, 0, st>>>(vin, x, y, z, m, n, root,
                                                  t->body.as<float4>(), t->moments.as<D4>());
    NB_LAUNCH_CHECK();
    NB_TRY(scan_exclusive<D4>(t->moments.as<D4>(), n, t->prefix.as<D4>(), t->scan_tmp, st));
    chain_kernel<<<div_up(n, 256), 256, 0, st>>>(kin, n, leaf_capacity, root,
                                                 t->chain_len.as<int>(),
                                                 t->chain_depth.as<int>(), t->pstart.as<int>());
    NB_LAUNCH_CHECK();
    NB_TRY(scan_exclusive<int>(t->chain_len.as<int>(), n, t->offsets.as<int>(), t->scan_tmp,
                               st));
    // No host read of the node count before the walk: node storage is sized
    // for the bound, the kernels read the count on the device, and the count
    // comes back to the host asynchronously for later launches and queries.
    const size_t cap = node_bound(n, leaf_capacity);
    NB_TRY(t->nodes.reserve(sizeof(BHNode) * cap));
    NB_TRY(t->node_depth.reserve(cap));
    NB_TRY(t->parent.reserve(sizeof(int) * cap));
    NB_TRY(t->octant.reserve(cap));
    NB_TRY(t->occ.reserve(sizeof(unsigned) * cap));
    NB_TRY(t->kidflag.reserve(8 * cap));
    if (!t->h_total) NB_CUDA_TRY(cudaMallocHost(&t->h_total, sizeof(int)));
    if (!t->total_ready) NB_CUDA_TRY(cudaEventCreateWithFlags(&t->total_ready,
                                                              cudaEventDisableTiming));
    NB_CUDA_TRY(cudaMemcpyAsync(t->h_total, t->offsets.as<int>() + n, sizeof(int),
                                cudaMemcpyDeviceToHost, st));
    // inside a captured step graph the record must be an external event node
    // (recorded by every replay) for the host to be able to wait for the count
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    NB_CUDA_TRY(cudaStreamIsCapturing(st, &capturing));
    if (capturing == cudaStreamCaptureStatusActive)
        NB_CUDA_TRY(cudaEventRecordWithFlags(t->total_ready, st, cudaEventRecordExternal));
    else
        NB_CUDA_TRY(cudaEventRecord(t->total_ready, st));
    t->node_cap = (int)std::min(cap, (size_t)INT32_MAX);
    t->num_nodes = -1;
    t->n = n;
    NB_CUDA_TRY(cudaMemsetAsync(stats, 0, offsetof(BHStats, total), st));
    NB_CUDA_TRY(cudaMemsetAsync(t->kidflag.ptr, 0, 8 * cap, st));
    node_kernel<<<div_up(n, 256), 256, 0, st>>>(kin, n, leaf_capacity, root,
                                                t->chain_len.as<int>(), t->chain_depth.as<int>(),
                                                t->offsets.as<int>(), t->prefix.as<D4>(),
                                                t->nodes.as<BHNode>(),
                                                t->node_depth.as<unsigned char>(),
                                                t->pstart.as<int>(), t->parent.as<int>(),
                                                t->octant.as<unsigned char>(),
                                                t->kidflag.as<unsigned char>(), stats,
                                                t->node_cap);
    NB_LAUNCH_CHECK();
    if (quad) NB_TRY(compute_quads(t, x, y, z, m, n, st));
    t->pcen_valid = false;
    NB_TRY(ensure_pcen(t, st));
    NB_TRY(group_nodes(t, st, true));
    t->tree_valid = true;
    t->evals_since_build = 0;
    if (!ax) return NB_OK;
    t->evals_since_build = 1;
    return launch_walk(t, n, G, eps2, theta, ax, ay, az, st, timer);
}

nb_status bh_info(BHTree *t, cudaStream_t st, nb_bh_info *info)
{
    if (!t->n) return fail(NB_ERR_NOT_LOADED, "no Barnes-Hut tree built");
    BHRoot r;
    BHStats s;
    NB_CUDA_TRY(cudaMemcpyAsync(&r, t->root.ptr, sizeof(r), cudaMemcpyDeviceToHost, st));
    NB_CUDA_TRY(cudaMemcpyAsync(&s, t->stats.ptr, sizeof(s), cudaMemcpyDeviceToHost, st));
    NB_CUDA_TRY(cudaStreamSynchronize(st));
    int nn = 0;
    NB_TRY(known_nodes(t, &nn));
    info->num_nodes = nn;
    info->num_leaves = s.leaves;
    info->max_depth = s.max_depth;
    info->split_levels = r.levels;
    info->root[0] = r.cx;
    info->root[1] = r.cy;
    info->root[2] = r.cz;
    info->root[3] = r.size;
    info->interactions_m2p = s.m2p;
    info->interactions_p2p = s.p2p;
    info->interactions_total = s.total;
    return NB_OK;
}

nb_status bh_read_order(BHTree *t, cudaStream_t st, uint64_t *codes, uint32_t *order)
{
    if (!t->n) return fail(NB_ERR_NOT_LOADED, "no Barnes-Hut tree built");
    if (codes)
        NB_CUDA_TRY(cudaMemcpyAsync(codes, t->sorted_codes, sizeof(uint64_t) * t->n,
                                    cudaMemcpyDeviceToHost, st));
    if (order)
        NB_CUDA_TRY(cudaMemcpyAsync(order, t->order, sizeof(uint32_t) * t->n,
                                    cudaMemcpyDeviceToHost, st));
    NB_CUDA_TRY(cudaStreamSynchronize(st));
    return NB_OK;
}

nb_status bh_read_nodes(BHTree *t, cudaStream_t st, int max_nodes, int *depth,
                        uint64_t *prefix, int *first, int *count, int *is_leaf, int *skip,
                        float *com_mass)
{
    if (!t->n) return fail(NB_ERR_NOT_LOADED, "no Barnes-Hut tree built");
    int nn = 0;
    NB_TRY(known_nodes(t, &nn));
    if (max_nodes < nn) return fail(NB_ERR_CAPACITY, "max_nodes is smaller than the node count");
    std::vector<BHNode> h(nn);
    std::vector<unsigned char> dep(nn);
    std::vector<uint64_t> codes(t->n);
    BHRoot r;
    NB_CUDA_TRY(cudaMemcpyAsync(h.data(), t->nodes.ptr, sizeof(BHNode) * h.size(),
                                cudaMemcpyDeviceToHost, st));
    NB_CUDA_TRY(cudaMemcpyAsync(dep.data(), t->node_depth.ptr, dep.size(),
                                cudaMemcpyDeviceToHost, st));
    NB_CUDA_TRY(cudaMemcpyAsync(codes.data(), t->sorted_codes, sizeof(uint64_t) * t->n,
                                cudaMemcpyDeviceToHost, st));
    NB_CUDA_TRY(cudaMemcpyAsync(&r, t->root.ptr, sizeof(r), cudaMemcpyDeviceToHost, st));
    NB_CUDA_TRY(cudaStreamSynchronize(st));
    for (int k = 0; k < nn; ++k) {
        const BHNode &nd = h[k];
        const int d = dep[k];
        if (depth) depth[k] = d;
        if (prefix) prefix[k] = d == 0 ? 0 : codes[nd.first] >> (63 - 3 * d);
        if (first) first[k] = nd.first;
        if (count) count[k] = nd.count;
        if (is_leaf) is_leaf[k] = nd.skip == k + 1;
        if (skip) skip[k] = nd.skip;
        if (com_mass) {
            com_mass[4 * k + 0] = (float)(r.cx + (double)nd.com_mass.x);
            com_mass[4 * k + 1] = (float)(r.cy + (double)nd.com_mass.y);
            com_mass[4 * k + 2] = (float)(r.cz + (double)nd.com_mass.z);
            com_mass[4 * k + 3] = nd.com_mass.w;
        }
    }
    return NB_OK;
}

} // namespace nb
