// nb_internal.h -- internal declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "../../include/nbody_c.h"

namespace nb {

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
nb_status fail(nb_status s, const std::string &msg);
nb_status cuda_fail(cudaError_t e, const char *what);

#define NB_CUDA_TRY(call)                                                  \
    do {                                                                   \
        cudaError_t nb_e_ = (call);                                        \
        if (nb_e_ != cudaSuccess) return ::nb::cuda_fail(nb_e_, #call);    \
    } while (0)

// Counts one kernel launch of this library and checks the launch status.
void count_launch();
#define NB_LAUNCH_CHECK()                                                  \
    do {                                                                   \
        ::nb::count_launch();                                              \
        cudaError_t nb_e_ = cudaGetLastError();                            \
        if (nb_e_ != cudaSuccess) return ::nb::cuda_fail(nb_e_, "kernel launch"); \
    } while (0)

#define NB_TRY(call)                                                       \
    do {                                                                   \
        nb_status nb_s_ = (call);                                          \
        if (nb_s_ != NB_OK) return nb_s_;                                  \
    } while (0)

// An NVTX range over a host scope: the phases of a step (sort, build, walk,
// direct sum, serving tick) appear by name in timeline profilers and can be
// selected with ncu --nvtx --nvtx-include; a few nanoseconds when no tool is
// attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// The first failed device-side index check of a translation unit of a
// checked build (nb_check.cuh): source line, index and bound.
struct DeviceCheck {
    int failed;
    int line;
    long long index;
    long long bound;
};
using CheckReader = nb_status (*)(DeviceCheck *out, bool clear);
// Called by every checked translation unit at load time.
void register_check_reader(const char *file, CheckReader reader);

// ---------------------------------------------------------------- memory
// A device buffer that grows on demand and is freed with its owner.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    nb_status reserve(size_t want);
    void release();
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

struct DeviceProps {
    int device = 0;
    int num_sms = 0;
    int max_smem_optin = 0;
};
const DeviceProps &device_props();

// A pair of events recorded around the dominant kernel of a force evaluation
// (null members: not recorded).
struct KernelTimer {
    cudaEvent_t start = nullptr, stop = nullptr;
};

// ---------------------------------------------------------------- direct sum
struct DirectPlan {
    int block = 256;    // threads per CTA
    int ipt = 4;        // i-bodies per thread
    int segments = 1;   // j-split factor (CTAs along y)
    int seg_tiles = 1;  // j-tiles per segment
};

// Mixed FP32/double-single all-pairs kernel.  hi/lo: float4 (x, y, z, m) and
// (x_lo, y_lo, z_lo, 0) of every body.  Writes G * sum into ax/ay/az (FP64).
nb_status direct_mixed(const float4 *hi, const float4 *lo, int n, double G, double eps2,
                       double *ax, double *ay, double *az, DevBuf &partials,
                       cudaStream_t st, const KernelTimer *timer = nullptr,
                       const DirectPlan *plan_override = nullptr);
DirectPlan direct_mixed_plan(int n);
// j-split count filling whole waves of `slots` resident CTAs.
int direct_pick_segments(int iblocks, int tiles, int slots);

// Thresholds of the sorted near/far kernels as (gap / D)^2, D the diameter of
// a warp's i-box: a j-chunk at least D/8 away takes the plain FP32 term, one
// at least D/4 away also drops the Newton step (kFarFactor = 1/8, kVeryFar =
// 1/4).
constexpr float kFarFactor2 = 0.015625f;
constexpr float kVeryFar2 = 0.0625f;
// Pairs of the sorted single-system kernel closer than R = min(kExact D,
// kExactSpacing s) (s: the mean body spacing in the warp's box) leave its FP32
// sum and are evaluated in double-single: they carry the largest terms of a
// body's sum, whose FP32 rounding would otherwise set its error.
constexpr float kExact2 = 0.015625f;        // kExact = 1/8
constexpr float kExactSpacing2 = 0.5625f;   // kExactSpacing = 3/4

// Hilbert-sorted near/far variant of the mixed path (nb_direct_sorted.cu).
struct BHTree;
struct SortedBuffers {
    DevBuf hi, lo, partials, boxes;
    DevBuf exact;  // the left-out pairs' sums, 3 n doubles (sorted order)
    cudaStream_t side = nullptr;              // the exact-pair kernel's stream
    cudaEvent_t fork = nullptr, join = nullptr;
    BHTree *sorter = nullptr;
    // The sort order is a performance device only (near/far decisions use
    // the current chunk boxes, any order gives results within tolerance), so
    // it is recomputed every kResortEvals force evaluations and when n
    // changes -- not at every call, and not on a load (the next periodic
    // re-sort adapts it to bodies that moved or were replaced).
    const uint32_t *order = nullptr;  // sorted index -> body (sorter-owned)
    const double *centre = nullptr;   // origin of the hi/lo split (sorter-owned)
    int order_n = -1;
    int evals_since_sort = 0;
    void invalidate_order() { order_n = -1; }
    void release();
};
// Bodies are sorted along a Hilbert curve; every warp re-centres the j-chunks
// (32 bodies) on its own (compact) i-box and runs the plain FP32 pair term on
// those that lie at least an eighth of the box diameter away; near chunks keep
// the double-single one.
nb_status direct_mixed_sorted(const double *x, const double *y, const double *z,
                              const double *m, int n, double G, double eps2, double *ax,
                              double *ay, double *az, SortedBuffers &b, cudaStream_t st,
                              const KernelTimer *timer = nullptr);
// Whether an evaluation of n bodies takes the sorted variant: flags
// NB_FLAG_MIXED_SORTED / NB_FLAG_MIXED_UNSORTED decide, else n >= kSortedMinBodies
// (measured on GB300 per evaluation of a Plummer sphere, unsorted vs sorted:
// 12,288 bodies 0.120 vs 0.136 ms, 16,384 bodies 0.201 vs 0.194 ms).
constexpr int kSortedMinBodies = 16384;
bool direct_sorted_enabled(int n, int flags);

// FP64 all-pairs kernel.
nb_status direct_fp64(const double *x, const double *y, const double *z, const double *m,
                      int n, double G, double eps2, double *ax, double *ay, double *az,
                      DevBuf &partials, cudaStream_t st, const KernelTimer *timer = nullptr);

// Builds the float4 hi/lo mirror of FP64 positions + masses.
nb_status split_positions(const double *x, const double *y, const double *z,
                          const double *m, int n, float4 *hi, float4 *lo, cudaStream_t st);

// ---------------------------------------------------------------- integrators
nb_status kick_drift(int kind, int n, double dt, double *x, double *y, double *z, double *vx,
                     double *vy, double *vz, const double *ax, const double *ay,
                     const double *az, double *oax, double *oay, double *oaz,
                     cudaStream_t st);
nb_status kick(int kind, int n, double dt, double *vx, double *vy, double *vz,
               const double *ax, const double *ay, const double *az, const double *oax,
               const double *oay, const double *oaz, cudaStream_t st);

// RK4 stage kernels.  stage 2/3/4 positions/velocities from the base state.
nb_status rk4_stage(int n, double h, const double *x, const double *y, const double *z,
                    const double *vx, const double *vy, const double *vz, const double *kvx,
                    const double *kvy, const double *kvz, const double *kax,
                    const double *kay, const double *kaz, double *ox, double *oy,
                    double *oz, double *ovx, double *ovy, double *ovz, cudaStream_t st);
nb_status rk4_combine(int n, double dt, double *x, double *y, double *z, double *vx,
                      double *vy, double *vz, const double *ax, const double *ay,
                      const double *az, const double *k2, const double *k3, const double *k4,
                      cudaStream_t st);

// One integrator step over the ten FP64 planes f (x y z vx vy vz ax ay az m)
// of n bodies; `force` evaluates accelerations of given positions.
struct StepBuffers {
    double *old_acc = nullptr;  // 3 planes (velocity Verlet)
    double *rk4 = nullptr;      // 27 planes (RK4 stages K2, K3, K4: x v a each)
    size_t ps = 0;              // plane stride in doubles
};
using ForceFn = std::function<nb_status(const double *, const double *, const double *,
                                        double *, double *, double *)>;
nb_status integrate_step(int integ, int n, double dt, double *const f[10], StepBuffers &b,
                         bool &forces_valid, const ForceFn &force, cudaStream_t st);

// ---------------------------------------------------------------- diagnostics
// Packed-FMA lane operations per second of the current device (a register-only
// probe kernel, best of three timed launches).
nb_status fp32_rate(double *lane_ops_per_s);
nb_status diagnostics(const double *x, const double *y, const double *z, const double *vx,
                      const double *vy, const double *vz, const double *m, int n, double G,
                      double eps2, DevBuf &scratch, cudaStream_t st, nb_diag *out);

// ---------------------------------------------------------------- batches
// A system of a batch: bodies [first, first + n) of the batch's pool, summed
// with ipt i-bodies per lane.
struct SysDesc {
    int first;
    int n;
    int ipt;
    int chunk0;  // first 32-body chunk of the system (the sorted batch path)
};
// One queue item: i-bodies [i0, i0 + 32 * ipt) of system `sys`.
struct WorkItem {
    int sys;
    int i0;
};
int bucket_of(int n);  // floor(log2(n))
// Hilbert-sorted variant of the batched forces (nb_batch.cu): each system's
// bodies are sorted along a Hilbert curve through its own cube; an item is one
// or two 32-body i-chunks; j-chunks far from its box take the plain FP32 term.
struct BHTree;
struct BatchSorted {
    BHTree *sorter = nullptr;
    DevBuf body_sys, chunks, geom, boxes;
    const uint32_t *order = nullptr;  // sorted index -> body (sorter-owned)
    int num_sys = 0, num_chunks = 0, total = 0, key_shift = 0, first_shift = 0;
    void release();
};
// i-chunks per warp item of an n-body system in the sorted variant (1 or 2).
int batch_sorted_ipt(int n);
// Sets every system's ipt (batch_sorted_ipt) and chunk0; returns the chunk count.
int batch_sorted_chunks(std::vector<SysDesc> &sys);
// Device tables for the systems of d_sys (already uploaded with chunk0).
nb_status batch_sorted_setup(BatchSorted &b, const SysDesc *d_sys, int num_sys, int num_chunks,
                             int total, cudaStream_t st);
// (Re)computes the order from the positions x, y, z.
nb_status batch_sorted_sort(BatchSorted &b, const SysDesc *d_sys, const double *x,
                            const double *y, const double *z, cudaStream_t st);
// a = G sum_j ... for every body, in the order of the last sort (hi/lo are
// scratch mirrors of total entries).
nb_status batch_sorted_forces(BatchSorted &b, const double *x, const double *y, const double *z,
                              const double *m, const SysDesc *d_sys, const WorkItem *d_items,
                              int num_items, int *d_counter, double G, double eps2, float4 *hi,
                              float4 *lo, double *ax, double *ay, double *az, cudaStream_t st,
                              const KernelTimer *timer);

// Items of every system, largest cost first.
void build_work_items(const std::vector<SysDesc> &sys, std::vector<WorkItem> &items);
// Mixed-precision forces of all systems of the queue (persistent kernel).
nb_status batch_forces(const float4 *hi, const float4 *lo, const SysDesc *d_sys,
                       const WorkItem *d_items, int num_items, int *d_counter, double G,
                       double eps2, double *ax, double *ay, double *az, int total,
                       cudaStream_t st, const KernelTimer *timer = nullptr);

// ---------------------------------------------------------------- Barnes-Hut
struct BHTree;  // opaque, defined in nb_bh.cu
BHTree *bh_create();
void bh_destroy(BHTree *t);
// Builds the tree of (x,y,z,m) and, when ax != nullptr, walks it writing
// G * acceleration (FP64) in the original body order.  reuse > 1: the tree is
// rebuilt every `reuse` walks; the walks in between keep its topology and
// refit monopoles and cell sides to the current positions.  quad: accepted
// cells act with their quadrupole moments too.  ref_open: the walk also opens,
// of every node it opens, the child toward the body (the reference's rule).
nb_status bh_compute(BHTree *t, const double *x, const double *y, const double *z,
                     const double *m, int n, double G, double eps2, double theta,
                     int leaf_capacity, double *ax, double *ay, double *az, cudaStream_t st,
                     const KernelTimer *timer = nullptr, int reuse = 1, bool quad = false,
                     bool ref_open = false);
// The next bh_compute rebuilds (the bodies were replaced).
void bh_invalidate(BHTree *t);
// A replayed build changed the node count behind the host's back.
void bh_mark_count_stale(BHTree *t);
nb_status bh_info(BHTree *t, cudaStream_t st, nb_bh_info *info);
// Morton order of the bodies by the top 3*levels code bits: *order maps a
// sorted index to the original one; *root_centre points at the device copy of
// the root cube centre (3 doubles), followed by the cube's side (a 4th
// double).  Both stay valid until the next call on t.
nb_status bh_morton_order(BHTree *t, const double *x, const double *y, const double *z, int n,
                          int levels, cudaStream_t st, const uint32_t **order,
                          const double **root_centre);
// The same for the order along the Hilbert curve through the 2^10-cell grid of
// the root cube (runs of sorted bodies fill compact regions).
nb_status bh_hilbert_order(BHTree *t, const double *x, const double *y, const double *z, int n,
                           cudaStream_t st, const uint32_t **order, const double **root_centre);
// A stable sort of caller-made keys: bh_sort_buffers returns the key and
// value arrays (n entries) to fill on the device; bh_sort_keys then sorts them
// by the key bits [first_shift, 64) and returns the sorted values (valid until
// the next call on t).
nb_status bh_sort_buffers(BHTree *t, int n, uint64_t **keys, uint32_t **vals);
nb_status bh_sort_keys(BHTree *t, int n, int first_shift, cudaStream_t st,
                       const uint32_t **order);
nb_status bh_read_order(BHTree *t, cudaStream_t st, uint64_t *codes, uint32_t *order);
nb_status bh_read_nodes(BHTree *t, cudaStream_t st, int max_nodes, int *depth,
                        uint64_t *prefix, int *first, int *count, int *is_leaf, int *skip,
                        float *com_mass);

} // namespace nb

// The simulation object behind nb_sim*.
struct nb_sim {
    nb_config cfg{};
    size_t capacity = 0;
    size_t n = 0;
    cudaStream_t stream = nullptr;
    int device = 0;

    // FP64 state: x y z vx vy vz ax ay az m, each `capacity` doubles.
    nb::DevBuf state;
    double *f[10] = {};
    bool forces_valid = false;

    nb::DevBuf split_hi, split_lo;   // float4 mirrors for the mixed kernel
    nb::SortedBuffers sorted;        // Hilbert-sorted near/far variant of the mixed kernel
    nb::DevBuf partials;             // j-split partial sums
    nb::DevBuf old_acc;              // velocity-Verlet a(t)
    nb::DevBuf rk4;                  // RK4 stage states and accelerations
    nb::DevBuf diag_scratch;
    nb::BHTree *bh = nullptr;

    // One step as a CUDA graph (nb_step): captured on the second of two
    // consecutive eligible steps with the same integrator and dt, replayed
    // while they and the accelerations-valid flag stay the same; any load,
    // configuration or flag change drops it.
    cudaGraphExec_t step_graph = nullptr;
    int graph_integ = -1;
    double graph_dt = 0.0;
    bool graph_fv_before = false, graph_fv_after = false;  // forces_valid around the step
    uint64_t graph_kernels = 0;     // kernel nodes per replay (launch accounting)
    int warm_integ = -1;            // the last uncaptured eligible step
    double warm_dt = 0.0;
    bool graphs_off = false;        // a capture failed: run steps directly

    // Optional timing of the dominant force kernel (nb_profile_*).
    bool profiling = false;
    std::vector<nb::KernelTimer> timers;
    size_t timers_used = 0;

    double *x() const { return f[0]; }
    double *y() const { return f[1]; }
    double *z() const { return f[2]; }
    double *vx() const { return f[3]; }
    double *vy() const { return f[4]; }
    double *vz() const { return f[5]; }
    double *ax() const { return f[6]; }
    double *ay() const { return f[7]; }
    double *az() const { return f[8]; }
    double *m() const { return f[9]; }
};

namespace nb {
// Evaluates accelerations of positions (px,py,pz) with masses m into out*.
nb_status eval_forces(nb_sim *s, const double *px, const double *py, const double *pz,
                      double *oax, double *oay, double *oaz);
// Drops the captured step graph (the next steps run directly).
void reset_step_graph(nb_sim *s);
// Kernel launches made by a graph replay (the launch counter's evidence).
void count_launches(uint64_t k);
}
