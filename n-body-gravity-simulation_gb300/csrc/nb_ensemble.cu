// nb_ensemble.cu -- the batched ensemble behind nb_ensemble_* (include/nbody_c.h).
//
// Thousands of independent systems of uneven N advance together: the state of
// all systems is concatenated (system order) in one set of FP64 planes; the
// forces of every system come from one persistent launch over a per-system
// work queue (nb_batch.cu); the per-body integrator updates run once over the
// concatenation; the step loop is captured in a CUDA graph and replayed.
//
// By default the force launch is the Hilbert-sorted near/far variant: every
// system is sorted along a Hilbert curve through its own cube at the start of
// each nb_ensemble_step call and every kGraphChunk steps (between graph
// replays, the same points whether or not the steps are replayed), and far
// j-chunks of an i-chunk take the plain FP32 term.  NB_FLAG_MIXED_UNSORTED
// selects the all-pairs double-single kernel, whose i-bodies per lane are
// autotuned per N bucket before the first evaluation.
#include "nb_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

struct nb_ensemble {
    nb_config cfg{};
    int num_sys = 0;
    size_t total = 0;
    size_t ps = 0;  // plane stride
    std::vector<int> sizes;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool loaded = false;

    nb::DevBuf state, hi, lo, old_acc, rk4, d_sys, d_items, d_counter;
    double *f[10] = {};
    std::vector<nb::SysDesc> sys;
    int num_items = 0;
    int ipt_bucket[32];
    bool tuned = false;
    bool forces_valid = false;

    // captured step loop
    cudaGraphExec_t graph = nullptr;
    int graph_integ = -1;
    double graph_dt = 0.0;
    int graph_steps = 0;
    unsigned long long graph_launches = 0;

    bool profiling = false;
    std::vector<nb::KernelTimer> timers;
    size_t timers_used = 0;

    bool sorted = true;  // the Hilbert-sorted near/far force launch
    nb::BatchSorted sb;
    int num_chunks = 0;
};

namespace nb {
namespace {

constexpr int kGraphChunk = 25;
const int kIptCandidates[] = {1, 2, 4};

nb_status upload_items(nb_ensemble *e)
{
    std::vector<WorkItem> items;
    build_work_items(e->sys, items);
    e->num_items = (int)items.size();
    NB_TRY(e->d_sys.reserve(sizeof(SysDesc) * e->sys.size()));
    NB_TRY(e->d_items.reserve(sizeof(WorkItem) * std::max<size_t>(1, items.size())));
    NB_CUDA_TRY(cudaMemcpyAsync(e->d_sys.ptr, e->sys.data(), sizeof(SysDesc) * e->sys.size(),
                                cudaMemcpyHostToDevice, e->stream));
    if (!items.empty())
        NB_CUDA_TRY(cudaMemcpyAsync(e->d_items.ptr, items.data(),
                                    sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice,
                                    e->stream));
    // the host vectors go out of scope: wait for the copies
    NB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    return NB_OK;
}

const KernelTimer *ens_timer(nb_ensemble *e, bool capturing)
{
    if (!e->profiling || capturing) return nullptr;
    if (e->timers_used == e->timers.size()) {
        KernelTimer t;
        if (cudaEventCreate(&t.start) != cudaSuccess) return nullptr;
        if (cudaEventCreate(&t.stop) != cudaSuccess) return nullptr;
        e->timers.push_back(t);
    }
    return &e->timers[e->timers_used++];
}

nb_status ens_force(nb_ensemble *e, const double *px, const double *py, const double *pz,
                    double *ax, double *ay, double *az, bool capturing)
{
    const int n = (int)e->total;
    float4 *hi = e->hi.as<float4>(), *lo = e->lo.as<float4>();
    if (e->sorted)
        return batch_sorted_forces(e->sb, px, py, pz, e->f[9], e->d_sys.as<SysDesc>(),
                                   e->d_items.as<WorkItem>(), e->num_items,
                                   e->d_counter.as<int>(), e->cfg.G,
                                   e->cfg.softening * e->cfg.softening, hi, lo, ax, ay, az,
                                   e->stream, ens_timer(e, capturing));
    NB_TRY(split_positions(px, py, pz, e->f[9], n, hi, lo, e->stream));
    const double eps2 = e->cfg.softening * e->cfg.softening;
    return batch_forces(hi, lo, e->d_sys.as<SysDesc>(), e->d_items.as<WorkItem>(), e->num_items,
                        e->d_counter.as<int>(), e->cfg.G, eps2, ax, ay, az, n, e->stream,
                        ens_timer(e, capturing));
}

// Times each candidate ipt on the systems of each N bucket and keeps the
// fastest; then builds the full work queue.
nb_status tune(nb_ensemble *e)
{
    const double eps2 = e->cfg.softening * e->cfg.softening;
    const int n = (int)e->total;
    float4 *hi = e->hi.as<float4>(), *lo = e->lo.as<float4>();
    NB_TRY(split_positions(e->f[0], e->f[1], e->f[2], e->f[9], n, hi, lo, e->stream));
    cudaEvent_t t0, t1;
    NB_CUDA_TRY(cudaEventCreate(&t0));
    NB_CUDA_TRY(cudaEventCreate(&t1));
    std::vector<SysDesc> all = e->sys;
    for (int b = 0; b < 32; ++b) {
        std::vector<SysDesc> bs;
        for (const SysDesc &s : all)
            if (bucket_of(s.n) == b) bs.push_back(s);
        if (bs.empty()) continue;
        float best = 1e30f;
        for (int ipt : kIptCandidates) {
            for (SysDesc &s : bs) s.ipt = ipt;
            e->sys = bs;
            NB_TRY(upload_items(e));
            // warm, then two timed launches into the real acceleration planes
            NB_TRY(batch_forces(hi, lo, e->d_sys.as<SysDesc>(), e->d_items.as<WorkItem>(),
                                e->num_items, e->d_counter.as<int>(), e->cfg.G, eps2, e->f[6],
                                e->f[7], e->f[8], n, e->stream));
            NB_CUDA_TRY(cudaEventRecord(t0, e->stream));
            for (int r = 0; r < 2; ++r)
                NB_TRY(batch_forces(hi, lo, e->d_sys.as<SysDesc>(), e->d_items.as<WorkItem>(),
                                    e->num_items, e->d_counter.as<int>(), e->cfg.G, eps2,
                                    e->f[6], e->f[7], e->f[8], n, e->stream));
            NB_CUDA_TRY(cudaEventRecord(t1, e->stream));
            NB_CUDA_TRY(cudaEventSynchronize(t1));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (ms < best) {
                best = ms;
                e->ipt_bucket[b] = ipt;
            }
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    for (SysDesc &s : all) s.ipt = e->ipt_bucket[bucket_of(s.n)];
    e->sys = all;
    NB_TRY(upload_items(e));
    e->tuned = true;
    e->forces_valid = false;  // tuning overwrote the acceleration planes
    return NB_OK;
}

nb_status step_direct(nb_ensemble *e, int integ, double dt, bool capturing)
{
    StepBuffers b;
    b.old_acc = e->old_acc.as<double>();
    b.rk4 = e->rk4.as<double>();
    b.ps = e->ps;
    ForceFn force = [e, capturing](const double *px, const double *py, const double *pz,
                                   double *ax, double *ay, double *az) {
        return ens_force(e, px, py, pz, ax, ay, az, capturing);
    };
    return integrate_step(integ, (int)e->total, dt, e->f, b, e->forces_valid, force, e->stream);
}

// The sorted path's tables (its shape is fixed: one 32-body i-chunk per item).
nb_status setup_sorted(nb_ensemble *e)
{
    for (const SysDesc &sd : e->sys) e->ipt_bucket[bucket_of(sd.n)] = sd.ipt;
    NB_TRY(upload_items(e));
    NB_TRY(batch_sorted_setup(e->sb, e->d_sys.as<SysDesc>(), e->num_sys, e->num_chunks,
                              (int)e->total, e->stream));
    e->tuned = true;
    return NB_OK;
}

// Every system's order from the current positions (sorted path only).
nb_status sort_systems(nb_ensemble *e)
{
    if (!e->sorted) return NB_OK;
    return batch_sorted_sort(e->sb, e->d_sys.as<SysDesc>(), e->f[0], e->f[1], e->f[2],
                             e->stream);
}

nb_status ready(nb_ensemble *e)
{
    if (!e->loaded) return fail(NB_ERR_NOT_LOADED, "ensemble: nothing loaded");
    if (!e->tuned) NB_TRY(e->sorted ? setup_sorted(e) : tune(e));
    return NB_OK;
}

} // namespace
} // namespace nb

using namespace nb;

extern "C" {

nb_status nb_ensemble_create(const nb_config *cfg, int num_systems, const int *sizes,
                             void *stream, nb_ensemble **out)
{
    if (!out || !cfg || !sizes) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (cfg->method != NB_DIRECT_MIXED)
        return fail(NB_ERR_UNSUPPORTED, "ensemble: only NB_DIRECT_MIXED is batched");
    if (!(cfg->softening >= 0.0)) return fail(NB_ERR_INVALID_ARGUMENT, "softening must be >= 0");
    if (num_systems <= 0) return fail(NB_ERR_INVALID_ARGUMENT, "num_systems must be > 0");
    size_t total = 0;
    for (int s = 0; s < num_systems; ++s) {
        if (sizes[s] <= 0) return fail(NB_ERR_INVALID_ARGUMENT, "every system needs n > 0");
        total += (size_t)sizes[s];
    }
    if (total > (size_t)1 << 30) return fail(NB_ERR_CAPACITY, "ensemble larger than 2^30 bodies");
    nb_ensemble *e = new nb_ensemble();
    e->cfg = *cfg;
    e->num_sys = num_systems;
    e->sizes.assign(sizes, sizes + num_systems);
    e->total = total;
    e->ps = (total + 31) / 32 * 32;
    for (int b = 0; b < 32; ++b) e->ipt_bucket[b] = 1;
    if (stream) {
        e->stream = static_cast<cudaStream_t>(stream);
    } else {
        // graph capture needs a stream other than the legacy default stream
        cudaError_t err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
        if (err != cudaSuccess) {
            delete e;
            return cuda_fail(err, "cudaStreamCreate");
        }
        e->own_stream = true;
    }
    nb_status st = NB_OK;
    if (st == NB_OK) st = e->state.reserve(sizeof(double) * 10 * e->ps);
    if (st == NB_OK) st = e->hi.reserve(sizeof(float4) * e->ps);
    if (st == NB_OK) st = e->lo.reserve(sizeof(float4) * e->ps);
    if (st == NB_OK) st = e->d_counter.reserve(sizeof(int));
    if (st != NB_OK) {
        nb_ensemble_destroy(e);
        return st;
    }
    for (int k = 0; k < 10; ++k) e->f[k] = e->state.as<double>() + k * e->ps;
    size_t first = 0;
    e->sys.resize(num_systems);
    for (int s = 0; s < num_systems; ++s) {
        e->sys[s] = SysDesc{(int)first, sizes[s], 1, 0};
        first += sizes[s];
    }
    e->sorted = (cfg->flags & NB_FLAG_MIXED_UNSORTED) == 0;
    if (e->sorted) e->num_chunks = batch_sorted_chunks(e->sys);
    *out = e;
    return NB_OK;
}

nb_status nb_ensemble_destroy(nb_ensemble *e)
{
    if (!e) return NB_OK;
    cudaStreamSynchronize(e->stream);
    if (e->graph) cudaGraphExecDestroy(e->graph);
    for (auto &t : e->timers) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    nb::DevBuf *bufs[] = {&e->state, &e->hi, &e->lo, &e->old_acc, &e->rk4, &e->d_sys,
                          &e->d_items, &e->d_counter};
    for (nb::DevBuf *b : bufs) b->release();
    e->sb.release();
    if (e->own_stream) cudaStreamDestroy(e->stream);
    delete e;
    return NB_OK;
}

nb_status nb_ensemble_load(nb_ensemble *e, const double *x, const double *y, const double *z,
                           const double *vx, const double *vy, const double *vz,
                           const double *m)
{
    if (!e) return fail(NB_ERR_INVALID_ARGUMENT, "ensemble is NULL");
    const double *src[7] = {x, y, z, vx, vy, vz, m};
    static const int plane[7] = {0, 1, 2, 3, 4, 5, 9};
    for (int k = 0; k < 7; ++k)
        if (!src[k]) return fail(NB_ERR_INVALID_ARGUMENT, "NULL input array");
    const size_t bytes = e->total * sizeof(double);
    for (int k = 0; k < 7; ++k)
        NB_CUDA_TRY(cudaMemcpyAsync(e->f[plane[k]], src[k], bytes, cudaMemcpyHostToDevice,
                                    e->stream));
    for (int k = 6; k < 9; ++k) NB_CUDA_TRY(cudaMemsetAsync(e->f[k], 0, bytes, e->stream));
    NB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->loaded = true;
    e->forces_valid = false;
    return NB_OK;
}

nb_status nb_ensemble_read_state(nb_ensemble *e, double *x, double *y, double *z, double *vx,
                                 double *vy, double *vz, double *ax, double *ay, double *az,
                                 double *m)
{
    if (!e) return fail(NB_ERR_INVALID_ARGUMENT, "ensemble is NULL");
    double *dst[10] = {x, y, z, vx, vy, vz, ax, ay, az, m};
    for (int k = 0; k < 10; ++k)
        if (dst[k])
            NB_CUDA_TRY(cudaMemcpyAsync(dst[k], e->f[k], e->total * sizeof(double),
                                        cudaMemcpyDeviceToHost, e->stream));
    NB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    return NB_OK;
}

nb_status nb_ensemble_tune(nb_ensemble *e, int *ipt_by_bucket)
{
    if (!e) return fail(NB_ERR_INVALID_ARGUMENT, "ensemble is NULL");
    if (!e->loaded) return fail(NB_ERR_NOT_LOADED, "ensemble: nothing loaded");
    if (e->graph) {
        cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
    }
    NB_TRY(e->sorted ? setup_sorted(e) : tune(e));
    if (ipt_by_bucket)
        for (int b = 0; b < 32; ++b) ipt_by_bucket[b] = e->ipt_bucket[b];
    return NB_OK;
}

nb_status nb_ensemble_compute_forces(nb_ensemble *e)
{
    if (!e) return fail(NB_ERR_INVALID_ARGUMENT, "ensemble is NULL");
    NB_TRY(ready(e));
    NB_TRY(sort_systems(e));
    NB_TRY(ens_force(e, e->f[0], e->f[1], e->f[2], e->f[6], e->f[7], e->f[8], false));
    e->forces_valid = true;
    return NB_OK;
}

nb_status nb_ensemble_step(nb_ensemble *e, int integrator, double dt, int nsteps)
{
    NvtxRange range("nb_ensemble_step");
    if (!e) return fail(NB_ERR_INVALID_ARGUMENT, "ensemble is NULL");
    if (integrator < NB_EULER || integrator > NB_RK4)
        return fail(NB_ERR_INVALID_ARGUMENT, "unknown integrator");
    if (nsteps < 0) return fail(NB_ERR_INVALID_ARGUMENT, "nsteps must be >= 0");
    NB_TRY(ready(e));
    if (integrator == NB_VELOCITY_VERLET) NB_TRY(e->old_acc.reserve(sizeof(double) * 3 * e->ps));
    if (integrator == NB_RK4) NB_TRY(e->rk4.reserve(sizeof(double) * 27 * e->ps));
    int done = 0;
    // the sorted path re-sorts here and every `chunk` steps after the first
    // replay's start: the same points for replayed and for direct steps
    NB_TRY(sort_systems(e));
    // Leapfrog / Verlet need a valid start-of-step force before the loop is
    // captured, so that every captured step is the same sequence.
    if ((integrator == NB_LEAPFROG || integrator == NB_VELOCITY_VERLET) && !e->forces_valid &&
        nsteps > 0) {
        NB_TRY(step_direct(e, integrator, dt, false));
        ++done;
    }
    const int remaining = nsteps - done;
    const int chunk = std::min(kGraphChunk, remaining);
    const int launches = chunk >= 2 ? remaining / chunk : 0;
    const bool use_graph = launches > 0 && !e->profiling;
    if (use_graph && (!e->graph || e->graph_integ != integrator || e->graph_dt != dt ||
                      e->graph_steps != chunk)) {
        if (e->graph) {
            cudaGraphExecDestroy(e->graph);
            e->graph = nullptr;
        }
        bool valid_before = e->forces_valid;
        NB_CUDA_TRY(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        nb_status cs = NB_OK;
        for (int k = 0; k < chunk && cs == NB_OK; ++k) cs = step_direct(e, integrator, dt, true);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        e->forces_valid = valid_before;
        if (cs != NB_OK) {
            if (g) cudaGraphDestroy(g);
            return cs;
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&e->graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            e->graph = nullptr;
            return cuda_fail(ce, "cudaGraphInstantiate");
        }
        e->graph_integ = integrator;
        e->graph_dt = dt;
        e->graph_steps = chunk;
    }
    for (int k = 0; k < launches; ++k) {
        if (k > 0) NB_TRY(sort_systems(e));
        if (use_graph) {
            NB_CUDA_TRY(cudaGraphLaunch(e->graph, e->stream));
            ++e->graph_launches;
            // a replayed chunk leaves the force valid exactly as direct steps would
            e->forces_valid = (integrator == NB_LEAPFROG || integrator == NB_VELOCITY_VERLET);
        } else {
            for (int c = 0; c < chunk; ++c) NB_TRY(step_direct(e, integrator, dt, false));
        }
        done += chunk;
    }
    for (; done < nsteps; ++done) NB_TRY(step_direct(e, integrator, dt, false));
    return NB_OK;
}

nb_status nb_ensemble_synchronize(nb_ensemble *e)
{
    if (!e) return fail(NB_ERR_INVALID_ARGUMENT, "ensemble is NULL");
    NB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    return NB_OK;
}

nb_status nb_ensemble_info(nb_ensemble *e, nb_ensemble_info_t *info)
{
    if (!e || !info) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    NB_CUDA_TRY(cudaStreamSynchronize(e->stream));
    info->num_systems = e->num_sys;
    info->total_bodies = (int64_t)e->total;
    double inter = 0.0;
    for (int n : e->sizes) inter += (double)n * (double)(n - 1);
    info->interactions_per_eval = inter;
    info->work_items = e->num_items;
    for (int b = 0; b < 32; ++b) info->ipt_by_bucket[b] = e->ipt_bucket[b];
    info->graph_launches = e->graph_launches;
    info->graph_steps = e->graph_steps;
    double total_ms = 0.0;
    for (size_t k = 0; k < e->timers_used; ++k) {
        float ms = 0.f;
        NB_CUDA_TRY(cudaEventElapsedTime(&ms, e->timers[k].start, e->timers[k].stop));
        total_ms += ms;
    }
    info->force_launches = e->timers_used;
    info->force_kernel_ms = total_ms;
    return NB_OK;
}

nb_status nb_ensemble_profile(nb_ensemble *e, int enable)
{
    if (!e) return fail(NB_ERR_INVALID_ARGUMENT, "ensemble is NULL");
    e->profiling = enable != 0;
    e->timers_used = 0;
    return NB_OK;
}

} // extern "C"
