// nb_sim.cu -- the C ABI (include/nbody_c.h): simulation lifetime, particle
// load/readback, force evaluation and the integrator step loop.
//
// Device layout: one allocation holds the FP64 structure-of-arrays state
// x y z vx vy vz ax ay az m (ten planes of `capacity` doubles, each plane
// 256-byte aligned).  The mixed-precision force path keeps a float4 (x, y, z, m)
// "hi" mirror and a float4 "lo" mirror (32 B per body) that are rebuilt from
// the FP64 positions before each evaluation.  Velocity Verlet keeps a(t) in a
// 3-plane buffer and RK4 keeps three 9-plane stage blocks; both are allocated
// on first use.  Everything is enqueued on the simulation's stream.
#include "nb_internal.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#ifndef NB_DEVICE_CHECKS
#define NB_DEVICE_CHECKS 0
#endif
#define NB_DEVICE_CHECKS_BUILD NB_DEVICE_CHECKS

namespace nb {

std::vector<std::pair<const char *, CheckReader>> &check_readers()
{
    static std::vector<std::pair<const char *, CheckReader>> readers;
    return readers;
}

void register_check_reader(const char *file, CheckReader reader)
{
    check_readers().emplace_back(file, reader);
}

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_fail_allocs_after{-1};  // nb_debug_fail_device_allocations
constexpr size_t kMaxTimers = 1 << 14;

// The next free event pair of a profiling simulation, or nullptr.
const KernelTimer *next_timer(nb_sim *s)
{
    if (!s->profiling || s->timers_used >= kMaxTimers) return nullptr;
    if (s->timers_used == s->timers.size()) {
        KernelTimer t;
        if (cudaEventCreate(&t.start) != cudaSuccess) return nullptr;
        if (cudaEventCreate(&t.stop) != cudaSuccess) {
            cudaEventDestroy(t.start);
            return nullptr;
        }
        s->timers.push_back(t);
    }
    return &s->timers[s->timers_used++];
}
} // namespace

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

void set_error(const std::string &msg) { g_last_error = msg; }

nb_status fail(nb_status s, const std::string &msg)
{
    set_error(msg);
    return s;
}

nb_status cuda_fail(cudaError_t e, const char *what)
{
    std::string msg = std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                      cudaGetErrorString(e) + ")";
    set_error(msg);
    return e == cudaErrorMemoryAllocation ? NB_ERR_OUT_OF_MEMORY : NB_ERR_CUDA;
}

nb_status DevBuf::reserve(size_t want)
{
    if (want <= bytes && ptr) return NB_OK;
    release();
    // the test hook: count down armed allocations, fail the one at zero
    int armed = g_fail_allocs_after.load();
    while (armed >= 0 && !g_fail_allocs_after.compare_exchange_weak(armed, armed - 1)) {
    }
    if (armed == 0) return fail(NB_ERR_OUT_OF_MEMORY, "injected allocation failure");
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        return cuda_fail(e, "cudaMalloc");
    }
    bytes = want;
    return NB_OK;
}

void DevBuf::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

const DeviceProps &device_props()
{
    static DeviceProps p;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaGetDevice(&p.device);
        cudaDeviceGetAttribute(&p.num_sms, cudaDevAttrMultiProcessorCount, p.device);
        cudaDeviceGetAttribute(&p.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                               p.device);
        if (p.num_sms <= 0) p.num_sms = 1;
    });
    return p;
}

static size_t plane_stride(size_t capacity) { return (capacity + 31) / 32 * 32; }

nb_status eval_forces(nb_sim *s, const double *px, const double *py, const double *pz,
                      double *oax, double *oay, double *oaz)
{
    const int n = (int)s->n;
    const double eps2 = s->cfg.softening * s->cfg.softening;
    const KernelTimer *timer = next_timer(s);
    switch (s->cfg.method) {
    case NB_DIRECT_FP64:
        return direct_fp64(px, py, pz, s->m(), n, s->cfg.G, eps2, oax, oay, oaz, s->partials,
                           s->stream, timer);
    case NB_DIRECT_MIXED: {
        if (direct_sorted_enabled(n, s->cfg.flags))
            return direct_mixed_sorted(px, py, pz, s->m(), n, s->cfg.G, eps2, oax, oay, oaz,
                                       s->sorted, s->stream, timer);
        NB_TRY(s->split_hi.reserve(sizeof(float4) * s->capacity));
        NB_TRY(s->split_lo.reserve(sizeof(float4) * s->capacity));
        float4 *hi = s->split_hi.as<float4>(), *lo = s->split_lo.as<float4>();
        NB_TRY(split_positions(px, py, pz, s->m(), n, hi, lo, s->stream));
        return direct_mixed(hi, lo, n, s->cfg.G, eps2, oax, oay, oaz, s->partials, s->stream,
                            timer);
    }
    case NB_BARNES_HUT:
        if (!s->bh) s->bh = bh_create();
        return bh_compute(s->bh, px, py, pz, s->m(), n, s->cfg.G, eps2, s->cfg.theta,
                          s->cfg.leaf_capacity, oax, oay, oaz, s->stream, timer,
                          NB_FLAG_BH_REUSE_OF(s->cfg.flags),
                          (s->cfg.flags & NB_FLAG_BH_QUADRUPOLE) != 0,
                          (s->cfg.flags & NB_FLAG_BH_REFERENCE_OPENING) != 0);
    default:
        return fail(NB_ERR_INVALID_ARGUMENT, "unknown force method");
    }
}

static nb_status check_config(const nb_config *c)
{
    if (!c) return fail(NB_ERR_INVALID_ARGUMENT, "config is NULL");
    if (c->method < NB_DIRECT_FP64 || c->method > NB_BARNES_HUT)
        return fail(NB_ERR_INVALID_ARGUMENT, "config.method out of range");
    if (!(c->softening >= 0.0)) return fail(NB_ERR_INVALID_ARGUMENT, "softening must be >= 0");
    if (c->method == NB_BARNES_HUT) {
        if (!(c->theta >= 0.0)) return fail(NB_ERR_INVALID_ARGUMENT, "theta must be >= 0");
        if (c->leaf_capacity < 1 || c->leaf_capacity > 64)
            return fail(NB_ERR_INVALID_ARGUMENT, "leaf_capacity must be in [1, 64]");
    }
    return NB_OK;
}

static nb_status step_once(nb_sim *s, int integ, double dt)
{
    const int n = (int)s->n;
    cudaStream_t st = s->stream;
    switch (integ) {
    case NB_EULER:
    case NB_EULER_CROMER:
        NB_TRY(eval_forces(s, s->x(), s->y(), s->z(), s->ax(), s->ay(), s->az()));
        NB_TRY(kick_drift(integ, n, dt, s->x(), s->y(), s->z(), s->vx(), s->vy(), s->vz(),
                          s->ax(), s->ay(), s->az(), nullptr, nullptr, nullptr, st));
        s->forces_valid = false;
        return NB_OK;
    case NB_LEAPFROG:
        if (!s->forces_valid)
            NB_TRY(eval_forces(s, s->x(), s->y(), s->z(), s->ax(), s->ay(), s->az()));
        NB_TRY(kick_drift(integ, n, dt, s->x(), s->y(), s->z(), s->vx(), s->vy(), s->vz(),
                          s->ax(), s->ay(), s->az(), nullptr, nullptr, nullptr, st));
        s->forces_valid = false;
        NB_TRY(eval_forces(s, s->x(), s->y(), s->z(), s->ax(), s->ay(), s->az()));
        NB_TRY(kick(integ, n, dt, s->vx(), s->vy(), s->vz(), s->ax(), s->ay(), s->az(), nullptr,
                    nullptr, nullptr, st));
        s->forces_valid = true;
        return NB_OK;
    case NB_VELOCITY_VERLET: {
        const size_t ps = plane_stride(s->capacity);
        NB_TRY(s->old_acc.reserve(sizeof(double) * 3 * ps));
        double *o = s->old_acc.as<double>();
        if (!s->forces_valid)
            NB_TRY(eval_forces(s, s->x(), s->y(), s->z(), s->ax(), s->ay(), s->az()));
        NB_TRY(kick_drift(integ, n, dt, s->x(), s->y(), s->z(), s->vx(), s->vy(), s->vz(),
                          s->ax(), s->ay(), s->az(), o, o + ps, o + 2 * ps, st));
        s->forces_valid = false;
        NB_TRY(eval_forces(s, s->x(), s->y(), s->z(), s->ax(), s->ay(), s->az()));
        NB_TRY(kick(integ, n, dt, s->vx(), s->vy(), s->vz(), s->ax(), s->ay(), s->az(), o,
                    o + ps, o + 2 * ps, st));
        s->forces_valid = true;
        return NB_OK;
    }
    case NB_RK4: {
        const size_t ps = plane_stride(s->capacity);
        NB_TRY(s->rk4.reserve(sizeof(double) * 27 * ps));
        double *k2 = s->rk4.as<double>(), *k3 = k2 + 9 * ps, *k4 = k3 + 9 * ps;
        auto P = [ps](double *k, int c) { return k + c * ps; };
        NB_TRY(eval_forces(s, s->x(), s->y(), s->z(), s->ax(), s->ay(), s->az()));
        const double h = dt / 2.0;
        NB_TRY(rk4_stage(n, h, s->x(), s->y(), s->z(), s->vx(), s->vy(), s->vz(), s->vx(),
                         s->vy(), s->vz(), s->ax(), s->ay(), s->az(), P(k2, 0), P(k2, 1),
                         P(k2, 2), P(k2, 3), P(k2, 4), P(k2, 5), st));
        NB_TRY(eval_forces(s, P(k2, 0), P(k2, 1), P(k2, 2), P(k2, 6), P(k2, 7), P(k2, 8)));
        NB_TRY(rk4_stage(n, h, s->x(), s->y(), s->z(), s->vx(), s->vy(), s->vz(), P(k2, 3),
                         P(k2, 4), P(k2, 5), P(k2, 6), P(k2, 7), P(k2, 8), P(k3, 0), P(k3, 1),
                         P(k3, 2), P(k3, 3), P(k3, 4), P(k3, 5), st));
        NB_TRY(eval_forces(s, P(k3, 0), P(k3, 1), P(k3, 2), P(k3, 6), P(k3, 7), P(k3, 8)));
        NB_TRY(rk4_stage(n, dt, s->x(), s->y(), s->z(), s->vx(), s->vy(), s->vz(), P(k3, 3),
                         P(k3, 4), P(k3, 5), P(k3, 6), P(k3, 7), P(k3, 8), P(k4, 0), P(k4, 1),
                         P(k4, 2), P(k4, 3), P(k4, 4), P(k4, 5), st));
        NB_TRY(eval_forces(s, P(k4, 0), P(k4, 1), P(k4, 2), P(k4, 6), P(k4, 7), P(k4, 8)));
        NB_TRY(rk4_combine(n, dt, s->x(), s->y(), s->z(), s->vx(), s->vy(), s->vz(), s->ax(),
                           s->ay(), s->az(), k2, k3, k4, st));
        s->forces_valid = false;
        return NB_OK;
    }
    default:
        return fail(NB_ERR_INVALID_ARGUMENT, "unknown integrator");
    }
}

void reset_step_graph(nb_sim *s)
{
    if (s->step_graph) cudaGraphExecDestroy(s->step_graph);
    s->step_graph = nullptr;
    s->graph_integ = -1;
    s->warm_integ = -1;
}

// Steps whose launch sequence is the same every time (no host-side choice
// that depends on earlier evaluations: not the re-sorting mixed kernel, not
// Barnes-Hut tree reuse), on a stream that may be captured.
static bool graph_eligible(const nb_sim *s)
{
    if (s->graphs_off || s->profiling || s->stream == nullptr) return false;
    switch (s->cfg.method) {
    case NB_DIRECT_FP64: return true;
    case NB_DIRECT_MIXED: return !direct_sorted_enabled((int)s->n, s->cfg.flags);
    case NB_BARNES_HUT: return NB_FLAG_BH_REUSE_OF(s->cfg.flags) <= 1;
    default: return false;
    }
}

// Captures one step into a graph and launches it.  A failed capture (a call
// that cannot be captured) turns graphs off for this simulation and runs the
// step directly.
static nb_status capture_step(nb_sim *s, int integ, double dt)
{
    reset_step_graph(s);
    const bool fv = s->forces_valid;
    NB_CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    const nb_status r = step_once(s, integ, dt);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (r != NB_OK) {
        if (g) cudaGraphDestroy(g);
        return r;
    }
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess && g && cudaGraphInstantiate(&exec, g, 0) == cudaSuccess) {
        size_t count = 0;
        cudaGraphGetNodes(g, nullptr, &count);
        std::vector<cudaGraphNode_t> nodes(count);
        if (count) cudaGraphGetNodes(g, nodes.data(), &count);
        uint64_t kernels = 0;
        for (auto nd : nodes) {
            cudaGraphNodeType type;
            if (cudaGraphNodeGetType(nd, &type) == cudaSuccess && type == cudaGraphNodeTypeKernel)
                ++kernels;
        }
        cudaGraphDestroy(g);
        s->step_graph = exec;
        s->graph_integ = integ;
        s->graph_dt = dt;
        s->graph_fv_before = fv;
        s->graph_fv_after = s->forces_valid;
        s->graph_kernels = kernels;
        NB_CUDA_TRY(cudaGraphLaunch(exec, s->stream));
        return NB_OK;
    }
    // capture did not produce a graph: nothing ran; run the step directly
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    s->graphs_off = true;
    s->forces_valid = fv;
    return step_once(s, integ, dt);
}

static nb_status step_with_graphs(nb_sim *s, int integ, double dt)
{
    if (!graph_eligible(s)) return step_once(s, integ, dt);
    if (s->step_graph && s->graph_integ == integ && s->graph_dt == dt &&
        s->graph_fv_before == s->forces_valid) {
        NB_CUDA_TRY(cudaGraphLaunch(s->step_graph, s->stream));
        count_launches(s->graph_kernels);
        s->forces_valid = s->graph_fv_after;
        if (s->cfg.method == NB_BARNES_HUT) bh_mark_count_stale(s->bh);
        return NB_OK;
    }
    if (s->warm_integ == integ && s->warm_dt == dt) return capture_step(s, integ, dt);
    reset_step_graph(s);
    NB_TRY(step_once(s, integ, dt));
    s->warm_integ = integ;
    s->warm_dt = dt;
    return NB_OK;
}

} // namespace nb

using namespace nb;

extern "C" {

nb_status nb_config_default(nb_config *cfg)
{
    if (!cfg) return fail(NB_ERR_INVALID_ARGUMENT, "cfg is NULL");
    cfg->method = NB_DIRECT_MIXED;
    cfg->G = 1.0;
    cfg->softening = 0.0;
    cfg->theta = 0.5;
    cfg->leaf_capacity = 8;
    cfg->flags = 0;
    return NB_OK;
}

nb_status nb_create(const nb_config *cfg, size_t capacity, void *stream, nb_sim **out)
{
    if (!out) return fail(NB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    NB_TRY(check_config(cfg));
    if (capacity == 0 || capacity > (size_t)1 << 30)
        return fail(NB_ERR_INVALID_ARGUMENT, "capacity must be in [1, 2^30]");
    int dev = 0;
    NB_CUDA_TRY(cudaGetDevice(&dev));
    (void)device_props();
    nb_sim *s = new nb_sim();
    s->cfg = *cfg;
    s->capacity = capacity;
    s->stream = static_cast<cudaStream_t>(stream);
    s->device = dev;
    const size_t ps = plane_stride(capacity);
    nb_status st = s->state.reserve(sizeof(double) * 10 * ps);
    if (st != NB_OK) {
        delete s;
        return st;
    }
    for (int k = 0; k < 10; ++k) s->f[k] = s->state.as<double>() + k * ps;
    cudaError_t e = cudaMemsetAsync(s->state.ptr, 0, s->state.bytes, s->stream);
    if (e != cudaSuccess) {
        s->state.release();
        delete s;
        return cuda_fail(e, "cudaMemsetAsync");
    }
    *out = s;
    return NB_OK;
}

nb_status nb_destroy(nb_sim *s)
{
    if (!s) return NB_OK;
    cudaStreamSynchronize(s->stream);
    reset_step_graph(s);
    for (auto &t : s->timers) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    if (s->bh) bh_destroy(s->bh);
    s->state.release();
    s->split_hi.release();
    s->split_lo.release();
    s->sorted.release();
    s->partials.release();
    s->old_acc.release();
    s->rk4.release();
    s->diag_scratch.release();
    delete s;
    return NB_OK;
}

nb_status nb_set_config(nb_sim *s, const nb_config *cfg)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    NB_TRY(check_config(cfg));
    const bool same = s->cfg.method == cfg->method && s->cfg.G == cfg->G &&
                      s->cfg.softening == cfg->softening && s->cfg.theta == cfg->theta &&
                      s->cfg.leaf_capacity == cfg->leaf_capacity;
    const bool flags_changed = s->cfg.flags != cfg->flags;
    s->cfg = *cfg;
    if (!same || flags_changed) reset_step_graph(s);
    if (!same) {
        s->forces_valid = false;
        bh_invalidate(s->bh);
    }
    return NB_OK;
}

nb_status nb_get_config(const nb_sim *s, nb_config *cfg)
{
    if (!s || !cfg) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    *cfg = s->cfg;
    return NB_OK;
}

static nb_status load_impl(nb_sim *s, size_t n, const double *const *src, cudaMemcpyKind kind)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (n > s->capacity) return fail(NB_ERR_CAPACITY, "n exceeds the capacity of the simulation");
    for (int k = 0; k < 7; ++k)
        if (n > 0 && !src[k]) return fail(NB_ERR_INVALID_ARGUMENT, "NULL input array");
    // x y z vx vy vz -> planes 0..5, m -> plane 9
    static const int dst_plane[7] = {0, 1, 2, 3, 4, 5, 9};
    const size_t bytes = n * sizeof(double);
    for (int k = 0; k < 7 && n > 0; ++k)
        NB_CUDA_TRY(cudaMemcpyAsync(s->f[dst_plane[k]], src[k], bytes, kind, s->stream));
    // a = 0 until forces are computed: one memset when the three planes are
    // the engine's own (adjacent in its state allocation), else one per plane
    const size_t ps = plane_stride(s->capacity);
    const double *own = s->state.as<double>();
    if (n > 0 && s->f[6] == own + 6 * ps && s->f[7] == own + 7 * ps && s->f[8] == own + 8 * ps)
        NB_CUDA_TRY(cudaMemsetAsync(s->f[6], 0, sizeof(double) * (2 * ps + n), s->stream));
    else
        for (int k = 6; k < 9 && n > 0; ++k)
            NB_CUDA_TRY(cudaMemsetAsync(s->f[k], 0, bytes, s->stream));
    s->n = n;
    s->forces_valid = false;
    bh_invalidate(s->bh);
    reset_step_graph(s);
    return NB_OK;
}

nb_status nb_load(nb_sim *s, size_t n, const double *x, const double *y, const double *z,
                  const double *vx, const double *vy, const double *vz, const double *m)
{
    const double *src[7] = {x, y, z, vx, vy, vz, m};
    return load_impl(s, n, src, cudaMemcpyHostToDevice);
}

nb_status nb_load_device(nb_sim *s, size_t n, const double *x, const double *y, const double *z,
                         const double *vx, const double *vy, const double *vz, const double *m)
{
    const double *src[7] = {x, y, z, vx, vy, vz, m};
    return load_impl(s, n, src, cudaMemcpyDeviceToDevice);
}

nb_status nb_read_state(nb_sim *s, double *x, double *y, double *z, double *vx, double *vy,
                        double *vz, double *ax, double *ay, double *az, double *m)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    double *dst[10] = {x, y, z, vx, vy, vz, ax, ay, az, m};
    const size_t bytes = s->n * sizeof(double);
    for (int k = 0; k < 10; ++k)
        if (dst[k] && bytes)
            NB_CUDA_TRY(cudaMemcpyAsync(dst[k], s->f[k], bytes, cudaMemcpyDeviceToHost,
                                        s->stream));
    NB_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return NB_OK;
}

nb_status nb_bind_device(nb_sim *s, size_t n, double *const *arrays10)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (!arrays10) {
        const size_t ps = plane_stride(s->capacity);
        for (int k = 0; k < 10; ++k) s->f[k] = s->state.as<double>() + k * ps;
        s->n = std::min(s->n, s->capacity);
        s->forces_valid = false;
        return NB_OK;
    }
    if (n > s->capacity) return fail(NB_ERR_CAPACITY, "n exceeds the capacity of the simulation");
    for (int k = 0; k < 10; ++k)
        if (n > 0 && !arrays10[k]) return fail(NB_ERR_INVALID_ARGUMENT, "NULL device array");
    bool same = s->n == n;
    for (int k = 0; k < 10; ++k) {
        same = same && s->f[k] == arrays10[k];
        s->f[k] = arrays10[k];
    }
    s->n = n;
    if (!same) {
        s->forces_valid = false;
        bh_invalidate(s->bh);
        reset_step_graph(s);
    }
    return NB_OK;
}

nb_status nb_device_arrays(nb_sim *s, double **ptrs10)
{
    if (!s || !ptrs10) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    for (int k = 0; k < 10; ++k) ptrs10[k] = s->f[k];
    return NB_OK;
}

nb_status nb_num_bodies(const nb_sim *s, size_t *n)
{
    if (!s || !n) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    *n = s->n;
    return NB_OK;
}

nb_status nb_compute_forces(nb_sim *s)
{
    NvtxRange range("nb_compute_forces");
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (s->n == 0) return fail(NB_ERR_NOT_LOADED, "no bodies loaded");
    NB_TRY(eval_forces(s, s->x(), s->y(), s->z(), s->ax(), s->ay(), s->az()));
    s->forces_valid = true;
    return NB_OK;
}

nb_status nb_step(nb_sim *s, int integrator, double dt, int nsteps)
{
    NvtxRange range("nb_step");
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (nsteps < 0) return fail(NB_ERR_INVALID_ARGUMENT, "nsteps must be >= 0");
    if (integrator < NB_EULER || integrator > NB_RK4)
        return fail(NB_ERR_INVALID_ARGUMENT, "unknown integrator");
    if (s->n == 0) return fail(NB_ERR_NOT_LOADED, "no bodies loaded");
    for (int k = 0; k < nsteps; ++k) NB_TRY(step_with_graphs(s, integrator, dt));
    return NB_OK;
}

nb_status nb_invalidate_forces(nb_sim *s)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    s->forces_valid = false;
    return NB_OK;
}

nb_status nb_synchronize(nb_sim *s)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    NB_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return NB_OK;
}

nb_status nb_diagnostics(nb_sim *s, nb_diag *out)
{
    if (!s || !out) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    if (s->n == 0) return fail(NB_ERR_NOT_LOADED, "no bodies loaded");
    return diagnostics(s->x(), s->y(), s->z(), s->vx(), s->vy(), s->vz(), s->m(), (int)s->n,
                       s->cfg.G, s->cfg.softening * s->cfg.softening, s->diag_scratch,
                       s->stream, out);
}

nb_status nb_bh_build(nb_sim *s, nb_bh_info *info)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (s->n == 0) return fail(NB_ERR_NOT_LOADED, "no bodies loaded");
    if (!s->bh) s->bh = bh_create();
    const double eps2 = s->cfg.softening * s->cfg.softening;
    NB_TRY(bh_compute(s->bh, s->x(), s->y(), s->z(), s->m(), (int)s->n, s->cfg.G, eps2,
                      s->cfg.theta, s->cfg.leaf_capacity, nullptr, nullptr, nullptr,
                      s->stream));
    if (info) NB_TRY(bh_info(s->bh, s->stream, info));
    return NB_OK;
}

nb_status nb_bh_get_info(nb_sim *s, nb_bh_info *info)
{
    if (!s || !info) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->bh) return fail(NB_ERR_NOT_LOADED, "no Barnes-Hut tree built");
    return bh_info(s->bh, s->stream, info);
}

nb_status nb_bh_read_order(nb_sim *s, uint64_t *codes, uint32_t *order)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (!s->bh) return fail(NB_ERR_NOT_LOADED, "no Barnes-Hut tree built");
    return bh_read_order(s->bh, s->stream, codes, order);
}

nb_status nb_bh_read_nodes(nb_sim *s, int max_nodes, int *depth, uint64_t *prefix, int *first,
                           int *count, int *is_leaf, int *skip, float *com_mass)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    if (!s->bh) return fail(NB_ERR_NOT_LOADED, "no Barnes-Hut tree built");
    return bh_read_nodes(s->bh, s->stream, max_nodes, depth, prefix, first, count, is_leaf,
                         skip, com_mass);
}

nb_status nb_profile_enable(nb_sim *s, int enable)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "sim is NULL");
    s->profiling = enable != 0;
    reset_step_graph(s);
    return NB_OK;
}

nb_status nb_profile_read(nb_sim *s, nb_profile *out, int reset)
{
    if (!s || !out) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    NB_CUDA_TRY(cudaStreamSynchronize(s->stream));
    out->kernel_launches = g_launches.load();
    out->force_launches = s->timers_used;
    double total = 0.0;
    for (size_t k = 0; k < s->timers_used; ++k) {
        float ms = 0.f;
        NB_CUDA_TRY(cudaEventElapsedTime(&ms, s->timers[k].start, s->timers[k].stop));
        total += ms;
    }
    out->force_kernel_ms = total;
    if (reset) s->timers_used = 0;
    return NB_OK;
}

uint64_t nb_kernel_launch_count(void) { return g_launches.load(); }

const char *nb_status_string(nb_status s)
{
    switch (s) {
    case NB_OK: return "ok";
    case NB_ERR_INVALID_ARGUMENT: return "invalid argument";
    case NB_ERR_CUDA: return "CUDA error";
    case NB_ERR_OUT_OF_MEMORY: return "out of device memory";
    case NB_ERR_CAPACITY: return "capacity exceeded";
    case NB_ERR_NOT_LOADED: return "no bodies loaded";
    case NB_ERR_DEVICE_FAULT: return "device-reported error";
    case NB_ERR_UNSUPPORTED: return "unsupported";
    case NB_ERR_IO: return "file input/output error";
    case NB_ERR_CANCELLED: return "cancelled";
    }
    return "unknown status";
}

const char *nb_last_error(void) { return g_last_error.c_str(); }

const char *nb_version(void) { return "nbody-gb300 0.1 (sm_103a)"; }

nb_status nb_debug_device_checks(int *enabled)
{
    if (enabled) *enabled = NB_DEVICE_CHECKS_BUILD;
    std::string first;
    for (const auto &r : check_readers()) {
        DeviceCheck c{};
        NB_TRY(r.second(&c, true));
        if (c.failed && first.empty())
            first = std::string(r.first) + ":" + std::to_string(c.line) + ": index " +
                    std::to_string(c.index) + " outside [0, " + std::to_string(c.bound) + ")";
    }
    if (!first.empty()) return fail(NB_ERR_DEVICE_FAULT, "device check failed at " + first);
    return NB_OK;
}

nb_status nb_debug_fp32_rate(double *lane_ops_per_s)
{
    if (!lane_ops_per_s) return fail(NB_ERR_INVALID_ARGUMENT, "lane_ops_per_s is NULL");
    return nb::fp32_rate(lane_ops_per_s);
}

nb_status nb_debug_fail_device_allocations(int after)
{
    g_fail_allocs_after.store(after < 0 ? -1 : after);
    return NB_OK;
}

} // extern "C"
