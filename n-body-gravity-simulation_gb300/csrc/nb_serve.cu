// nb_serve.cu -- continuous-batching server for simulation jobs (nb_server_*).
//
// No reference counterpart.  Jobs are submitted with their initial state and
// a step count; each tick
//   1. admits queued jobs (in arrival order, later small jobs may pass a job
//      that does not fit) while their device memory fits the HBM budget;
//   2. advances every running job by one leapfrog step:
//      - direct jobs (n < direct_max_n) live in one body pool and advance
//        together: one per-body kick-drift and kick over the pool and one
//        persistent batched force launch over all of them (nb_batch.cu);
//      - Barnes-Hut jobs each own a simulation object and run on one of
//        kBHStreams streams (the process should allow that many hardware
//        queues: CUDA_DEVICE_MAX_CONNECTIONS >= 16), each stream's jobs issued
//        by that stream's thread of a pool kept for the server's lifetime (a
//        tree build reads its node count on the host, which then blocks only
//        that stream's later jobs), overlapping with the direct batch and
//        with each other;
//   3. retires jobs that reached their step count (state copied to the host,
//      memory returned).
// A job's arithmetic does not depend on the other jobs of a tick (the batched
// kernel sums each system alone, updates are per body, Barnes-Hut jobs are
// separate objects), so its result is the same alone and in any mix.
// Per-step latency is the time from the start of a tick to the completion of
// that job's step (CUDA events).
#include "nb_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace nb {
namespace {

using Clock = std::chrono::steady_clock;

constexpr size_t kDirectBytesPerBody = 10 * 8 + 32;  // FP64 planes + hi/lo mirror
constexpr size_t kBHBytesPerBody = 320;              // state + sort + tree buffers (upper bound)
constexpr int kBHStreams = 16;

struct Job {
    int64_t id = 0;
    size_t n = 0;
    int steps = 0;
    int done = 0;
    bool direct = true;
    std::vector<double> init;   // 7 n: x y z vx vy vz m (until admitted)
    std::vector<double> result; // 10 n after retirement
    size_t first = 0;           // pool slot (direct)
    nb_sim *sim = nullptr;      // Barnes-Hut
    int stream_index = 0;
    Clock::time_point submitted, admitted;
    bool finished = false;
    cudaEvent_t step_done = nullptr;
    nb_status status = NB_OK;   // a failure of this job alone, or NB_ERR_CANCELLED
    std::string error;
};

// First-fit free list over [0, capacity) body slots.
struct SlotAllocator {
    std::map<size_t, size_t> free;  // start -> length
    size_t capacity = 0, high_water = 0;
    void init(size_t cap)
    {
        free.clear();
        free[0] = cap;
        capacity = cap;
        high_water = 0;
    }
    bool take(size_t n, size_t *out)
    {
        for (auto it = free.begin(); it != free.end(); ++it) {
            if (it->second >= n) {
                const size_t s = it->first, len = it->second;
                free.erase(it);
                if (len > n) free[s + n] = len - n;
                *out = s;
                high_water = std::max(high_water, s + n);
                return true;
            }
        }
        return false;
    }
    void give(size_t s, size_t n)
    {
        auto it = free.emplace(s, n).first;
        auto next = std::next(it);
        if (next != free.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free.erase(next);
        }
        if (it != free.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free.erase(it);
                it = prev;
            }
        }
        // shrink the high-water mark when the top block is free
        auto last = std::prev(free.end());
        if (last->first + last->second == capacity && last->first < high_water)
            high_water = last->first;
    }
};

int default_ipt(int n) { return n < 1024 ? 1 : (n < 4096 ? 2 : 4); }

double quantile(std::vector<double> v, double q)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = q * (double)(v.size() - 1);
    const size_t lo = (size_t)std::floor(pos), hi = std::min(v.size() - 1, lo + 1);
    return v[lo] + (pos - (double)lo) * (v[hi] - v[lo]);
}

// One host thread per Barnes-Hut stream for the server's lifetime.  Each tick
// dispatches a task to the busy streams (each thread issues its stream's
// steps; a node-count read-back then blocks only that thread) and later waits
// until all of them are done.
class StreamPool {
public:
    // false when the threads cannot be created (the pool is then empty)
    bool start(int threads, int device)
    {
        busy_.assign(threads, false);
        try {
            for (int k = 0; k < threads; ++k)
                pool_.emplace_back([this, k, device] { loop(k, device); });
        } catch (...) {
            stop();
            return false;
        }
        return true;
    }
    void dispatch(std::function<void(int)> task, const std::vector<bool> &busy)
    {
        std::lock_guard<std::mutex> lock(mu_);
        task_ = std::move(task);
        busy_ = busy;
        pending_ = 0;
        for (bool b : busy_) pending_ += b;
        ++generation_;
        cv_work_.notify_all();
    }
    void wait()
    {
        std::unique_lock<std::mutex> lock(mu_);
        cv_done_.wait(lock, [this] { return pending_ == 0; });
    }
    void stop()
    {
        {
            std::lock_guard<std::mutex> lock(mu_);
            stop_ = true;
            cv_work_.notify_all();
        }
        for (auto &t : pool_)
            if (t.joinable()) t.join();
        pool_.clear();
    }

private:
    void loop(int k, int device)
    {
        cudaSetDevice(device);
        uint64_t seen = 0;
        while (true) {
            std::function<void(int)> task;
            {
                std::unique_lock<std::mutex> lock(mu_);
                cv_work_.wait(lock, [&] { return stop_ || generation_ != seen; });
                if (stop_) return;
                seen = generation_;
                if (!busy_[k]) continue;
                task = task_;
            }
            task(k);
            std::lock_guard<std::mutex> lock(mu_);
            if (--pending_ == 0) cv_done_.notify_all();
        }
    }
    std::vector<std::thread> pool_;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::function<void(int)> task_;
    std::vector<bool> busy_;
    uint64_t generation_ = 0;
    int pending_ = 0;
    bool stop_ = false;
};

} // namespace
} // namespace nb

struct nb_server {
    nb_server_config cfg{};
    cudaStream_t stream = nullptr;
    cudaStream_t bh_streams[nb::kBHStreams] = {};
    nb::StreamPool pool_threads;  // issues the Barnes-Hut streams' steps
    size_t ps = 0;
    nb::DevBuf pool, hi, lo, d_sys, d_items, d_counter, d_new_sys, d_new_items;
    double *f[10] = {};
    nb::SlotAllocator slots;
    int64_t next_id = 1;
    std::deque<std::unique_ptr<nb::Job>> queue;
    std::vector<std::unique_ptr<nb::Job>> running;
    std::map<int64_t, std::unique_ptr<nb::Job>> finished;
    size_t bh_bytes = 0;
    size_t peak_bytes = 0;
    bool items_dirty = true;
    int num_items = 0;
    cudaEvent_t tick_start = nullptr, direct_done = nullptr;
    // statistics
    std::vector<double> step_ms, queue_ms;
    double interactions = 0.0, busy_ms = 0.0;
    uint64_t submitted = 0, steps_done = 0, ticks = 0, failed = 0, cancelled = 0;
    int max_running = 0;
    double admit_ms = 0.0, issue_ms = 0.0, wait_ms = 0.0, retire_ms = 0.0;
    double upload_ms = 0.0, direct_ms = 0.0, join_ms = 0.0;  // parts of issue_ms
};

namespace nb {
namespace {

size_t pool_bytes(const nb_server *s) { return s->pool.bytes + s->hi.bytes + s->lo.bytes; }

nb_status upload_systems(nb_server *s, const std::vector<Job *> &jobs, DevBuf &d_sys,
                         DevBuf &d_items, int *num_items)
{
    std::vector<SysDesc> sys;
    for (Job *j : jobs) sys.push_back(SysDesc{(int)j->first, (int)j->n, default_ipt((int)j->n), 0});
    std::vector<WorkItem> items;
    build_work_items(sys, items);
    *num_items = (int)items.size();
    if (sys.empty()) return NB_OK;
    NB_TRY(d_sys.reserve(sizeof(SysDesc) * sys.size()));
    NB_TRY(d_items.reserve(sizeof(WorkItem) * items.size()));
    NB_CUDA_TRY(cudaMemcpyAsync(d_sys.ptr, sys.data(), sizeof(SysDesc) * sys.size(),
                                cudaMemcpyHostToDevice, s->stream));
    NB_CUDA_TRY(cudaMemcpyAsync(d_items.ptr, items.data(), sizeof(WorkItem) * items.size(),
                                cudaMemcpyHostToDevice, s->stream));
    NB_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return NB_OK;
}

// Frees a running job's device state (pool slot, or its simulation and its
// share of the budget) and its event.  Only between ticks: nothing of the job
// is in flight then.
void drop_resources(nb_server *s, Job *j)
{
    if (j->direct) {
        s->slots.give(j->first, j->n);
    } else if (j->sim) {
        nb_destroy(j->sim);
        j->sim = nullptr;
        s->bh_bytes -= kBHBytesPerBody * j->n;
    }
    if (j->step_done) cudaEventDestroy(j->step_done);
    j->step_done = nullptr;
    s->items_dirty = true;
}

// Moves a job that ends without a result (failed or cancelled) to the
// finished table.
void end_job(nb_server *s, std::unique_ptr<Job> j)
{
    j->finished = true;
    if (j->status == NB_ERR_CANCELLED) ++s->cancelled;
    else ++s->failed;
    const int64_t id = j->id;
    s->finished[id] = std::move(j);
}

nb_status admit(nb_server *s, std::vector<Job *> &new_direct)
{
    for (auto it = s->queue.begin(); it != s->queue.end();) {
        Job *j = it->get();
        bool ok = false;
        if (j->direct) {
            size_t first = 0;
            if (s->slots.take(j->n, &first)) {
                j->first = first;
                static const int plane[7] = {0, 1, 2, 3, 4, 5, 9};
                for (int k = 0; k < 7; ++k)
                    NB_CUDA_TRY(cudaMemcpyAsync(s->f[plane[k]] + first, j->init.data() + k * j->n,
                                                j->n * sizeof(double), cudaMemcpyHostToDevice,
                                                s->stream));
                new_direct.push_back(j);
                ok = true;
            }
        } else {
            const size_t need = kBHBytesPerBody * j->n;
            if (pool_bytes(s) + s->bh_bytes + need <= s->cfg.hbm_budget_bytes) {
                nb_config c;
                nb_config_default(&c);
                c.method = NB_BARNES_HUT;
                c.G = s->cfg.G;
                c.softening = s->cfg.softening;
                c.theta = s->cfg.theta;
                c.leaf_capacity = s->cfg.leaf_capacity;
                j->stream_index = (int)(j->id % kBHStreams);
                cudaStream_t st = s->bh_streams[j->stream_index];
                const double *p = j->init.data();
                const size_t n = j->n;
                nb_status r = nb_create(&c, n, st, &j->sim);
                if (r == NB_OK)
                    r = nb_load(j->sim, n, p, p + n, p + 2 * n, p + 3 * n, p + 4 * n,
                                p + 5 * n, p + 6 * n);
                if (r == NB_OK) {
                    const cudaError_t e = cudaStreamSynchronize(st);
                    if (e != cudaSuccess) r = cuda_fail(e, "cudaStreamSynchronize");
                }
                if (r != NB_OK) {  // this job alone fails; the others carry on
                    j->status = r;
                    j->error = nb_last_error();
                    if (j->sim) nb_destroy(j->sim);
                    j->sim = nullptr;
                    std::vector<double>().swap(j->init);
                    end_job(s, std::move(*it));
                    it = s->queue.erase(it);
                    continue;
                }
                s->bh_bytes += need;
                ok = true;
            }
        }
        if (ok) {
            j->admitted = Clock::now();
            s->queue_ms.push_back(
                std::chrono::duration<double, std::milli>(j->admitted - j->submitted).count());
            std::vector<double>().swap(j->init);
            NB_CUDA_TRY(cudaEventCreateWithFlags(&j->step_done, cudaEventDefault));
            s->running.push_back(std::move(*it));
            it = s->queue.erase(it);
            s->items_dirty = true;
        } else {
            ++it;
        }
    }
    s->peak_bytes = std::max(s->peak_bytes, pool_bytes(s) + s->bh_bytes);
    return NB_OK;
}

nb_status retire(nb_server *s)
{
    for (auto it = s->running.begin(); it != s->running.end();) {
        Job *j = it->get();
        if (j->status != NB_OK) {  // failed while stepping: free it, keep the error
            drop_resources(s, j);
            end_job(s, std::move(*it));
            it = s->running.erase(it);
            continue;
        }
        if (j->done < j->steps) {
            ++it;
            continue;
        }
        j->result.resize(10 * j->n);
        double *r = j->result.data();
        const size_t n = j->n;
        if (j->direct) {
            for (int k = 0; k < 10; ++k)
                NB_CUDA_TRY(cudaMemcpyAsync(r + k * n, s->f[k] + j->first, n * sizeof(double),
                                            cudaMemcpyDeviceToHost, s->stream));
            NB_CUDA_TRY(cudaStreamSynchronize(s->stream));
            s->slots.give(j->first, n);
        } else {
            NB_TRY(nb_read_state(j->sim, r, r + n, r + 2 * n, r + 3 * n, r + 4 * n, r + 5 * n,
                                 r + 6 * n, r + 7 * n, r + 8 * n, r + 9 * n));
            nb_bh_info info;
            if (nb_bh_get_info(j->sim, &info) == NB_OK)
                s->interactions += (double)info.interactions_total;
            nb_destroy(j->sim);
            j->sim = nullptr;
            s->bh_bytes -= kBHBytesPerBody * n;
        }
        cudaEventDestroy(j->step_done);
        j->step_done = nullptr;
        j->finished = true;
        s->finished[j->id] = std::move(*it);
        it = s->running.erase(it);
        s->items_dirty = true;
    }
    return NB_OK;
}

double ms_since(Clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

nb_status tick(nb_server *s)
{
    NvtxRange range("server_tick");
    std::vector<Job *> new_direct;
    auto t_phase = Clock::now();
    NB_TRY(admit(s, new_direct));
    s->admit_ms += ms_since(t_phase);
    t_phase = Clock::now();
    if (s->running.empty()) return NB_OK;
    s->max_running = std::max(s->max_running, (int)s->running.size());
    std::vector<Job *> direct, bh;
    for (auto &j : s->running) (j->direct ? direct : bh).push_back(j.get());
    const double eps2 = s->cfg.softening * s->cfg.softening;
    const double dt = s->cfg.dt;
    const int hw = (int)s->slots.high_water;
    if (s->items_dirty) {
        const auto t_up = Clock::now();
        NB_TRY(upload_systems(s, direct, s->d_sys, s->d_items, &s->num_items));
        s->items_dirty = false;
        s->upload_ms += ms_since(t_up);
    }
    NB_CUDA_TRY(cudaEventRecord(s->tick_start, s->stream));
    // BH streams wait for the tick start so that latencies share one origin
    for (int k = 0; k < kBHStreams; ++k)
        NB_CUDA_TRY(cudaStreamWaitEvent(s->bh_streams[k], s->tick_start, 0));
    // Barnes-Hut jobs: the pool's thread of each busy stream issues that
    // stream's steps; this thread issues the direct batch meanwhile
    std::vector<std::vector<Job *>> per_stream(kBHStreams);
    for (Job *j : bh) per_stream[j->stream_index].push_back(j);
    auto run_stream = [&](int k) {
        for (Job *j : per_stream[k]) {
            nb_status r = nb_step(j->sim, NB_LEAPFROG, dt, 1);
            if (r == NB_OK) {
                const cudaError_t e = cudaEventRecord(j->step_done, s->bh_streams[k]);
                if (e != cudaSuccess) r = cuda_fail(e, "cudaEventRecord");
            }
            if (r != NB_OK) {  // this job alone fails; it is retired below
                j->status = r;
                j->error = nb_last_error();
            }
        }
    };
    std::vector<bool> busy(kBHStreams);
    for (int k = 0; k < kBHStreams; ++k) busy[k] = !per_stream[k].empty();
    s->pool_threads.dispatch(run_stream, busy);
    // wait for the stream threads even when the direct batch below fails
    struct Waiter {
        StreamPool &p;
        ~Waiter() { p.wait(); }
    } waiter{s->pool_threads};
    const auto t_direct = Clock::now();
    if (!direct.empty()) {
        float4 *hi = s->hi.as<float4>(), *lo = s->lo.as<float4>();
        if (!new_direct.empty()) {
            // start-of-step force of the jobs admitted this tick
            int nn = 0;
            NB_TRY(upload_systems(s, new_direct, s->d_new_sys, s->d_new_items, &nn));
            NB_TRY(split_positions(s->f[0], s->f[1], s->f[2], s->f[9], hw, hi, lo, s->stream));
            NB_TRY(batch_forces(hi, lo, s->d_new_sys.as<SysDesc>(), s->d_new_items.as<WorkItem>(),
                                nn, s->d_counter.as<int>(), s->cfg.G, eps2, s->f[6], s->f[7],
                                s->f[8], hw, s->stream));
        }
        NB_TRY(kick_drift(NB_LEAPFROG, hw, dt, s->f[0], s->f[1], s->f[2], s->f[3], s->f[4],
                          s->f[5], s->f[6], s->f[7], s->f[8], nullptr, nullptr, nullptr,
                          s->stream));
        NB_TRY(split_positions(s->f[0], s->f[1], s->f[2], s->f[9], hw, hi, lo, s->stream));
        NB_TRY(batch_forces(hi, lo, s->d_sys.as<SysDesc>(), s->d_items.as<WorkItem>(),
                            s->num_items, s->d_counter.as<int>(), s->cfg.G, eps2, s->f[6],
                            s->f[7], s->f[8], hw, s->stream));
        NB_TRY(kick(NB_LEAPFROG, hw, dt, s->f[3], s->f[4], s->f[5], s->f[6], s->f[7], s->f[8],
                    nullptr, nullptr, nullptr, s->stream));
        NB_CUDA_TRY(cudaEventRecord(s->direct_done, s->stream));
    }
    s->direct_ms += ms_since(t_direct);
    const auto t_join = Clock::now();
    s->pool_threads.wait();
    s->join_ms += ms_since(t_join);
    s->issue_ms += ms_since(t_phase);
    t_phase = Clock::now();
    NB_CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (int k = 0; k < kBHStreams; ++k) NB_CUDA_TRY(cudaStreamSynchronize(s->bh_streams[k]));
    s->wait_ms += ms_since(t_phase);
    float tick_ms = 0.f;
    if (!direct.empty()) {
        NB_CUDA_TRY(cudaEventElapsedTime(&tick_ms, s->tick_start, s->direct_done));
        for (Job *j : direct) {
            s->step_ms.push_back(tick_ms);
            s->interactions += (double)j->n * (double)(j->n - 1);
            ++j->done;
        }
    }
    for (Job *j : bh) {
        if (j->status != NB_OK) continue;
        float ms = 0.f;
        NB_CUDA_TRY(cudaEventElapsedTime(&ms, s->tick_start, j->step_done));
        tick_ms = std::max(tick_ms, ms);
        s->step_ms.push_back(ms);
        ++j->done;  // its interactions are read once, at retirement
    }
    s->busy_ms += tick_ms;
    s->steps_done += direct.size();
    for (Job *j : bh) s->steps_done += j->status == NB_OK;
    ++s->ticks;
    t_phase = Clock::now();
    const nb_status r = retire(s);
    s->retire_ms += ms_since(t_phase);
    return r;
}

} // namespace
} // namespace nb

using namespace nb;

extern "C" {

nb_status nb_server_config_default(nb_server_config *c)
{
    if (!c) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    c->G = 1.0;
    c->softening = 1e-3;
    c->theta = 0.6;
    c->leaf_capacity = 8;
    c->direct_max_n = 16384;
    c->dt = 1e-3;
    c->hbm_budget_bytes = (size_t)16 << 30;
    c->pool_bodies = (size_t)1 << 22;
    return NB_OK;
}

nb_status nb_server_create(const nb_server_config *cfg, nb_server **out)
{
    if (!cfg || !out) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (cfg->pool_bodies == 0 || cfg->pool_bodies > ((size_t)1 << 30))
        return fail(NB_ERR_INVALID_ARGUMENT, "pool_bodies must be in [1, 2^30]");
    if (kDirectBytesPerBody * cfg->pool_bodies > cfg->hbm_budget_bytes)
        return fail(NB_ERR_CAPACITY, "the direct-job pool alone exceeds the HBM budget");
    nb_server *s = new nb_server();
    s->cfg = *cfg;
    s->ps = (cfg->pool_bodies + 31) / 32 * 32;
    nb_status st = NB_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    for (int k = 0; k < kBHStreams && e == cudaSuccess; ++k)
        e = cudaStreamCreateWithFlags(&s->bh_streams[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&s->tick_start);
    if (e == cudaSuccess) e = cudaEventCreate(&s->direct_done);
    if (e != cudaSuccess) st = cuda_fail(e, "server streams/events");
    if (st == NB_OK) st = s->pool.reserve(sizeof(double) * 10 * s->ps);
    if (st == NB_OK) st = s->hi.reserve(sizeof(float4) * s->ps);
    if (st == NB_OK) st = s->lo.reserve(sizeof(float4) * s->ps);
    if (st == NB_OK) st = s->d_counter.reserve(sizeof(int));
    if (st == NB_OK) {
        e = cudaMemsetAsync(s->pool.ptr, 0, s->pool.bytes, s->stream);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMemsetAsync");
    }
    if (st != NB_OK) {
        nb_server_destroy(s);
        return st;
    }
    for (int k = 0; k < 10; ++k) s->f[k] = s->pool.as<double>() + k * s->ps;
    s->slots.init(cfg->pool_bodies);
    int device = 0;
    cudaGetDevice(&device);
    if (!s->pool_threads.start(kBHStreams, device)) {
        nb_server_destroy(s);
        return fail(NB_ERR_CUDA, "server: cannot start the Barnes-Hut stream threads");
    }
    s->peak_bytes = pool_bytes(s);
    *out = s;
    return NB_OK;
}

nb_status nb_server_destroy(nb_server *s)
{
    if (!s) return NB_OK;
    s->pool_threads.stop();
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (auto &j : s->running) {
        if (j->sim) nb_destroy(j->sim);
        if (j->step_done) cudaEventDestroy(j->step_done);
    }
    DevBuf *bufs[] = {&s->pool, &s->hi, &s->lo, &s->d_sys, &s->d_items, &s->d_counter,
                      &s->d_new_sys, &s->d_new_items};
    for (DevBuf *b : bufs) b->release();
    if (s->tick_start) cudaEventDestroy(s->tick_start);
    if (s->direct_done) cudaEventDestroy(s->direct_done);
    for (int k = 0; k < kBHStreams; ++k)
        if (s->bh_streams[k]) cudaStreamDestroy(s->bh_streams[k]);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return NB_OK;
}

nb_status nb_server_submit(nb_server *s, size_t n, const double *x, const double *y,
                           const double *z, const double *vx, const double *vy,
                           const double *vz, const double *m, int steps, int64_t *job_id)
{
    if (!s || !job_id) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0 || steps <= 0) return fail(NB_ERR_INVALID_ARGUMENT, "n and steps must be > 0");
    const double *src[7] = {x, y, z, vx, vy, vz, m};
    for (const double *p : src)
        if (!p) return fail(NB_ERR_INVALID_ARGUMENT, "NULL input array");
    const bool direct = (int64_t)n < (int64_t)s->cfg.direct_max_n;
    if (direct && n > s->cfg.pool_bodies)
        return fail(NB_ERR_CAPACITY, "direct job larger than the body pool");
    if (!direct && kBHBytesPerBody * n + pool_bytes(s) > s->cfg.hbm_budget_bytes)
        return fail(NB_ERR_CAPACITY, "job can never fit the HBM budget");
    auto j = std::make_unique<Job>();
    j->id = s->next_id++;
    j->n = n;
    j->steps = steps;
    j->direct = direct;
    j->init.resize(7 * n);
    for (int k = 0; k < 7; ++k) std::memcpy(j->init.data() + k * n, src[k], n * sizeof(double));
    j->submitted = Clock::now();
    *job_id = j->id;
    s->queue.push_back(std::move(j));
    ++s->submitted;
    return NB_OK;
}

nb_status nb_server_tick(nb_server *s, int *running, int *queued)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "server is NULL");
    NB_TRY(tick(s));
    if (running) *running = (int)s->running.size();
    if (queued) *queued = (int)s->queue.size();
    return NB_OK;
}

nb_status nb_server_result(nb_server *s, int64_t job_id, double *x, double *y, double *z,
                           double *vx, double *vy, double *vz, double *ax, double *ay,
                           double *az, double *m)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "server is NULL");
    auto it = s->finished.find(job_id);
    if (it == s->finished.end()) return fail(NB_ERR_NOT_LOADED, "job not finished (or unknown)");
    const Job *j = it->second.get();
    if (j->status != NB_OK) return fail(j->status, "job " + std::to_string(job_id) + ": " + j->error);
    double *dst[10] = {x, y, z, vx, vy, vz, ax, ay, az, m};
    for (int k = 0; k < 10; ++k)
        if (dst[k]) std::memcpy(dst[k], j->result.data() + k * j->n, j->n * sizeof(double));
    return NB_OK;
}

nb_status nb_server_release(nb_server *s, int64_t job_id)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "server is NULL");
    s->finished.erase(job_id);
    return NB_OK;
}

nb_status nb_server_cancel(nb_server *s, int64_t job_id)
{
    if (!s) return fail(NB_ERR_INVALID_ARGUMENT, "server is NULL");
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
        if ((*it)->id == job_id) {
            (*it)->status = NB_ERR_CANCELLED;
            (*it)->error = "cancelled while queued";
            std::vector<double>().swap((*it)->init);
            end_job(s, std::move(*it));
            s->queue.erase(it);
            return NB_OK;
        }
    for (auto it = s->running.begin(); it != s->running.end(); ++it)
        if ((*it)->id == job_id) {
            // between ticks every stream of the server is idle (a tick ends
            // with them synchronised), so the job's memory can go at once
            (*it)->status = NB_ERR_CANCELLED;
            (*it)->error = "cancelled after " + std::to_string((*it)->done) + " steps";
            drop_resources(s, it->get());
            end_job(s, std::move(*it));
            s->running.erase(it);
            return NB_OK;
        }
    return fail(NB_ERR_INVALID_ARGUMENT, s->finished.count(job_id)
                                             ? "job " + std::to_string(job_id) + " already finished"
                                             : "unknown job " + std::to_string(job_id));
}

nb_status nb_server_get_stats(nb_server *s, nb_server_stats *out)
{
    if (!s || !out) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    out->jobs_submitted = s->submitted;
    out->jobs_finished = s->submitted - s->queue.size() - s->running.size();
    out->jobs_running = (int)s->running.size();
    out->jobs_queued = (int)s->queue.size();
    out->steps_done = s->steps_done;
    out->ticks = s->ticks;
    out->interactions = s->interactions;
    out->busy_ms = s->busy_ms;
    out->step_ms_p50 = quantile(s->step_ms, 0.5);
    out->step_ms_p99 = quantile(s->step_ms, 0.99);
    out->queue_ms_p50 = quantile(s->queue_ms, 0.5);
    out->queue_ms_p99 = quantile(s->queue_ms, 0.99);
    out->max_running = s->max_running;
    out->peak_device_bytes = s->peak_bytes;
    out->host_admit_ms = s->admit_ms;
    out->host_issue_ms = s->issue_ms;
    out->host_wait_ms = s->wait_ms;
    out->host_retire_ms = s->retire_ms;
    out->host_upload_ms = s->upload_ms;
    out->host_direct_ms = s->direct_ms;
    out->host_join_ms = s->join_ms;
    out->jobs_failed = s->failed;
    out->jobs_cancelled = s->cancelled;
    return NB_OK;
}

} // extern "C"
