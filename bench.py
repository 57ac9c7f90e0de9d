#!/usr/bin/env python
"""Headline benchmark: mixed-precision all-pairs gravity on one GB300.

Workload (the mixed-precision direct configuration): N = 65,536 equal-mass
Plummer sphere (G = 1, M = 1, a = 1, virial velocities, generator seed 0),
softening 1e-3, velocity Verlet with dt = 5e-4.  One step = one velocity-Verlet
step of the engine (the force of the new positions plus the two half-updates;
the start-of-step force is the previous step's end force).  Interactions per
step = N (N - 1).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is device-timed: CUDA events around
each step on the simulation's stream, inputs resident in HBM, L2 flushed
(a 256 MiB write) before every timed step.  `e2e` is one force evaluation
through the public C ABI with pinned host buffers per step: nb_load (H2D of the
7 input arrays) + nb_compute_forces + nb_read_state of the 3 acceleration
arrays (D2H), wall clock.  `--impl reference` times the reference's CPU
direct sum (its C restatement, the only CPU build of it that exists on the
GPU host) on all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

# The serving extra runs its Barnes-Hut jobs on 16 streams; the CUDA runtime
# maps streams onto CUDA_DEVICE_MAX_CONNECTIONS hardware queues (8 by
# default), so give it as many before CUDA starts (a per-process setting).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

REPO = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(REPO, "n-body-gravity-simulation_gb300")
sys.path.insert(0, PKG_DIR)

METRIC = "Ginteractions/s direct + BH N=2^20 steps/s, mixed vs FP64 GPU at stated err"
UNIT = "Ginteractions/s"
N_BODIES = 65536
EPS = 1e-3
DT = 5e-4
SEED = 0
WORKLOAD = "plummer_n65536_mixed_direct_velocity_verlet"
FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_BODIES)
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="target CPU time of the cpu_baseline sample")
    ap.add_argument("--skip-extras", action="store_true",
                    help="only the headline value (no FP64 / accuracy / energy extras)")
    ap.add_argument("--bh-steps", type=int, default=20,
                    help="leapfrog steps of the Barnes-Hut N=2^20 extra (0 skips it)")
    ap.add_argument("--bh-n", type=int, default=1 << 20)
    ap.add_argument("--bh-variants", default="rebuild,reuse4,quad,refopen",
                    help="Barnes-Hut variants to run: rebuild every step (the configuration), "
                         "reuse4 (tree reuse every 4 evaluations), quad (quadrupoles), refopen "
                         "(the reference's opening rule, NB_FLAG_BH_REFERENCE_OPENING)")
    ap.add_argument("--ens-steps", type=int, default=25,
                    help="RK4 steps of the 4096-system ensemble extra (0 skips it)")
    ap.add_argument("--ens-systems", type=int, default=4096)
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="seconds of Poisson arrivals for the serving extra (0 skips it)")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--drift-steps", type=int, default=1000,
                    help="velocity-Verlet steps of the mixed vs FP64 energy-drift comparison "
                         "(0 skips it; the target is stated over 1000)")
    ap.add_argument("--no-bh-cpu", dest="bh_cpu", action="store_false",
                    help="skip the CPU Barnes-Hut evaluation of the Barnes-Hut extra")
    ap.add_argument("--no-ens-cpu", dest="ens_cpu", action="store_false",
                    help="skip the CPU RK4 sample of the ensemble extra")
    ap.add_argument("--only", choices=["bh", "ensemble", "serving"], default=None,
                    help="run one extra workload alone and print its record (profiling)")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw",
              "clocks_event_reasons.active", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device_index: int):
        self.samples = []
        self.proc = None
        self.dev = device_index
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "100", "-i", str(self.dev)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == len(self.FIELDS):
                self.samples.append((time.time(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0: float, t1: float):
        inside = [p for t, p in self.samples if t0 <= t <= t1]
        if not inside and self.samples:  # short region: nearest samples
            inside = [min(self.samples, key=lambda s: abs(s[0] - 0.5 * (t0 + t1)))[1]]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"],
                    "samples": 0}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(p[1]) for p in inside if num(p[1]) is not None]
        smax = [num(p[2]) for p in inside if num(p[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for p in inside for k in range(4)
                          if p[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(inside),
                "power_w_max": max((num(p[3]) or 0.0) for p in inside)}


# ---------------------------------------------------------------- helpers
def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)), "measured"
        except ValueError:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def profiled_traffic(name: str):
    """DRAM bytes per launch from an ncu summary in profiles/ (the
    `dram_bytes_per_launch:` line), or None."""
    p = os.path.join(REPO, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return int(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def fp32_roofline_gint(num_sms: int, mhz: float) -> float:
    """All-pairs roofline: 12 FP32-pipe operations per interaction (3 FADD for
    the displacement, 3 FFMA for r^2, 3 FMUL for m r^-3, 3 FFMA to accumulate)
    on 128 FP32 lanes per SM per clock; the one MUFU rsqrt per interaction
    (16/clk/SM) does not bind."""
    return num_sms * mhz * 1e6 * 128.0 / 12.0 / 1e9


def load_oracle():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    if not os.path.exists(O.LIB_PATH):
        O.build(with_ref=False)
    return O


def host_cpu():
    """The host CPU's model name and the number of threads the oracle uses."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None and os.path.exists("/proc/cpuinfo"):
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                model = line.split(":", 1)[1].strip()
                break
    return {"cpu_model": model or "unknown", "host_threads": os.cpu_count()}


def cpu_reference_rate(n, target_seconds, threads=0):
    """The reference's FP64 direct sum on the host cores (its C restatement),
    timed on a bounded sample of i-rows of the same workload.  The inputs come
    from the oracle's restatement of the engine's generator (the same bits), so
    this process never loads the engine library."""
    O = load_oracle()
    x, y, z, vx, vy, vz, m = O.plummer(n, seed=SEED)
    cores = O.threads() if threads == 0 else threads
    rows = 256
    t0 = time.perf_counter()
    O.forces_naive_rows(x, y, z, m, 1.0, EPS, 0, rows, threads)
    dt = max(time.perf_counter() - t0, 1e-6)
    rows = int(min(n, max(256, rows * target_seconds / dt)))
    return x, y, z, m, rows, cores, O


def run_plain(nb, torch, stream):
    """The reference's CPU-runnable configuration on the GPU: N = 1024 Plummer
    (seed 0), FP64 direct sum, softening 0.01, leapfrog KDK dt = 1e-3, 100
    steps (its parity with the oracle is a GPU test); CUDA events around the
    100 steps after one untimed run of the same configuration."""
    n, steps = 1024, 100
    state = nb.plummer(n, seed=SEED)
    cfg = nb.Config(method=nb.DIRECT_FP64, G=1.0, softening=0.01)
    out = {}
    for timed in (False, True):
        sim = nb.Sim(cfg, capacity=n, stream=stream.cuda_stream)
        sim.load(*state)
        e0 = sim.diagnostics()["total_softened"]
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        sim.step(nb.LEAPFROG, 1e-3, steps)
        ev1.record(stream)
        torch.cuda.synchronize()
        e1 = sim.diagnostics()["total_softened"]
        sim.close()
        if timed:
            ms = ev0.elapsed_time(ev1) / steps
            out = {"workload": "plummer_n1024_fp64_direct_leapfrog_100_steps", "n": n,
                   "steps": steps, "ms_per_step": ms, "steps_per_s": 1e3 / ms,
                   "ginteractions_s": n * (n - 1) / (ms / 1e3) / 1e9,
                   "energy_rel_change": (e1 - e0) / abs(e0)}
    # the reference's CPU path on the same configuration: its leapfrog
    # integrator with the direct sum (two force evaluations per step), the
    # whole 100-step run (C restatement, all host threads)
    O = load_oracle()
    t0 = time.perf_counter()
    O.run(O.LEAPFROG, O.DIRECT, *state, 1.0, 0.01, 1e-3, steps)
    el = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": steps / el, "unit": "steps/s", "kind": "port",
                           "cores": O.threads(), "ms_per_step": el / steps * 1e3,
                           "sample": f"the whole run: {steps} leapfrog steps of N = {n}, "
                                     "FP64 direct sum", **host_cpu()}
    out["speedup_vs_cpu"] = out["steps_per_s"] / out["cpu_baseline"]["value"]
    return out


def max_over_ranks(local_ms: float, world: int, torch, device) -> float:
    """The job's elapsed time: the maximum of the ranks' times (all ranks call)."""
    if world <= 1:
        return local_ms
    t = torch.tensor([local_ms], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank: float, job_ms: float, world: int) -> float:
    """Whole-job rate in G units/s: every replica processes units_per_rank."""
    return world * units_per_rank / (job_ms / 1e3) / 1e9


def energy_drift_pair(nb, n, steps, stream):
    """Relative drift of the softened total energy over `steps` velocity-Verlet
    steps of the bench workload, mixed path and FP64 path from the same start."""
    state = nb.plummer(n, seed=SEED)
    out = {"steps": steps, "dt": DT}
    for name, method in (("mixed", nb.DIRECT_MIXED), ("fp64", nb.DIRECT_FP64)):
        sim = nb.Sim(nb.Config(method=method, G=1.0, softening=EPS), capacity=n,
                     stream=stream.cuda_stream)
        sim.load(*state)
        e0 = sim.diagnostics()["total_softened"]
        sim.step(nb.VELOCITY_VERLET, DT, steps)
        e1 = sim.diagnostics()["total_softened"]
        sim.close()
        out[name] = (e1 - e0) / abs(e0)
    out["ratio_mixed_over_fp64"] = abs(out["mixed"]) / max(abs(out["fp64"]), 1e-300)
    return out


def pair_abs_sums(st, torch, tile=2048):
    """S_i = sum_j m_j |r_j - r_i| / (|r_j - r_i|^2 + eps^2)^(3/2) in FP64 on
    the GPU (torch), the error scale of any FP32 evaluation of a_i."""
    import numpy as np
    p = torch.from_numpy(np.stack([st["x"], st["y"], st["z"]], 1)).cuda()
    m = torch.from_numpy(np.ascontiguousarray(st["m"])).cuda()
    out = torch.empty(p.shape[0], dtype=torch.float64, device="cuda")
    for i0 in range(0, p.shape[0], tile):
        d = p[None, :, :] - p[i0:i0 + tile, None, :]
        r2 = (d * d).sum(-1)
        t = m[None, :] * torch.sqrt(r2) / (r2 + EPS * EPS) ** 1.5
        out[i0:i0 + tile] = t.sum(1)
        del d, r2, t
    return out.cpu().numpy()


def reference_gpu_kernel_rate(st, n, inter, mixed_rate, torch, stream):
    """The reference's own FP64 GPU kernel (computeAccelerationNaiveKernel,
    compiled for sm_103a from its source into oracle/_ref) on the same bodies,
    launched as ForceCalculatorNaive does; CUDA events around two launches."""
    import numpy as np
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ref_gpu
    if not ref_gpu.available():
        return {"unavailable": "reference cubin not built (no reference sources here)"}
    k = ref_gpu.RefNaiveKernel()
    dev = [torch.from_numpy(np.ascontiguousarray(st[c])).cuda() for c in ("x", "y", "z", "m")]
    acc = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    ptrs = [t.data_ptr() for t in dev[:3] + acc] + [dev[3].data_ptr()]
    torch.cuda.synchronize()
    k.launch(*ptrs, n, EPS * EPS, stream=stream.cuda_stream)  # warm
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 2
    e0.record(stream)
    for _ in range(reps):
        k.launch(*ptrs, n, EPS * EPS, stream=stream.cuda_stream)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    k.close()
    rate = inter / (ms / 1e3) / 1e9
    return {"value": rate, "unit": UNIT, "kind": "reference",
            "kernel": "computeAccelerationNaiveKernel (CUDA/src/force_calculator_naive.cu:4-59),"
                      " sm_103a cubin, ceil(N/256) x 256 threads",
            "kernel_ms": ms, "mixed_kernel_speedup": mixed_rate / rate}


# ---------------------------------------------------------------- reference arm
def run_reference(a, rank, world):
    if rank != 0:
        return 0
    n = a.n
    per_step = max(0.5, min(3.0, 60.0 / max(1, a.steps + a.warmup)))
    x, y, z, m, rows, cores, O = cpu_reference_rate(n, per_step)
    for _ in range(a.warmup):
        O.forces_naive_rows(x, y, z, m, 1.0, EPS, 0, rows)
    t0 = time.perf_counter()
    for k in range(a.steps):
        i0 = (k * rows) % max(1, n - rows + 1)
        O.forces_naive_rows(x, y, z, m, 1.0, EPS, i0, i0 + rows)
    elapsed = time.perf_counter() - t0
    inter = a.steps * rows * (n - 1)
    value = inter / elapsed / 1e9
    sample = (f"{rows} of {n} i-rows x all {n} j per step (FP64 direct sum, the hot loop of the "
              f"reference's CPU velocity-Verlet step), {a.steps} steps")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": elapsed / a.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": n, "softening": EPS, "dt": DT,
                   "integrator": "velocity_verlet", "method": "direct_fp64_cpu"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample, **host_cpu()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- Barnes-Hut
BH_N = 1 << 20
BH_THETA = 0.5
BH_DT = 1e-3


def run_bh(a, nb, torch, dev, stream, flush, np):
    """The Barnes-Hut configuration: N = 2^20 bulge (Plummer, 20% of the mass,
    scale 0.2) + exponential disk (scale length 1, height 0.05, circular
    velocities + 0.1 dispersion), 63-bit Morton octree, theta 0.5, eps 1e-3,
    FP32 walk / FP64 integration, leapfrog dt = 1e-3.  Reports steps/s over
    a.bh_steps leapfrog steps (CUDA events per step, L2 flushed before each),
    the walk kernel's share and rate, and the force error against the mixed
    direct sum; then the same with the tree rebuilt every 4 evaluations and
    refitted in between (NB_FLAG_BH_REUSE(4)), and with quadrupole moments
    (NB_FLAG_BH_QUADRUPOLE)."""
    n = a.bh_n
    state = nb.disk_bulge(n, seed=SEED)

    def timed(flags):
        cfg = nb.Config(method=nb.BARNES_HUT, G=1.0, softening=EPS, theta=BH_THETA,
                        leaf_capacity=8, flags=flags)
        sim = nb.Sim(cfg, capacity=n, stream=stream.cuda_stream)
        sim.load(*state)
        for _ in range(3):
            sim.step(nb.LEAPFROG, BH_DT, 1)
        torch.cuda.synchronize()
        ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(a.bh_steps)]
        ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(a.bh_steps)]
        sim.profile(True)
        sim.profile_read(reset=True)
        for k in range(a.bh_steps):
            flush.zero_()
            ev0[k].record(stream)
            sim.step(nb.LEAPFROG, BH_DT, 1)
            ev1[k].record(stream)
        torch.cuda.synchronize()
        prof = sim.profile_read(reset=True)
        sim.profile(False)
        step_ms = [e0.elapsed_time(e1) for e0, e1 in zip(ev0, ev1)]
        info = sim.bh_info()
        inter = info["interactions_m2p"] + info["interactions_p2p"]
        walk_ms = prof["force_kernel_ms"] / max(1, prof["force_launches"])
        ms = sum(step_ms) / len(step_ms)
        out = {"ms_per_step": ms, "steps_per_s": 1e3 / ms,
               "walk_ms": walk_ms, "walk_share": walk_ms / ms,
               "interactions_per_body": inter / n,
               "m2p_per_body": info["interactions_m2p"] / n,
               "p2p_per_body": info["interactions_p2p"] / n,
               "walk_ginteractions_s": inter / (walk_ms / 1e3) / 1e9,
               "nodes": info["num_nodes"], "leaves": info["num_leaves"],
               "max_depth": info["max_depth"]}
        # accuracy of the last evaluation vs the mixed direct sum (itself
        # within ~1e-6 of FP64)
        st = sim.read_state()
        bh_acc = (st["ax"], st["ay"], st["az"])
        ref = nb.Sim(nb.Config(method=nb.DIRECT_MIXED, G=1.0, softening=EPS), capacity=n,
                     stream=stream.cuda_stream)
        ref.load(st["x"], st["y"], st["z"], st["vx"], st["vy"], st["vz"], st["m"])
        ref.compute_forces()
        ra = ref.accelerations()
        ref.close()
        sim.close()
        d = np.sqrt(sum((u - v) ** 2 for u, v in zip(bh_acc, ra)))
        r = np.sqrt(sum(v * v for v in ra))
        rel = d / np.maximum(r, 1e-300)
        out["force_error_vs_direct"] = {"mean_rel": float(rel.mean()),
                                        "max_rel": float(rel.max()),
                                        "p99_rel": float(np.quantile(rel, 0.99))}
        return out

    variants = set(a.bh_variants.split(","))
    out = {"workload": f"disk_bulge_n{n}_theta{BH_THETA}_leapfrog", "n": n,
           "steps": a.bh_steps}
    if "rebuild" in variants:
        out.update(timed(0))
        out["timing"] = ("CUDA events per leapfrog step, L2 flushed before each; a build "
                         "reads the node count on the host once per step")
    keys = ("ms_per_step", "steps_per_s", "walk_ms", "interactions_per_body",
            "force_error_vs_direct")
    if "reuse4" in variants:
        reuse = timed(nb.bh_reuse_flag(4))
        out["tree_reuse_4"] = {k: reuse[k] for k in keys}
    if "quad" in variants:
        quad = timed(nb.BH_QUADRUPOLE)
        out["quadrupole"] = {k: quad[k] for k in keys}
    if "refopen" in variants:
        ro = timed(nb.BH_REFERENCE_OPENING)
        out["reference_opening_rule"] = {k: ro[k] for k in keys}
    if a.bh_cpu:
        out["cpu_baseline"] = bh_cpu_baseline(state, out.get("ms_per_step"))
    return out


def bh_cpu_baseline(state, gpu_ms_per_step):
    """The reference's CPU Barnes-Hut (ForceCalculatorBarnesHutOptimized, leaf
    capacity 8, theta 0.5: its C restatement, serial build + walk over all host
    threads) timed on one force evaluation of the same bodies."""
    O = load_oracle()
    x, y, z, m = state[0], state[1], state[2], state[6]
    t0 = time.perf_counter()
    O.forces_bh_opt(x, y, z, m, 1.0, EPS, BH_THETA, 8)
    el = time.perf_counter() - t0
    out = {"value": 1.0 / el, "unit": "force evaluations/s", "kind": "port",
           "cores": O.threads(), "s_per_eval": el,
           "sample": f"one force evaluation of all {len(x)} bodies (node-pool tree, leaf 8, "
                     f"theta {BH_THETA})", **host_cpu()}
    if gpu_ms_per_step:
        out["gpu_step_speedup"] = el / (gpu_ms_per_step / 1e3)
    return out


# ---------------------------------------------------------------- ensemble
def run_ensemble(a, nb, torch, stream):
    """The batched-ensemble configuration: 4096 Plummer spheres (system s
    seeded with s), N log-uniform in [32, 4096], mixed direct forces, RK4
    dt = 1e-3; a.ens_steps steps replayed from the captured CUDA graph, timed
    with events around the whole loop (4 force evaluations per step)."""
    sizes = nb.ensemble_sizes(a.ens_systems, 32, 4096, SEED)
    state = nb.plummer_ensemble(sizes, seed=SEED)
    # graph capture needs a stream of its own (not the legacy default stream)
    stream = torch.cuda.Stream()
    e = nb.Ensemble(nb.Config(method=nb.DIRECT_MIXED, G=1.0, softening=EPS), sizes,
                    stream=stream.cuda_stream)
    e.load(*state)
    e.step(nb.RK4, 1e-3, 2 * 25)  # tunes, captures the graph, warms up
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    e.step(nb.RK4, 1e-3, a.ens_steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / a.ens_steps
    info = e.info()
    # the force kernel alone, timed per launch (steps without the graph)
    e.profile(True)
    e.step(nb.RK4, 1e-3, 2)
    pinfo = e.info()
    e.close()
    inter = info["interactions_per_eval"]
    kernel_ms = pinfo["force_kernel_ms"] / max(1, pinfo["force_launches"])
    cpu = ensemble_cpu_baseline(a, sizes, state, inter, ms) if a.ens_cpu else None
    return {"workload": f"{a.ens_systems}_plummer_systems_n32_4096_rk4",
            "systems": a.ens_systems, "bodies": int(sizes.sum()),
            "interactions_per_eval": inter, "steps": a.ens_steps, "ms_per_step": ms,
            "ginteractions_s": 4 * inter / (ms / 1e3) / 1e9,
            "force_kernel_ms": kernel_ms,
            "force_kernel_ginteractions_s": inter / (kernel_ms / 1e3) / 1e9,
            "work_items": info["work_items"], "graph_steps_per_replay": info["graph_steps"],
            "ipt_by_bucket": {str(b): info["ipt_by_bucket"][b] for b in range(5, 13)},
            "timing": "CUDA events around the graph-replayed step loop",
            "cpu_baseline": cpu}


def ensemble_cpu_baseline(a, sizes, state, inter, gpu_ms_per_step):
    """The reference's CPU RK4 integrator with the direct sum (four force
    evaluations per step; its C restatement over all host threads): one step of
    every k-th system, k chosen so that the sample holds about a.cpu_seconds of
    work, scaled to the whole ensemble by its sum of N (N - 1)."""
    import numpy as np
    O = load_oracle()
    offs = np.concatenate([[0], np.cumsum(sizes)])
    per_sys = sizes.astype(np.float64) * (sizes - 1)
    # calibrate on the largest system
    big = int(np.argmax(sizes))
    sl = slice(int(offs[big]), int(offs[big + 1]))
    t0 = time.perf_counter()
    O.run(O.RK4, O.DIRECT, *(v[sl] for v in state), 1.0, EPS, 1e-3, 1)
    rate = 4 * per_sys[big] / max(time.perf_counter() - t0, 1e-6)
    want = rate * a.cpu_seconds / 4.0
    stride = max(1, int(np.ceil(per_sys.sum() / max(want, 1.0))))
    picked = list(range(0, len(sizes), stride))
    t0 = time.perf_counter()
    for s_ in picked:
        sl = slice(int(offs[s_]), int(offs[s_ + 1]))
        O.run(O.RK4, O.DIRECT, *(v[sl] for v in state), 1.0, EPS, 1e-3, 1)
    el = time.perf_counter() - t0
    done = 4 * per_sys[picked].sum()
    gint = done / el / 1e9
    full_step_s = 4 * inter / (gint * 1e9)
    return {"value": gint, "unit": UNIT, "kind": "port", "cores": O.threads(),
            "sample": f"one RK4 step of every {stride}-th system ({len(picked)} of {len(sizes)}"
                      f" systems, {done:.3g} interactions), FP64 direct sum",
            "full_ensemble_s_per_step": full_step_s,
            "gpu_step_speedup": full_step_s / (gpu_ms_per_step / 1e3), **host_cpu()}


# ---------------------------------------------------------------- serving
def run_serving(a, nb, np):
    """The serving configuration, shortened: Poisson arrivals at a.serve_rate
    jobs/s for a.serve_seconds of wall time, N log-uniform in [1024, 262144],
    Plummer or disk+bulge (alternating), 100 leapfrog steps each, direct below
    16384 bodies and Barnes-Hut theta 0.6 above; the server admits by HBM
    budget and ticks until drained."""
    rng = np.random.default_rng(SEED)
    t_arr, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / a.serve_rate)
        if t > a.serve_seconds:
            break
        t_arr.append(t)
    sizes = np.floor(np.exp(rng.uniform(np.log(1024), np.log(262145), len(t_arr)))).astype(int)
    jobs = [(nb.plummer(int(n), seed=k) if k % 2 == 0 else nb.disk_bulge(int(n), seed=k))
            for k, n in enumerate(sizes)]
    srv = nb.Server(theta=0.6, softening=EPS, dt=1e-3, hbm_budget_bytes=64 << 30,
                    pool_bodies=1 << 21)
    t0 = time.perf_counter()
    k = 0
    while True:
        now = time.perf_counter() - t0
        while k < len(jobs) and t_arr[k] <= now:
            srv.submit(jobs[k], 100)
            k += 1
        r, q = srv.tick()
        if k == len(jobs) and r == 0 and q == 0:
            break
        if r == 0 and q == 0 and k < len(jobs):
            time.sleep(max(0.0, min(0.01, t_arr[k] - now)))
        if time.perf_counter() - t0 > a.serve_seconds + 300:
            break
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    return {"workload": "poisson_jobs_n1024_262144_100_leapfrog_steps",
            "rate_per_s": a.serve_rate, "arrival_seconds": a.serve_seconds,
            "jobs": len(jobs), "direct_jobs": int((sizes < 16384).sum()),
            "jobs_finished": st["jobs_finished"], "wall_s": wall,
            "step_ms_p50": st["step_ms_p50"], "step_ms_p99": st["step_ms_p99"],
            "queue_ms_p50": st["queue_ms_p50"], "queue_ms_p99": st["queue_ms_p99"],
            "ginteractions_s": st["interactions"] / wall / 1e9,
            "device_busy_fraction": st["busy_ms"] / 1e3 / wall,
            "max_running": st["max_running"], "peak_device_gb": st["peak_device_bytes"] / 1e9,
            "host_s": {"admit": st["host_admit_ms"] / 1e3, "issue": st["host_issue_ms"] / 1e3,
                       "wait": st["host_wait_ms"] / 1e3, "retire": st["host_retire_ms"] / 1e3,
                       "issue_upload": st["host_upload_ms"] / 1e3,
                       "issue_direct": st["host_direct_ms"] / 1e3,
                       "issue_join": st["host_join_ms"] / 1e3},
            "ticks": st["ticks"]}


# ---------------------------------------------------------------- our arm
def run_ours(a, rank, world, local_rank):
    import numpy as np
    import torch
    import nbody_gb300 as nb

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream(dev)
    n = a.n
    inter = n * (n - 1)
    state = nb.plummer(n, seed=SEED)
    cfg = nb.Config(method=nb.DIRECT_MIXED, G=1.0, softening=EPS)
    sim = nb.Sim(cfg, capacity=n, stream=stream.cuda_stream)
    sim.load(*state)
    e_start = None if a.skip_extras else sim.diagnostics()

    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(a.warmup):
        sim.step(nb.VELOCITY_VERLET, DT, 1)
    torch.cuda.synchronize()

    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sim.profile(True)
    sim.profile_read(reset=True)
    launches0 = nb.kernel_launch_count()
    t_wall0 = time.time()
    for k in range(a.steps):
        flush.zero_()
        ev0[k].record(stream)
        sim.step(nb.VELOCITY_VERLET, DT, 1)
        ev1[k].record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.time()
    launches = nb.kernel_launch_count() - launches0
    prof = sim.profile_read(reset=True)
    sim.profile(False)
    clocks.stop()
    step_ms = [e0.elapsed_time(e1) for e0, e1 in zip(ev0, ev1)]
    total_ms = max_over_ranks(sum(step_ms), world, torch, dev)
    value = replica_rate(a.steps * inter, total_ms, world)
    # the evolved state, before the end-to-end loop below reloads the start
    e_end = None if a.skip_extras else sim.diagnostics()
    evolved = None if a.skip_extras else sim.read_state()

    # e2e: the same force evaluation through the C ABI with pinned host buffers
    # (H2D of the inputs and D2H of the accelerations every step), every rank,
    # max wall time over ranks
    host = [torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for v in state]
    outs = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(3)]
    ptr_in = [h.data_ptr() for h in host]
    ptr_out = [0] * 6 + [o.data_ptr() for o in outs] + [0]
    for _ in range(max(1, a.warmup)):
        sim.load_pointers(n, ptr_in)
        sim.compute_forces()
        sim.read_pointers(ptr_out)
    ke = min(a.steps, 200)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        sim.load_pointers(n, ptr_in)
        sim.compute_forces()
        sim.read_pointers(ptr_out)
    el_ms = max_over_ranks((time.perf_counter() - t0) * 1e3, world, torch, dev)
    e2e = {"value": replica_rate(ke * inter, el_ms, world), "unit": UNIT,
           "h2d_bytes_per_step": 7 * 8 * n, "d2h_bytes_per_step": 3 * 8 * n,
           "step": "nb_load (7 FP64 arrays) + nb_compute_forces + nb_read_state "
                   "(3 acceleration arrays), pinned host memory, wall clock"}

    # roofline of the dominant kernel (the all-pairs kernel)
    props = torch.cuda.get_device_properties(local_rank)
    peaks, peak_kind = measured_peaks()
    kernel_ms = prof["force_kernel_ms"] / max(1, prof["force_launches"])
    achieved = inter / (kernel_ms / 1e3) / 1e9
    clk = clocks.summary(t_wall0, t_wall1)
    peak = fp32_roofline_gint(props.multi_processor_count, peaks.get("sm_max_mhz", 2070.0))
    roofline = {
        "bound": "fp32",
        "kernel": "direct_sorted_kernel" if n >= 16384 else "direct_mixed_kernel",
        "achieved": achieved,
        "peak": peak, "unit": "Ginteractions/s", "frac": achieved / peak,
        "peak_basis": (f"{props.multi_processor_count} SMs x {peaks.get('sm_max_mhz', 2070.0)}"
                       f" MHz ({peak_kind} sm_max_mhz) x 128 FP32 lanes / 12 FP32 ops per "
                       "interaction"),
        "traffic": None,
        "kernel_ms": kernel_ms,
    }
    if clk.get("sm_mhz"):
        roofline["frac_at_measured_clock"] = achieved / fp32_roofline_gint(
            props.multi_processor_count, clk["sm_mhz"])
    # the same fraction in FP32-pipe operations per second (12 per interaction)
    roofline["achieved_fp32_tops"] = achieved * 12.0 / 1e3
    roofline["peak_fp32_tops"] = peak * 12.0 / 1e3
    roofline["traffic"] = profiled_traffic("direct_sorted_n65536.md") if n == N_BODIES else None
    roofline["algorithmic_bytes"] = 32 * n  # hi + lo mirror of every body, read once
    # the same kernel against a measured FP32-pipe rate (packed FMAs on every
    # SM, register-only probe), beside the lanes x clock peak above
    fma_rate = nb.debug_fp32_rate()
    roofline["peak_measured_fp32"] = {
        "value": fma_rate / 12.0 / 1e9, "unit": "Ginteractions/s",
        "frac": achieved / (fma_rate / 12.0 / 1e9), "fma_lane_tops": fma_rate / 1e12,
        "basis": "nb_debug_fp32_rate (independent packed FMAs, best of 3 launches) / 12"}

    extras = {}
    if not a.skip_extras and rank == 0:
        extras["energy_drift"] = {
            "steps": a.warmup + a.steps,
            "rel": (e_end["total_softened"] - e_start["total_softened"]) /
                   abs(e_start["total_softened"]),
            "note": "softened total energy, FP64 GPU reduction, mixed-precision run"}
        # accuracy and speed of the mixed kernel vs the FP64 kernel on the
        # current state (the FP64 path is pinned to the CPU oracle at 1e-12 by
        # the tests)
        st = evolved
        sim.load(st["x"], st["y"], st["z"], st["vx"], st["vy"], st["vz"], st["m"])
        sim.compute_forces()
        mixed_acc = sim.accelerations()
        ref = nb.Sim(nb.Config(method=nb.DIRECT_FP64, G=1.0, softening=EPS), capacity=n,
                     stream=stream.cuda_stream)
        ref.load(st["x"], st["y"], st["z"], st["vx"], st["vy"], st["vz"], st["m"])
        ref.compute_forces()  # warm
        ref.profile(True)
        ref.profile_read(reset=True)
        ref.compute_forces()
        p64 = ref.profile_read(reset=True)
        ref_acc = ref.accelerations()
        ref.close()
        d = np.sqrt(sum((u - v) ** 2 for u, v in zip(mixed_acc, ref_acc)))
        r = np.sqrt(sum(v * v for v in ref_acc))
        rel = d / np.maximum(r, 1e-300)
        fp64_rate = inter / (p64["force_kernel_ms"] / 1e3) / 1e9
        sabs = pair_abs_sums(st, torch)
        kappa = sabs / np.maximum(r, 1e-300)
        well = kappa <= 10.0
        extras["force_error_vs_fp64"] = {
            "max_rel": float(rel.max()),
            "rms_rel": float(np.sqrt(np.mean(rel * rel))),
            "max_abs_over_rms_a": float(d.max() / np.sqrt(np.mean(r * r))),
            "max_rel_kappa_le_10": float(rel[well].max(initial=0.0)),
            "max_err_over_abs_sum": float((d / np.maximum(sabs, 1e-300)).max()),
            "kappa_at_max_rel": float(kappa[rel.argmax()]),
            "bodies_kappa_gt_10": int((~well).sum()),
            "note": ("kappa = sum_j |pair term| / |a|: a body whose force nearly cancels "
                     "(large kappa) carries a relative error ~kappa x that of its terms")}
        extras["fp64_direct"] = {"gint_s": fp64_rate, "kernel": "direct_fp64_kernel",
                                 "mixed_speedup": achieved / fp64_rate}
        extras["gpu_baseline"] = reference_gpu_kernel_rate(st, n, inter, achieved, torch,
                                                           stream)
        if a.drift_steps > 0:
            extras["energy_drift_vs_fp64"] = energy_drift_pair(nb, n, a.drift_steps, stream)
        extras["plain_fp64_n1024"] = run_plain(nb, torch, stream)

    if not a.skip_extras and rank == 0 and a.bh_steps > 0:
        extras["barnes_hut"] = run_bh(a, nb, torch, dev, stream, flush, np)
    if not a.skip_extras and rank == 0 and a.ens_steps > 0:
        extras["ensemble"] = run_ensemble(a, nb, torch, stream)
    if not a.skip_extras and rank == 0 and a.serve_seconds > 0:
        extras["serving"] = run_serving(a, nb, np)

    cpu = None
    if rank == 0 and not a.skip_extras:
        x, y, z, m, rows, cores, O = cpu_reference_rate(n, a.cpu_seconds)
        t0 = time.perf_counter()
        O.forces_naive_rows(x, y, z, m, 1.0, EPS, 0, rows)
        el = time.perf_counter() - t0
        cpu = {"value": rows * (n - 1) / el / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"FP64 direct sum of the reference (C restatement), {rows} of {n} "
                         f"i-rows x all {n} j, one pass", **host_cpu()}
    sim.close()
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": total_ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+ds/f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": n, "softening": EPS, "dt": DT, "G": 1.0,
                   "integrator": "velocity_verlet", "method": "direct_mixed",
                   "parallelism": "replicas" if world > 1 else "single_gpu",
                   "l2": "flushed (256 MiB write) before every timed step",
                   "timing": "CUDA events per step on the simulation stream"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
    }
    line.update(extras)
    line["summary"] = summarize(line)
    print(json.dumps(line), flush=True)
    return 0


def summarize(line):
    """The figures a reader looks for first, repeated at the end of the line."""
    def get(*keys):
        v = line
        for k in keys:
            if not isinstance(v, dict) or k not in v or v[k] is None:
                return None
            v = v[k]
        return v
    return {
        "gint_s": line["value"], "e2e_gint_s": get("e2e", "value"),
        "roofline_frac": get("roofline", "frac"),
        "force_err_max_rel": get("force_error_vs_fp64", "max_rel"),
        "force_err_rms_rel": get("force_error_vs_fp64", "rms_rel"),
        "mixed_over_fp64_gpu": get("fp64_direct", "mixed_speedup"),
        "mixed_over_reference_gpu_kernel": get("gpu_baseline", "mixed_kernel_speedup"),
        "drift_ratio_mixed_over_fp64": get("energy_drift_vs_fp64", "ratio_mixed_over_fp64"),
        "drift_steps": get("energy_drift_vs_fp64", "steps"),
        "bh_steps_per_s": get("barnes_hut", "steps_per_s"),
        "bh_cpu_s_per_eval": get("barnes_hut", "cpu_baseline", "s_per_eval"),
        "ensemble_gint_s": get("ensemble", "ginteractions_s"),
        "serving_p50_p99_ms": [get("serving", "step_ms_p50"), get("serving", "step_ms_p99")],
        "serving_gint_s": get("serving", "ginteractions_s"),
        "cpu_baseline_gint_s": get("cpu_baseline", "value"),
    }


def run_only(a, local_rank):
    import numpy as np
    import torch
    import nbody_gb300 as nb
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    if a.only == "bh":
        flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
        rec = run_bh(a, nb, torch, dev, stream, flush, np)
    elif a.only == "ensemble":
        rec = run_ensemble(a, nb, torch, stream)
    else:
        rec = run_serving(a, nb, np)
    print(json.dumps({a.only: rec}), flush=True)
    return 0


def main():
    a = parse()
    rank, world, local_rank = dist_env()
    if a.impl == "reference":
        return run_reference(a, rank, world)
    if a.only:
        return run_only(a, local_rank)
    return run_ours(a, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
