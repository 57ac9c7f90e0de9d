"""Regenerates the golden fixtures in this folder from the reference checkout.

    REF_ROOT=/root/reference python tests/golden/make_golden.py

Reads only the reference's published outputs (never its sources):
  - CPU/outputs/output2_4.txt: the seed-42 force-benchmark error tables of
    CPU/tests/test2_ForceBenchmark.cpp (5 runs x N in {100,500,1000,5000,10000},
    pointer Barnes-Hut and node-pool Barnes-Hut vs the direct sum, theta 0.5,
    leaf 8, no softening) -> force_benchmark_seed42.json
  - CPU/orbit.csv: the Earth-Sun trajectory written by CPU/src/n-body.cpp
    (pointer Barnes-Hut theta 0.3, velocity Verlet, dt = 1/365, 366 steps)
    -> orbit_earth_sun.csv (every 5th row and the last one)
  - CUDA/outputs/output1_2.txt: the GPU Barnes-Hut accuracy envelope
    -> cuda_bh_envelope.json
and, with the host C++ compiler, the first draws of std::mt19937(42) and of
std::uniform_real_distribution<double> -> mt19937_seed42.json.
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("REF_ROOT", "/root/reference")


def force_tables():
    path = os.path.join(REF, "CPU", "outputs", "output2_4.txt")
    runs = []
    cur_run = None
    n = None
    section = None
    for line in open(path):
        line = line.strip()
        m = re.match(r"Run : (\d+)", line)
        if m:
            cur_run = {"run": int(m.group(1)), "cases": []}
            runs.append(cur_run)
            continue
        m = re.match(r"Number of Particles : (\d+)", line)
        if m:
            n = int(m.group(1))
            cur_run["cases"].append({"n": n, "bh": {}, "bh_opt": {}})
            continue
        if line == "Barnes-Hut":
            section = "bh"
        elif line == "Barnes-Hut Optimized":
            section = "bh_opt"
        m = re.match(r"(Average|Maximum) (Absolute|Relative) Error : ([0-9.eE+-]+)", line)
        if m and section:
            key = ("avg" if m.group(1) == "Average" else "max") + "_" + \
                  ("abs" if m.group(2) == "Absolute" else "rel")
            cur_run["cases"][-1][section][key] = float(m.group(3))
    return {
        "source": "CPU/outputs/output2_4.txt",
        "generator": "CPU/tests/test2_ForceBenchmark.cpp: std::mt19937 rng(42) shared by all "
                     "runs and N; positions U(-100,100), masses U(0.5,2); G = 4 pi^2; "
                     "softening 0; theta 0.5; leaf capacity 8",
        "printed_digits": 6,
        "runs": runs,
    }


def orbit():
    path = os.path.join(REF, "CPU", "orbit.csv")
    lines = open(path).read().strip().splitlines()
    header, rows = lines[0], lines[1:]
    keep = [(i, r) for i, r in enumerate(rows) if i % 5 == 0 or i == len(rows) - 1]
    with open(os.path.join(HERE, "orbit_earth_sun.csv"), "w") as f:
        f.write("row," + header + "\n")
        for i, r in keep:
            f.write(f"{i},{r}\n")


def cuda_envelope():
    path = os.path.join(REF, "CUDA", "outputs", "output1_2.txt")
    out = []
    n = None
    for line in open(path):
        m = re.match(r"Particles : (\d+)", line.strip())
        if m:
            n = int(m.group(1))
            out.append({"n": n})
        m = re.match(r"(Average|Maximum) (Absolute|Relative) Error : ([0-9.eE+-]+)",
                     line.strip())
        if m and out:
            key = ("avg" if m.group(1) == "Average" else "max") + "_" + \
                  ("abs" if m.group(2) == "Absolute" else "rel")
            out[-1][key] = float(m.group(3))
    return {"source": "CUDA/outputs/output1_2.txt",
            "note": "reference GPU Barnes-Hut (FP32 walk, theta 0.5, leaf 8) vs its FP64 "
                    "direct kernel, uniform cube seed 42, two runs",
            "cases": out}


MT_PROGRAM = r"""
#include <cstdio>
#include <random>
int main() {
    std::mt19937 g(42);
    for (int i = 0; i < 8; ++i) std::printf("%u\n", (unsigned)g());
    std::mt19937 h(42);
    std::uniform_real_distribution<double> u(-100.0, 100.0);
    for (int i = 0; i < 8; ++i) std::printf("%.17g\n", u(h));
    return 0;
}
"""


def mt_fixture():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "mt.cpp")
        exe = os.path.join(d, "mt")
        open(src, "w").write(MT_PROGRAM)
        subprocess.run(["g++", "-O2", "-o", exe, src], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    return {"engine": "std::mt19937(42)", "u32": [int(v) for v in out[:8]],
            "uniform_m100_100": [float(v) for v in out[8:16]]}


def main():
    with open(os.path.join(HERE, "force_benchmark_seed42.json"), "w") as f:
        json.dump(force_tables(), f, indent=1)
    orbit()
    with open(os.path.join(HERE, "cuda_bh_envelope.json"), "w") as f:
        json.dump(cuda_envelope(), f, indent=1)
    with open(os.path.join(HERE, "mt19937_seed42.json"), "w") as f:
        json.dump(mt_fixture(), f, indent=1)


if __name__ == "__main__":
    main()
