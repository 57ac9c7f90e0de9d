#!/usr/bin/env bash
# Builds the two CPU checkers used by the tests (test infrastructure only):
#   oracle/liboracle.so   -- the C restatement (nbody_oracle.c); builds anywhere.
#   oracle/_ref/libnbref.so -- the reference's own CPU sources, compiled where they
#                            lie (REF_ROOT, default /root/reference) with the shim
#                            ref_shim.cpp.  Skipped when the sources are absent.
# Both use -ffp-contract=off so that no multiply-add is fused on any host.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
CC="${CC:-gcc}"
CXX="${CXX:-g++}"

"$CC" -std=c11 -O3 -fopenmp -ffp-contract=off -fPIC -shared -Wall -Wextra \
    -o "$HERE/liboracle.so.tmp" "$HERE/nbody_oracle.c" -lm
mv -f "$HERE/liboracle.so.tmp" "$HERE/liboracle.so"

if [[ "${1:-}" == "--no-ref" ]]; then exit 0; fi
SRC="$REF_ROOT/CPU/src"
if [[ ! -d "$SRC" ]]; then
    echo "build_ref: reference sources not found at $SRC; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
REF_SOURCES=(
    "$SRC/force_calculator_naive.cpp"
    "$SRC/force_calculator_barnes_hut.cpp"
    "$SRC/force_calculator_barnes_hut_optimized.cpp"
    "$SRC/integrator_euler.cpp"
    "$SRC/integrator_euler-cromer.cpp"
    "$SRC/integrator_leapfrog.cpp"
    "$SRC/integrator_velocity_verlet.cpp"
    "$SRC/integrator_rk4.cpp"
)
"$CXX" -std=c++23 -O3 -fopenmp -ffp-contract=off -fPIC -shared -w \
    -I"$REF_ROOT/CPU/include" -o "$HERE/_ref/libnbref.so.tmp" \
    "$HERE/ref_shim.cpp" "${REF_SOURCES[@]}"
mv -f "$HERE/_ref/libnbref.so.tmp" "$HERE/_ref/libnbref.so"
# where the reference lies, for the tests that read its fixtures and programs
printf '%s\n' "$REF_ROOT" > "$HERE/_ref/ref_root.txt"

# The reference's FP64 GPU kernel (computeAccelerationNaiveKernel,
# CUDA/src/force_calculator_naive.cu:4-59) as a standalone sm_103a cubin, compiled
# where it lies with the reference Makefile's flags (-std=c++17 -O3) and the
# architecture switched to sm_103a.  Device code only: it carries no host code,
# so it runs on any sm_103a host (x86 or Arm); ref_gpu.py loads it with the CUDA driver API.
CUDA_SRC="$REF_ROOT/CUDA/src/force_calculator_naive.cu"
NVCC="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
if [[ -f "$CUDA_SRC" && -x "$NVCC" ]]; then
    "$NVCC" -std=c++17 -O3 -cubin -gencode arch=compute_103a,code=sm_103a \
        -I"$REF_ROOT/CUDA/include" -o "$HERE/_ref/ref_naive_sm103a.cubin.tmp" "$CUDA_SRC"
    mv -f "$HERE/_ref/ref_naive_sm103a.cubin.tmp" "$HERE/_ref/ref_naive_sm103a.cubin"
fi
