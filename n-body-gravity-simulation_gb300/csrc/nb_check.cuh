// nb_check.cuh -- device-side index checks of a checked build.
//
// compute-sanitizer is not available where this engine is tested, so a build
// with -DNB_DEVICE_CHECKS=1 (build.py --checks) makes the kernels test the
// indices they are about to use against their bounds.  A failed test records
// the first failure of its translation unit (source line, index, bound) in a
// device status word and the kernel skips the access: no trap, no hang.
// nb_debug_device_checks() reads and clears every unit's word.  In the normal
// build NB_IN_RANGE is the constant true and costs nothing.
#pragma once

#ifndef NB_DEVICE_CHECKS
#define NB_DEVICE_CHECKS 0
#endif

#include "nb_internal.h"

namespace nb {

#if NB_DEVICE_CHECKS
namespace {
__device__ DeviceCheck g_check;  // this translation unit's status word

__device__ __noinline__ bool record_check(long long i, long long n, int line)
{
    if (atomicCAS(&g_check.failed, 0, 1) == 0) {
        g_check.line = line;
        g_check.index = i;
        g_check.bound = n;
    }
    return false;
}

nb_status read_check(DeviceCheck *out, bool clear)
{
    NB_CUDA_TRY(cudaMemcpyFromSymbol(out, g_check, sizeof(DeviceCheck)));
    if (clear) {
        const DeviceCheck zero{};
        NB_CUDA_TRY(cudaMemcpyToSymbol(g_check, &zero, sizeof(DeviceCheck)));
    }
    return NB_OK;
}

struct CheckRegistrar {
    CheckRegistrar() { register_check_reader(__BASE_FILE__, &read_check); }
} g_check_registrar;
} // namespace

#define NB_IN_RANGE(i, n)                                                               \
    ((unsigned long long)(long long)(i) < (unsigned long long)(long long)(n) ||           \
     ::nb::record_check((long long)(i), (long long)(n), __LINE__))
#else
#define NB_IN_RANGE(i, n) true
#endif

} // namespace nb
