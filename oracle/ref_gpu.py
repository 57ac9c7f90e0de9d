"""The reference's FP64 GPU kernel as a measured baseline (test and baseline
infrastructure only; nothing in the product imports this file).

`computeAccelerationNaiveKernel` (CUDA/src/force_calculator_naive.cu:4-59) is
compiled for sm_103a from the reference source by `build_ref.sh` into
`_ref/ref_naive_sm103a.cubin` (device code only, so it runs on any host of the
GPU machine).  This module loads it with the CUDA driver API and launches it
exactly as `ForceCalculatorNaive::computeAccelerations` does
(force_calculator_naive.cu:61-77): ceil(N / BLOCK_SIZE) CTAs of BLOCK_SIZE = 256
threads (CUDA/include/common.hpp:44), arguments (pos_x, pos_y, pos_z, acc_x,
acc_y, acc_z, mass, N, softening^2), G = 4 pi^2 folded in by the kernel.
"""
import ctypes
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_naive_sm103a.cubin")
# Itanium mangling of computeAccelerationNaiveKernel(const double*, const double*,
# const double*, double*, double*, double*, const double*, int, double)
KERNEL = b"_Z30computeAccelerationNaiveKernelPKdS0_S0_PdS1_S1_S0_id"
BLOCK_SIZE = 256
G_REF = 4.0 * math.pi * math.pi


def available() -> bool:
    return os.path.exists(CUBIN)


class RefNaiveKernel:
    """The reference kernel in the current (torch primary) CUDA context."""

    def __init__(self):
        import torch

        torch.zeros(1, device="cuda")  # makes the primary context current
        self._cu = ctypes.CDLL("libcuda.so.1")
        cu = self._cu
        cu.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p,
                                           ctypes.c_char_p]
        cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
            ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        cu.cuModuleUnload.argtypes = [ctypes.c_void_p]
        with open(CUBIN, "rb") as f:
            self._image = ctypes.create_string_buffer(f.read())
        self._mod = ctypes.c_void_p()
        self._check(cu.cuModuleLoadData(ctypes.byref(self._mod), self._image), "cuModuleLoadData")
        self._fn = ctypes.c_void_p()
        self._check(cu.cuModuleGetFunction(ctypes.byref(self._fn), self._mod, KERNEL),
                    "cuModuleGetFunction")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def launch(self, px, py, pz, ax, ay, az, m, n: int, eps2: float, stream: int = 0):
        """Device pointers (ints) of FP64 arrays of n bodies; asynchronous."""
        args = [ctypes.c_void_p(px), ctypes.c_void_p(py), ctypes.c_void_p(pz),
                ctypes.c_void_p(ax), ctypes.c_void_p(ay), ctypes.c_void_p(az),
                ctypes.c_void_p(m), ctypes.c_int(n), ctypes.c_double(eps2)]
        params = (ctypes.c_void_p * len(args))(*[ctypes.addressof(a) for a in args])
        grid = (n + BLOCK_SIZE - 1) // BLOCK_SIZE
        self._check(self._cu.cuLaunchKernel(self._fn, grid, 1, 1, BLOCK_SIZE, 1, 1, 0,
                                            ctypes.c_void_p(stream), params, None),
                    "cuLaunchKernel")

    def forces(self, x, y, z, m, eps: float):
        """Accelerations (numpy FP64) of host arrays, synchronously."""
        import numpy as np
        import torch

        n = len(x)
        dev = [torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).cuda()
               for v in (x, y, z, m)]
        acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()
        self.launch(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), acc[0].data_ptr(),
                    acc[1].data_ptr(), acc[2].data_ptr(), dev[3].data_ptr(), n, eps * eps)
        torch.cuda.synchronize()
        return tuple(a.cpu().numpy() for a in acc)

    def close(self):
        if self._mod:
            self._cu.cuModuleUnload(self._mod)
            self._mod = ctypes.c_void_p()
