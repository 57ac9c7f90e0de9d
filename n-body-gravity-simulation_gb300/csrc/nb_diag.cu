// nb_diag.cu -- energy and momentum diagnostics reduced on the GPU in FP64.
//
// Replaces the host loops of CUDA/src/test_common.cpp:63-182 (and
// CPU/include/tests_common.hpp:33-75), which needed a full device-to-host copy
// of the state every step and an O(N^2) host loop for the potential.
//   - per-body sums (kinetic energy, angular momentum, centre of mass, linear
//     momentum, mass): one HBM-bound pass (56 B per body), block partials in a
//     fixed tree order, then one block that adds the partials in index order;
//   - potential energy: an O(N^2) FP64 pass (one thread per body i, j-tiles in
//     shared memory, j in index order) that returns per-body sums
//     sum_{j != i} m_j / r_ij, unsoftened and softened, reduced like the above.
// All reductions have a fixed order, so results do not depend on scheduling.
#include "nb_internal.h"

#include <algorithm>

namespace nb {
namespace {

constexpr int kRed = 256;     // threads per reduction block
constexpr int kNSum = 11;     // KE, Lx, Ly, Lz, Mx, My, Mz, Px, Py, Pz, M

template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], double *sh /* [NV][kRed] */)
{
    const int t = threadIdx.x;
#pragma unroll
    for (int c = 0; c < NV; ++c) sh[c * kRed + t] = v[c];
    __syncthreads();
    for (int w = kRed / 2; w > 0; w >>= 1) {
        if (t < w) {
#pragma unroll
            for (int c = 0; c < NV; ++c) sh[c * kRed + t] += sh[c * kRed + t + w];
        }
        __syncthreads();
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) v[c] = sh[c * kRed];
}

__global__ void __launch_bounds__(kRed)
body_sums_kernel(const double *__restrict__ x, const double *__restrict__ y,
                 const double *__restrict__ z, const double *__restrict__ vx,
                 const double *__restrict__ vy, const double *__restrict__ vz,
                 const double *__restrict__ m, int n, double *__restrict__ part)
{
    __shared__ double sh[kNSum * kRed];
    double acc[kNSum];
#pragma unroll
    for (int c = 0; c < kNSum; ++c) acc[c] = 0.0;
    for (int i = blockIdx.x * kRed + threadIdx.x; i < n; i += gridDim.x * kRed) {
        const double X = x[i], Y = y[i], Z = z[i];
        const double U = vx[i], V = vy[i], W = vz[i], M = m[i];
        acc[0] += 0.5 * M * (U * U + V * V + W * W);
        acc[1] += (Y * W - Z * V) * M;
        acc[2] += (Z * U - X * W) * M;
        acc[3] += (X * V - Y * U) * M;
        acc[4] += X * M;
        acc[5] += Y * M;
        acc[6] += Z * M;
        acc[7] += U * M;
        acc[8] += V * M;
        acc[9] += W * M;
        acc[10] += M;
    }
    block_reduce<kNSum>(acc, sh);
    if (threadIdx.x == 0)
        for (int c = 0; c < kNSum; ++c) part[blockIdx.x * kNSum + c] = acc[c];
}

// Per-body potential sums: pu[i] = sum_{j!=i} m_j / r_ij,
// ps[i] = sum_{j!=i} m_j / sqrt(r_ij^2 + eps2).
__global__ void __launch_bounds__(kRed)
potential_rows_kernel(const double *__restrict__ x, const double *__restrict__ y,
                      const double *__restrict__ z, const double *__restrict__ m, int n,
                      double eps2, double *__restrict__ pu, double *__restrict__ ps)
{
    __shared__ double4_32a sh[kRed];
    const int i = blockIdx.x * kRed + threadIdx.x;
    const double xi = i < n ? x[i] : 0.0, yi = i < n ? y[i] : 0.0, zi = i < n ? z[i] : 0.0;
    double su = 0.0, ss = 0.0;
    for (int t0 = 0; t0 < n; t0 += kRed) {
        const int j = t0 + threadIdx.x;
        __syncthreads();
        sh[threadIdx.x] = j < n ? make_double4_32a(x[j], y[j], z[j], m[j])
                                : make_double4_32a(0.0, 0.0, 0.0, 0.0);
        __syncthreads();
        const int lim = min(kRed, n - t0);
        for (int jj = 0; jj < lim; ++jj) {
            if (t0 + jj == i) continue;
            const double4_32a B = sh[jj];
            const double dx = B.x - xi, dy = B.y - yi, dz = B.z - zi;
            const double r2 = dx * dx + dy * dy + dz * dz;
            su += B.w / sqrt(r2);
            ss += B.w / sqrt(r2 + eps2);
        }
    }
    if (i < n) {
        pu[i] = su;
        ps[i] = ss;
    }
}

// Final pass: one block.  Adds the body-sum partials in block order and the
// per-body potential terms m_i * row_i in index order (per thread, then a
// fixed tree).
__global__ void __launch_bounds__(kRed)
finish_kernel(const double *__restrict__ part, int nparts, const double *__restrict__ m,
              const double *__restrict__ pu, const double *__restrict__ ps, int n,
              double *__restrict__ out)
{
    __shared__ double sh[2 * kRed];
    const int t = threadIdx.x;
    if (t == 0) {
        double s[kNSum];
        for (int c = 0; c < kNSum; ++c) s[c] = 0.0;
        for (int b = 0; b < nparts; ++b)
            for (int c = 0; c < kNSum; ++c) s[c] += part[b * kNSum + c];
        for (int c = 0; c < kNSum; ++c) out[c] = s[c];
    }
    double v[2] = {0.0, 0.0};
    if (pu) {
        for (int i = t; i < n; i += kRed) {
            v[0] += m[i] * pu[i];
            v[1] += m[i] * ps[i];
        }
    }
    block_reduce<2>(v, sh);
    if (t == 0) {
        out[kNSum + 0] = v[0];
        out[kNSum + 1] = v[1];
    }
}

// FP32 pipe rate probe: every thread runs kFmaRounds rounds of kFmaChains
// independent packed FMAs on register values (no memory traffic in the loop)
// and stores one sum, so that nothing is optimised away.
constexpr int kFmaChains = 8, kFmaRounds = 4096;
__global__ void __launch_bounds__(256) fma_rate_kernel(float seed, float *__restrict__ out)
{
    float2 a[kFmaChains];
    const float2 m = make_float2(0.9999999f, 0.9999998f), c = make_float2(1e-7f, 2e-7f);
#pragma unroll
    for (int k = 0; k < kFmaChains; ++k)
        a[k] = make_float2(seed + (float)(threadIdx.x + k), seed - (float)k);
    for (int r = 0; r < kFmaRounds; ++r)
#pragma unroll
        for (int k = 0; k < kFmaChains; ++k) a[k] = __ffma2_rn(a[k], m, c);
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < kFmaChains; ++k) sum += a[k].x + a[k].y;
    out[blockIdx.x * 256 + threadIdx.x] = sum;
}

} // namespace

nb_status fp32_rate(double *lane_ops_per_s)
{
    const int blocks = 8 * device_props().num_sms;
    DevBuf out;
    NB_TRY(out.reserve(sizeof(float) * 256 * (size_t)blocks));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    NB_CUDA_TRY(cudaEventCreate(&e0));
    NB_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    nb_status st = NB_OK;
    for (int r = 0; r < 4 && st == NB_OK; ++r) {  // the first launch warms up
        cudaEventRecord(e0, 0);
        fma_rate_kernel<<<blocks, 256>>>(1.0f + r, out.as<float>());
        const cudaError_t launched = cudaGetLastError();
        cudaEventRecord(e1, 0);
        if (launched != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
            st = fail(NB_ERR_CUDA, "fp32 rate probe");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0) best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    out.release();
    NB_TRY(st);
    const double ops = (double)blocks * 256.0 * kFmaRounds * kFmaChains * 2.0;
    *lane_ops_per_s = ops / (best * 1e-3);
    return NB_OK;
}

nb_status diagnostics(const double *x, const double *y, const double *z, const double *vx,
                      const double *vy, const double *vz, const double *m, int n, double G,
                      double eps2, DevBuf &scratch, cudaStream_t st, nb_diag *out)
{
    if (n <= 0) return fail(NB_ERR_NOT_LOADED, "diagnostics: no bodies");
    const int nparts = std::min((n + kRed - 1) / kRed, 4 * device_props().num_sms);
    const size_t bytes = sizeof(double) * ((size_t)nparts * kNSum + 2 * (size_t)n + 16);
    NB_TRY(scratch.reserve(bytes));
    double *part = scratch.as<double>();
    double *pu = part + (size_t)nparts * kNSum;
    double *ps = pu + n;
    double *res = ps + n;
    body_sums_kernel<<<nparts, kRed, 0, st>>>(x, y, z, vx, vy, vz, m, n, part);
    NB_LAUNCH_CHECK();
    potential_rows_kernel<<<(n + kRed - 1) / kRed, kRed, 0, st>>>(x, y, z, m, n, eps2, pu, ps);
    NB_LAUNCH_CHECK();
    finish_kernel<<<1, kRed, 0, st>>>(part, nparts, m, pu, ps, n, res);
    NB_LAUNCH_CHECK();
    double h[kNSum + 2];
    NB_CUDA_TRY(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, st));
    NB_CUDA_TRY(cudaStreamSynchronize(st));
    out->kinetic = h[0];
    out->angular_momentum[0] = h[1];
    out->angular_momentum[1] = h[2];
    out->angular_momentum[2] = h[3];
    out->mass = h[10];
    for (int c = 0; c < 3; ++c) {
        out->center_of_mass[c] = h[4 + c] / h[10];
        out->momentum[c] = h[7 + c];
    }
    // each unordered pair appears twice in sum_i m_i row_i
    out->potential = -0.5 * G * h[kNSum + 0];
    out->potential_softened = -0.5 * G * h[kNSum + 1];
    out->total = out->kinetic + out->potential;
    out->total_softened = out->kinetic + out->potential_softened;
    return NB_OK;
}

} // namespace nb
