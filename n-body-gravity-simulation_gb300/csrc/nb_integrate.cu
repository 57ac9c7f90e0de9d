// nb_integrate.cu -- per-body update kernels of the integrators.
//
// Each kernel restates one update of the reference integrators in FP64 with the
// same operation order as the reference's CPU code, written with explicit
// round-to-nearest intrinsics so that no multiply-add is fused: given equal
// accelerations the GPU state equals the reference's CPU state bit for bit.
//   Euler            CPU/src/integrator_euler.cpp:9-16     (CUDA: integrator_euler.cu:3-22)
//   Euler-Cromer     CPU/src/integrator_euler-cromer.cpp:9-16 (CUDA: integrator_euler-cromer.cu:3-25)
//   Leapfrog KDK     CPU/src/integrator_leapfrog.cpp:6-22  (CUDA: integrator_leafrog.cu:3-45)
//   Velocity Verlet  CPU/src/integrator_velocity_verlet.cpp:7-21 (CUDA: integrator_velocity_verlet.cu:3-44)
//   RK4              CPU/src/integrator_rk4.cpp:14-43      (no CUDA counterpart in the reference)
// These passes are HBM-bound (48-120 B per body); the force evaluation between
// them dominates every step.
#include "nb_internal.h"

namespace nb {
namespace {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

enum { kEuler = NB_EULER, kEulerCromer = NB_EULER_CROMER, kLeapfrog = NB_LEAPFROG,
       kVerlet = NB_VELOCITY_VERLET };

template <int KIND>
__global__ void kick_drift_kernel(int n, double dt, double h, double *__restrict__ x,
                                  double *__restrict__ y, double *__restrict__ z,
                                  double *__restrict__ vx, double *__restrict__ vy,
                                  double *__restrict__ vz, const double *__restrict__ ax,
                                  const double *__restrict__ ay, const double *__restrict__ az,
                                  double *__restrict__ oax, double *__restrict__ oay,
                                  double *__restrict__ oaz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double p[3] = {x[i], y[i], z[i]};
    double v[3] = {vx[i], vy[i], vz[i]};
    const double a[3] = {ax[i], ay[i], az[i]};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (KIND == kEuler) {           // x = x + v dt ; v = v + a dt
            p[c] = add(p[c], mul(v[c], dt));
            v[c] = add(v[c], mul(a[c], dt));
        } else if (KIND == kEulerCromer) {  // v = v + a dt ; x = x + v dt
            v[c] = add(v[c], mul(a[c], dt));
            p[c] = add(p[c], mul(v[c], dt));
        } else if (KIND == kLeapfrog) {  // v += a dt/2 ; x += v dt
            v[c] = add(v[c], mul(a[c], h));
            p[c] = add(p[c], mul(v[c], dt));
        } else {  // Verlet: x += v dt + ((a*0.5)*dt)*dt ; a_old = a
            p[c] = add(p[c], add(mul(v[c], dt), mul(mul(mul(a[c], 0.5), dt), dt)));
        }
    }
    x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
    if (KIND != kVerlet) {
        vx[i] = v[0]; vy[i] = v[1]; vz[i] = v[2];
    } else {
        oax[i] = a[0]; oay[i] = a[1]; oaz[i] = a[2];
    }
}

template <int KIND>
__global__ void kick_kernel(int n, double h, double *__restrict__ vx, double *__restrict__ vy,
                            double *__restrict__ vz, const double *__restrict__ ax,
                            const double *__restrict__ ay, const double *__restrict__ az,
                            const double *__restrict__ oax, const double *__restrict__ oay,
                            const double *__restrict__ oaz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (KIND == kLeapfrog) {  // v += a dt/2
        vx[i] = add(vx[i], mul(ax[i], h));
        vy[i] = add(vy[i], mul(ay[i], h));
        vz[i] = add(vz[i], mul(az[i], h));
    } else {  // v += (a_old + a) * (0.5 dt)
        vx[i] = add(vx[i], mul(add(oax[i], ax[i]), h));
        vy[i] = add(vy[i], mul(add(oay[i], ay[i]), h));
        vz[i] = add(vz[i], mul(add(oaz[i], az[i]), h));
    }
}

// Stage state: pos = x + kv*h ; vel = v + ka*h   (integrator_rk4.cpp:15-31)
__global__ void rk4_stage_kernel(int n, double h, const double *__restrict__ x,
                                 const double *__restrict__ y, const double *__restrict__ z,
                                 const double *__restrict__ vx, const double *__restrict__ vy,
                                 const double *__restrict__ vz, const double *__restrict__ kvx,
                                 const double *__restrict__ kvy, const double *__restrict__ kvz,
                                 const double *__restrict__ kax, const double *__restrict__ kay,
                                 const double *__restrict__ kaz, double *__restrict__ ox,
                                 double *__restrict__ oy, double *__restrict__ oz,
                                 double *__restrict__ ovx, double *__restrict__ ovy,
                                 double *__restrict__ ovz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ox[i] = add(x[i], mul(kvx[i], h));
    oy[i] = add(y[i], mul(kvy[i], h));
    oz[i] = add(z[i], mul(kvz[i], h));
    ovx[i] = add(vx[i], mul(kax[i], h));
    ovy[i] = add(vy[i], mul(kay[i], h));
    ovz[i] = add(vz[i], mul(kaz[i], h));
}

// x += (v + 2 K2.v + 2 K3.v + K4.v) dt/6 ; v += (a + 2 K2.a + 2 K3.a + K4.a) dt/6
// (integrator_rk4.cpp:34-38), summed left to right.
__global__ void rk4_combine_kernel(int n, double w, double *__restrict__ x,
                                   double *__restrict__ y, double *__restrict__ z,
                                   double *__restrict__ vx, double *__restrict__ vy,
                                   double *__restrict__ vz, const double *__restrict__ ax,
                                   const double *__restrict__ ay,
                                   const double *__restrict__ az,
                                   const double *__restrict__ k2, const double *__restrict__ k3,
                                   const double *__restrict__ k4, size_t cap)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double *pos[3] = {x, y, z};
    double *vel[3] = {vx, vy, vz};
    const double *acc[3] = {ax, ay, az};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double v = vel[c][i];
        const double sv = add(add(add(v, mul(k2[(3 + c) * cap + i], 2.0)),
                                  mul(k3[(3 + c) * cap + i], 2.0)),
                              k4[(3 + c) * cap + i]);
        const double sa = add(add(add(acc[c][i], mul(k2[(6 + c) * cap + i], 2.0)),
                                  mul(k3[(6 + c) * cap + i], 2.0)),
                              k4[(6 + c) * cap + i]);
        pos[c][i] = add(pos[c][i], mul(sv, w));
        vel[c][i] = add(v, mul(sa, w));
    }
}

inline int blocks_for(int n) { return (n + 255) / 256; }

} // namespace

nb_status kick_drift(int kind, int n, double dt, double *x, double *y, double *z, double *vx,
                     double *vy, double *vz, const double *ax, const double *ay,
                     const double *az, double *oax, double *oay, double *oaz, cudaStream_t st)
{
    if (n <= 0) return NB_OK;
    const double h = dt / 2.0;
    switch (kind) {
    case kEuler:
        kick_drift_kernel<kEuler><<<blocks_for(n), 256, 0, st>>>(n, dt, h, x, y, z, vx, vy, vz,
                                                                 ax, ay, az, oax, oay, oaz);
        break;
    case kEulerCromer:
        kick_drift_kernel<kEulerCromer><<<blocks_for(n), 256, 0, st>>>(
            n, dt, h, x, y, z, vx, vy, vz, ax, ay, az, oax, oay, oaz);
        break;
    case kLeapfrog:
        kick_drift_kernel<kLeapfrog><<<blocks_for(n), 256, 0, st>>>(
            n, dt, h, x, y, z, vx, vy, vz, ax, ay, az, oax, oay, oaz);
        break;
    case kVerlet:
        kick_drift_kernel<kVerlet><<<blocks_for(n), 256, 0, st>>>(n, dt, h, x, y, z, vx, vy, vz,
                                                                  ax, ay, az, oax, oay, oaz);
        break;
    default:
        return fail(NB_ERR_INVALID_ARGUMENT, "kick_drift: bad integrator");
    }
    NB_LAUNCH_CHECK();
    return NB_OK;
}

nb_status kick(int kind, int n, double dt, double *vx, double *vy, double *vz, const double *ax,
               const double *ay, const double *az, const double *oax, const double *oay,
               const double *oaz, cudaStream_t st)
{
    if (n <= 0) return NB_OK;
    if (kind == kLeapfrog) {
        kick_kernel<kLeapfrog><<<blocks_for(n), 256, 0, st>>>(n, dt / 2.0, vx, vy, vz, ax, ay, az,
                                                              oax, oay, oaz);
    } else if (kind == kVerlet) {
        kick_kernel<kVerlet><<<blocks_for(n), 256, 0, st>>>(n, 0.5 * dt, vx, vy, vz, ax, ay, az,
                                                            oax, oay, oaz);
    } else {
        return fail(NB_ERR_INVALID_ARGUMENT, "kick: bad integrator");
    }
    NB_LAUNCH_CHECK();
    return NB_OK;
}

nb_status rk4_stage(int n, double h, const double *x, const double *y, const double *z,
                    const double *vx, const double *vy, const double *vz, const double *kvx,
                    const double *kvy, const double *kvz, const double *kax, const double *kay,
                    const double *kaz, double *ox, double *oy, double *oz, double *ovx,
                    double *ovy, double *ovz, cudaStream_t st)
{
    if (n <= 0) return NB_OK;
    rk4_stage_kernel<<<blocks_for(n), 256, 0, st>>>(n, h, x, y, z, vx, vy, vz, kvx, kvy, kvz,
                                                    kax, kay, kaz, ox, oy, oz, ovx, ovy, ovz);
    NB_LAUNCH_CHECK();
    return NB_OK;
}

nb_status rk4_combine(int n, double dt, double *x, double *y, double *z, double *vx,
                      double *vy, double *vz, const double *ax, const double *ay,
                      const double *az, const double *k2, const double *k3, const double *k4,
                      cudaStream_t st)
{
    // k2/k3/k4 are 9 planes of `cap` doubles: x y z vx vy vz ax ay az; the
    // plane stride is passed as the distance between consecutive planes.
    if (n <= 0) return NB_OK;
    const size_t cap = (size_t)(k3 - k2) / 9;
    rk4_combine_kernel<<<blocks_for(n), 256, 0, st>>>(n, dt / 6.0, x, y, z, vx, vy, vz, ax, ay,
                                                      az, k2, k3, k4, cap);
    NB_LAUNCH_CHECK();
    return NB_OK;
}

} // namespace nb
