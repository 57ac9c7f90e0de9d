// nb_step.cu -- one integrator step over a set of FP64 planes with a pluggable
// force evaluation; used by the batched ensemble and the serving loop.
//
// The order of updates and force evaluations is the reference's
// (CPU/src/integrator_*.cpp, CUDA/src/integrator_*.cu); leapfrog and velocity
// Verlet reuse the end-of-step force of the previous step when it is valid,
// as the CUDA reference does through is_first_step.
#include "nb_internal.h"

namespace nb {

nb_status integrate_step(int integ, int n, double dt, double *const f[10], StepBuffers &b,
                         bool &forces_valid, const ForceFn &force, cudaStream_t st)
{
    double *x = f[0], *y = f[1], *z = f[2], *vx = f[3], *vy = f[4], *vz = f[5];
    double *ax = f[6], *ay = f[7], *az = f[8];
    switch (integ) {
    case NB_EULER:
    case NB_EULER_CROMER:
        NB_TRY(force(x, y, z, ax, ay, az));
        NB_TRY(kick_drift(integ, n, dt, x, y, z, vx, vy, vz, ax, ay, az, nullptr, nullptr,
                          nullptr, st));
        forces_valid = false;
        return NB_OK;
    case NB_LEAPFROG:
        if (!forces_valid) NB_TRY(force(x, y, z, ax, ay, az));
        NB_TRY(kick_drift(integ, n, dt, x, y, z, vx, vy, vz, ax, ay, az, nullptr, nullptr,
                          nullptr, st));
        forces_valid = false;
        NB_TRY(force(x, y, z, ax, ay, az));
        NB_TRY(kick(integ, n, dt, vx, vy, vz, ax, ay, az, nullptr, nullptr, nullptr, st));
        forces_valid = true;
        return NB_OK;
    case NB_VELOCITY_VERLET: {
        if (!b.old_acc) return fail(NB_ERR_INVALID_ARGUMENT, "velocity Verlet needs a(t) planes");
        double *o = b.old_acc;
        if (!forces_valid) NB_TRY(force(x, y, z, ax, ay, az));
        NB_TRY(kick_drift(integ, n, dt, x, y, z, vx, vy, vz, ax, ay, az, o, o + b.ps,
                          o + 2 * b.ps, st));
        forces_valid = false;
        NB_TRY(force(x, y, z, ax, ay, az));
        NB_TRY(kick(integ, n, dt, vx, vy, vz, ax, ay, az, o, o + b.ps, o + 2 * b.ps, st));
        forces_valid = true;
        return NB_OK;
    }
    case NB_RK4: {
        if (!b.rk4) return fail(NB_ERR_INVALID_ARGUMENT, "RK4 needs stage planes");
        const size_t ps = b.ps;
        double *k2 = b.rk4, *k3 = k2 + 9 * ps, *k4 = k3 + 9 * ps;
        auto P = [ps](double *k, int c) { return k + c * ps; };
        const double h = dt / 2.0;
        NB_TRY(force(x, y, z, ax, ay, az));
        NB_TRY(rk4_stage(n, h, x, y, z, vx, vy, vz, vx, vy, vz, ax, ay, az, P(k2, 0), P(k2, 1),
                         P(k2, 2), P(k2, 3), P(k2, 4), P(k2, 5), st));
        NB_TRY(force(P(k2, 0), P(k2, 1), P(k2, 2), P(k2, 6), P(k2, 7), P(k2, 8)));
        NB_TRY(rk4_stage(n, h, x, y, z, vx, vy, vz, P(k2, 3), P(k2, 4), P(k2, 5), P(k2, 6),
                         P(k2, 7), P(k2, 8), P(k3, 0), P(k3, 1), P(k3, 2), P(k3, 3), P(k3, 4),
                         P(k3, 5), st));
        NB_TRY(force(P(k3, 0), P(k3, 1), P(k3, 2), P(k3, 6), P(k3, 7), P(k3, 8)));
        NB_TRY(rk4_stage(n, dt, x, y, z, vx, vy, vz, P(k3, 3), P(k3, 4), P(k3, 5), P(k3, 6),
                         P(k3, 7), P(k3, 8), P(k4, 0), P(k4, 1), P(k4, 2), P(k4, 3), P(k4, 4),
                         P(k4, 5), st));
        NB_TRY(force(P(k4, 0), P(k4, 1), P(k4, 2), P(k4, 6), P(k4, 7), P(k4, 8)));
        NB_TRY(rk4_combine(n, dt, x, y, z, vx, vy, vz, ax, ay, az, k2, k3, k4, st));
        forces_valid = false;
        return NB_OK;
    }
    default:
        return fail(NB_ERR_INVALID_ARGUMENT, "unknown integrator");
    }
}

} // namespace nb
