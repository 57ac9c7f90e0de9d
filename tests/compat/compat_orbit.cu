// compat_orbit.cu -- the reference's Earth-Sun driver pattern
// (CUDA/tests/test1_EarthSun.cu) through libnbody_compat.so: Sun + Earth,
// ForceCalculatorNaive(0), one integrator (argv[1]: euler, euler-cromer,
// leapfrog, verlet, rk4), dt = 1/365, argv[2] steps; writes the final
// positions, velocities and accelerations (10 arrays of 2 doubles) to argv[3].
#include "force_calculator_naive.hpp"
#include "integrator_euler-cromer.hpp"
#include "integrator_euler.hpp"
#include "integrator_leapfrog.hpp"
#include "integrator_rk4.hpp"
#include "integrator_velocity_verlet.hpp"

#include <cstdio>
#include <cstring>
#include <memory>

int main(int argc, char **argv)
{
    if (argc < 4) return 2;
    std::unique_ptr<TimeIntegrator> integ;
    if (!std::strcmp(argv[1], "euler")) integ.reset(new EulerIntegrator());
    else if (!std::strcmp(argv[1], "euler-cromer")) integ.reset(new EulerCromerIntegrator());
    else if (!std::strcmp(argv[1], "leapfrog")) integ.reset(new LeapfrogIntegrator());
    else if (!std::strcmp(argv[1], "verlet")) integ.reset(new VelocityVerletIntegrator());
    else integ.reset(new RK4Integrator());
    const int steps = std::atoi(argv[2]);
    double x[2] = {0.0, 1.0}, y[2] = {0.0, 0.0}, z[2] = {0.0, 0.0};
    double vx[2] = {0.0, 0.0}, vy[2] = {0.0, 2.0 * constant::PI}, vz[2] = {0.0, 0.0};
    double m[2] = {1.0, 3.003e-6};
    ParticleArrays p;
    allocateParticles(p, 2);
    copyParticlesToDevice(p, x, y, z, vx, vy, vz, m);
    ForceCalculatorNaive calc(0.0);
    const double dt = 1.0 / 365.0;
    for (int s = 0; s < steps; ++s) integ->step(calc, p, dt);
    double out[10][2];
    copyParticlesToHost(p, out[0], out[1], out[2], out[3], out[4], out[5], out[6], out[7],
                        out[8], out[9]);
    FILE *f = std::fopen(argv[3], "wb");
    if (!f) return 3;
    std::fwrite(out, sizeof(double), 20, f);
    std::fclose(f);
    freeParticles(p);
    std::printf("%s: earth at (%.15f, %.15f)\n", integ->name().c_str(), out[0][1], out[1][1]);
    return 0;
}
