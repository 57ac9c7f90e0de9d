// integrator_rk4.hpp -- classic RK4 with the reference's CPU arithmetic
// (CPU/src/integrator_rk4.cpp:3-47), on the GPU.  The reference's CUDA API has
// no RK4 (CUDA/tests/test1_EarthSun.cu:51 names one in a comment); this class
// completes the family with the same step() signature.
#pragma once
#include "integrator.hpp"

class RK4Integrator : public TimeIntegrator {
protected:
    double total_compute_time_ms = 0.0;

public:
    RK4Integrator() = default;
    ~RK4Integrator() = default;
    void step(ForceCalculator &calculator, ParticleArrays &particles, double dt) override;
    std::string name() const override;
};
