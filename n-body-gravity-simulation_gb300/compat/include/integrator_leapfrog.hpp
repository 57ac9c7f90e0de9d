// integrator_leapfrog.hpp -- CUDA/include/integrator_leapfrog.hpp:5-27.
// Kick-drift-kick; the start-of-step force is reused after the first step.
#pragma once
#include "integrator.hpp"

class LeapfrogIntegrator : public TimeIntegrator {
protected:
    cudaEvent_t startEvent = nullptr, stopEvent = nullptr;
    double total_compute_time_ms;
    bool is_first_step = true;

public:
    LeapfrogIntegrator() : total_compute_time_ms(0.0) {}
    ~LeapfrogIntegrator() = default;
    void step(ForceCalculator &calculator, ParticleArrays &particles, double dt) override;
    std::string name() const override;
};
