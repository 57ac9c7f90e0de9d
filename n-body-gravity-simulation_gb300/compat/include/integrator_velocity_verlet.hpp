// integrator_velocity_verlet.hpp -- CUDA/include/integrator_velocity_verlet.hpp:5-26.
#pragma once
#include "integrator.hpp"

class VelocityVerletIntegrator : public TimeIntegrator {
protected:
    cudaEvent_t startEvent = nullptr, stopEvent = nullptr;
    double total_compute_time_ms;
    bool is_first_step = true;

public:
    VelocityVerletIntegrator() : total_compute_time_ms(0.0) {}
    ~VelocityVerletIntegrator() = default;
    void step(ForceCalculator &calculator, ParticleArrays &particles, double dt) override;
    std::string name() const override;
};
