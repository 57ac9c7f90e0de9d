// integrator_euler.hpp -- CUDA/include/integrator_euler.hpp:5-30.
#pragma once
#include "integrator.hpp"

class EulerIntegrator : public TimeIntegrator {
protected:
    std::string integrator_name = "Euler Integrator";
    cudaEvent_t startEvent = nullptr;
    cudaEvent_t stopEvent = nullptr;
    double total_compute_time_ms;

public:
    EulerIntegrator() : total_compute_time_ms(0.0) {}
    ~EulerIntegrator() = default;
    void step(ForceCalculator &calculator, ParticleArrays &particles, double dt) override;
    std::string name() const override;
};
