// integrator_euler-cromer.hpp -- CUDA/include/integrator_euler-cromer.hpp:5-31.
#pragma once
#include "integrator.hpp"

class EulerCromerIntegrator : public TimeIntegrator {
protected:
    std::string integrator_name = "Euler Integrator";
    cudaEvent_t startEvent = nullptr;
    cudaEvent_t stopEvent = nullptr;
    double total_compute_time_ms;
    bool is_first_step = true;

public:
    EulerCromerIntegrator() : total_compute_time_ms(0.0) {}
    ~EulerCromerIntegrator() = default;
    void step(ForceCalculator &calculator, ParticleArrays &particles, double dt) override;
    std::string name() const override;
};
