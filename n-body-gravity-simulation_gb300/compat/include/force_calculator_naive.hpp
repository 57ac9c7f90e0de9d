// force_calculator_naive.hpp -- all-pairs calculator of the reference's API
// (CUDA/include/force_calculator_naive.hpp:5-31).  Backed by the engine's FP64
// all-pairs kernel; NBODY_COMPAT_DIRECT=mixed selects the mixed-precision one.
#pragma once
#include "force_calculator.hpp"

class ForceCalculatorNaive : public ForceCalculator {
protected:
    cudaEvent_t startEvent;
    cudaEvent_t stopEvent;
    double total_compute_time_ms;

public:
    using ForceCalculator::ForceCalculator;
    ForceCalculatorNaive(double softening)
        : ForceCalculator(softening), startEvent(nullptr), stopEvent(nullptr),
          total_compute_time_ms(0.0)
    {
    }
    ~ForceCalculatorNaive() override = default;

    void computeAccelerations(ParticleArrays &particles) override;
    std::string name() const override;
    double getTotalComputeTime() const { return total_compute_time_ms; }
    void resetTimeStatistics() { total_compute_time_ms = 0.0; }
};
