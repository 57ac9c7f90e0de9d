// force_calculator.hpp -- the reference's force-calculator interface
// (CUDA/include/force_calculator.hpp:14-30).
#pragma once
#include <common.hpp>
#include <particle_data.hpp>

class ForceCalculator {
protected:
    double softening_squared;

public:
    ForceCalculator() : softening_squared(0.0) {}
    ForceCalculator(double softening) : softening_squared(softening * softening) {}
    virtual ~ForceCalculator() = default;

    // Accelerations of particles.pos_* into particles.acc_*; synchronous.
    virtual void computeAccelerations(ParticleArrays &particles) = 0;
    virtual std::string name() const = 0;
};
