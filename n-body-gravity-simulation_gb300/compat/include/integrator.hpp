// integrator.hpp -- the reference's integrator interface
// (CUDA/include/integrator.hpp:7-17); note its argument order (calculator first).
#pragma once
#include <common.hpp>
#include <force_calculator.hpp>
#include <particle_data.hpp>

class TimeIntegrator {
public:
    virtual ~TimeIntegrator() = default;
    virtual void step(ForceCalculator &calculator, ParticleArrays &particles, double dt) = 0;
    virtual std::string name() const = 0;
};
