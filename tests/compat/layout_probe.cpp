// layout_probe.cpp -- prints the size of every class of the reference's CUDA host
// API and the offsets of its data members.  Compiled once against the
// reference's headers and once against the compat headers; the outputs must be
// equal for code built against either header set to share objects.
#include "force_calculator_barnes_hut.hpp"
#include "force_calculator_naive.hpp"
#include "integrator_euler-cromer.hpp"
#include "integrator_euler.hpp"
#include "integrator_leapfrog.hpp"
#include "integrator_velocity_verlet.hpp"
#include "particle_data.hpp"

#include <cstddef>
#include <cstdio>

#pragma GCC diagnostic ignored "-Winvalid-offsetof"
#define OFF(T, m) std::printf("%s.%s %zu\n", #T, #m, (size_t)offsetof(T, m))

int main()
{
    std::printf("ParticleArrays %zu\n", sizeof(ParticleArrays));
    OFF(ParticleArrays, pos_x);
    OFF(ParticleArrays, acc_x);
    OFF(ParticleArrays, old_acc_x);
    OFF(ParticleArrays, mass);
    OFF(ParticleArrays, morton_codes);
    OFF(ParticleArrays, pos_x_sorted);
    OFF(ParticleArrays, acc_z_sorted);
    std::printf("Bounds %zu\nTreeArrays %zu\n", sizeof(Bounds), sizeof(TreeArrays));
    OFF(TreeArrays, mass);
    OFF(TreeArrays, node_depth);
    std::printf("ForceCalculatorNaive %zu\n", sizeof(ForceCalculatorNaive));
    std::printf("BarnesHutForceCalculator %zu\n", sizeof(BarnesHutForceCalculator));
    OFF(BarnesHutForceCalculator, softening_squared);
    OFF(BarnesHutForceCalculator, theta_sqr);
    OFF(BarnesHutForceCalculator, leaf_capacity);
    OFF(BarnesHutForceCalculator, total_compute_time_ms);
    OFF(BarnesHutForceCalculator, traverse_tree_time_ms);
    OFF(BarnesHutForceCalculator, radix_sort_temp_storage_bytes);
    OFF(BarnesHutForceCalculator, tree);
    OFF(BarnesHutForceCalculator, nextFreeNode);
    OFF(BarnesHutForceCalculator, level_counts);
    std::printf("EulerIntegrator %zu\n", sizeof(EulerIntegrator));
    std::printf("EulerCromerIntegrator %zu\n", sizeof(EulerCromerIntegrator));
    std::printf("LeapfrogIntegrator %zu\n", sizeof(LeapfrogIntegrator));
    std::printf("VelocityVerletIntegrator %zu\n", sizeof(VelocityVerletIntegrator));
    return 0;
}
