// particle_data.hpp -- device particle storage of the reference's CUDA host API
// (CUDA/include/particle_data.hpp:6-73): a plain struct of device pointers,
// one value per particle, allocated by allocateParticles.  Field order and
// types are those of the reference so that code built against either header
// shares one layout.
#pragma once
#include <common.hpp>

struct ParticleArrays {
    int num_particles;

    double *pos_x;
    double *pos_y;
    double *pos_z;

    double *vel_x;
    double *vel_y;
    double *vel_z;

    double *acc_x;
    double *acc_y;
    double *acc_z;

    double *old_acc_x;
    double *old_acc_y;
    double *old_acc_z;

    double *mass;

    // Barnes-Hut scratch of the reference implementation; allocated for
    // layout compatibility, unused by this engine (its tree keeps its own).
    uint32_t *morton_codes;
    uint32_t *morton_codes_sorted;
    int *particle_indices;
    int *particle_indices_sorted;
    float *pos_x_sorted;
    float *pos_y_sorted;
    float *pos_z_sorted;
    float *mass_sorted;
    float *acc_x_sorted;
    float *acc_y_sorted;
    float *acc_z_sorted;
};

void allocateParticles(ParticleArrays &particles, size_t num_particles);
void freeParticles(ParticleArrays &particles);
void copyParticlesToDevice(ParticleArrays &particles, const double *pos_x, const double *pos_y,
                           const double *pos_z, const double *vel_x, const double *vel_y,
                           const double *vel_z, const double *mass);
void copyParticlesToHost(const ParticleArrays &particles, double *pos_x, double *pos_y,
                         double *pos_z, double *vel_x, double *vel_y, double *vel_z,
                         double *acc_x, double *acc_y, double *acc_z, double *mass);
