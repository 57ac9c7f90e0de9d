// compat.cpp -- the reference's CUDA host API (CUDA/include/*.hpp) implemented on
// the engine's C ABI (include/nbody_c.h).
//
// Code written against PawanKiitb/N-body-gravity-simulation's CUDA/include
// headers (ParticleArrays, ForceCalculatorNaive, BarnesHutForceCalculator, the
// integrators, allocateParticles & co.) links against libnbody_compat.so
// unchanged: the classes keep the reference's member layout, and their
// out-of-line members are defined here.  Every calculator gets an engine
// simulation (nb_sim) that works in place on the caller's ParticleArrays
// (nb_bind_device), configured from the calculator's own fields on each call.
// Like the reference, calls are synchronous and a CUDA failure prints a
// message and exits (CUDA/src/force_calculator_naive.cu:86-90).
#include "force_calculator_barnes_hut.hpp"
#include "force_calculator_naive.hpp"
#include "integrator_euler-cromer.hpp"
#include "integrator_euler.hpp"
#include "integrator_leapfrog.hpp"
#include "integrator_rk4.hpp"
#include "integrator_velocity_verlet.hpp"
#include "particle_data.hpp"

#include "nbody_c.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <unordered_map>

namespace {

[[noreturn]] void die(const char *where, const char *what)
{
    std::cerr << "nbody compat: " << where << ": " << what << std::endl;
    std::exit(EXIT_FAILURE);
}

void check(nb_status st, const char *where)
{
    if (st != NB_OK) {
        std::string msg = std::string(nb_status_string(st)) + ": " + nb_last_error();
        die(where, msg.c_str());
    }
}

void check_cuda(cudaError_t e, const char *where)
{
    if (e != cudaSuccess) die(where, cudaGetErrorString(e));
}

// Reads the protected softening of the base class through a member pointer
// formed in a derived context (legal access to a protected member).
struct SofteningAccess : ForceCalculator {
    static double ForceCalculator::*field() { return &SofteningAccess::softening_squared; }
};

struct Engine {
    nb_sim *sim = nullptr;
    size_t capacity = 0;
    const double *bound_pos = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

std::mutex g_mutex;
std::unordered_map<const void *, Engine> g_engines;  // by calculator address

nb_config config_of(ForceCalculator &calc)
{
    nb_config c;
    nb_config_default(&c);
    c.G = constant::G;
    if (auto *bh = dynamic_cast<BarnesHutForceCalculator *>(&calc)) {
        // the reference's Barnes-Hut calculator keeps its own softening_squared
        // (force_calculator_barnes_hut.hpp:27), shadowing the base class's
        c.method = NB_BARNES_HUT;
        c.softening = std::sqrt(bh->softening_squared);
        c.theta = std::sqrt(bh->theta_sqr);
        c.leaf_capacity = bh->leaf_capacity;
        // the reference's walks open, of every node they open, the child
        // toward the body too (force_calculator_barnes_hut.cu:60-73)
        c.flags |= NB_FLAG_BH_REFERENCE_OPENING;
        return c;
    }
    if (dynamic_cast<ForceCalculatorNaive *>(&calc)) {
        const char *mode = std::getenv("NBODY_COMPAT_DIRECT");
        c.method = (mode && std::strcmp(mode, "mixed") == 0) ? NB_DIRECT_MIXED : NB_DIRECT_FP64;
        c.softening = std::sqrt(calc.*SofteningAccess::field());
        return c;
    }
    die("ForceCalculator", "unsupported calculator type (not one of the reference's)");
}

// The engine simulation of `calc`, bound to `p` and configured from `calc`.
Engine &engine_for(ForceCalculator &calc, ParticleArrays &p)
{
    const nb_config cfg = config_of(calc);
    std::lock_guard<std::mutex> lock(g_mutex);
    Engine &e = g_engines[&calc];
    const size_t n = (size_t)std::max(p.num_particles, 0);
    if (!e.sim || e.capacity < n) {
        if (e.sim) nb_destroy(e.sim);
        e.sim = nullptr;
        check(nb_create(&cfg, std::max<size_t>(n, 1), nullptr, &e.sim), "nb_create");
        e.capacity = std::max<size_t>(n, 1);
        if (!e.e0) check_cuda(cudaEventCreate(&e.e0), "cudaEventCreate");
        if (!e.e1) check_cuda(cudaEventCreate(&e.e1), "cudaEventCreate");
    } else {
        check(nb_set_config(e.sim, &cfg), "nb_set_config");
    }
    double *arrays[10] = {p.pos_x, p.pos_y, p.pos_z, p.vel_x, p.vel_y,
                          p.vel_z, p.acc_x, p.acc_y, p.acc_z, p.mass};
    check(nb_bind_device(e.sim, n, arrays), "nb_bind_device");
    e.bound_pos = p.pos_x;
    return e;
}

// Runs fn on the engine's stream between two events and returns the device ms.
template <class Fn> double timed(Engine &e, Fn fn)
{
    check_cuda(cudaEventRecord(e.e0, nullptr), "cudaEventRecord");
    fn();
    check_cuda(cudaEventRecord(e.e1, nullptr), "cudaEventRecord");
    check_cuda(cudaEventSynchronize(e.e1), "cudaEventSynchronize");
    float ms = 0.f;
    check_cuda(cudaEventElapsedTime(&ms, e.e0, e.e1), "cudaEventElapsedTime");
    return ms;
}

void invalidate_bound(const double *pos)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    for (auto &kv : g_engines)
        if (kv.second.sim && kv.second.bound_pos == pos) nb_invalidate_forces(kv.second.sim);
}

void integrate(ForceCalculator &calc, ParticleArrays &p, int integrator, double dt,
               bool *is_first_step, double *total_ms)
{
    if (p.num_particles <= 0) return;
    Engine &e = engine_for(calc, p);
    if (is_first_step && *is_first_step) {
        check(nb_invalidate_forces(e.sim), "nb_invalidate_forces");
        *is_first_step = false;
    }
    *total_ms += timed(e, [&] { check(nb_step(e.sim, integrator, dt, 1), "nb_step"); });
}

} // namespace

// ------------------------------------------------------------ particle storage
void allocateParticles(ParticleArrays &p, size_t n)
{
    std::memset(&p, 0, sizeof(p));
    p.num_particles = (int)n;
    const size_t bd = n * sizeof(double), bf = n * sizeof(float), bi = n * sizeof(int);
    double **dbl[] = {&p.pos_x, &p.pos_y, &p.pos_z, &p.vel_x, &p.vel_y, &p.vel_z,
                      &p.acc_x, &p.acc_y, &p.acc_z, &p.old_acc_x, &p.old_acc_y, &p.old_acc_z,
                      &p.mass};
    for (double **a : dbl) check_cuda(cudaMalloc((void **)a, bd), "allocateParticles");
    check_cuda(cudaMalloc((void **)&p.morton_codes, bi), "allocateParticles");
    check_cuda(cudaMalloc((void **)&p.morton_codes_sorted, bi), "allocateParticles");
    check_cuda(cudaMalloc((void **)&p.particle_indices, bi), "allocateParticles");
    check_cuda(cudaMalloc((void **)&p.particle_indices_sorted, bi), "allocateParticles");
    float **flt[] = {&p.pos_x_sorted, &p.pos_y_sorted, &p.pos_z_sorted, &p.mass_sorted,
                     &p.acc_x_sorted, &p.acc_y_sorted, &p.acc_z_sorted};
    for (float **a : flt) check_cuda(cudaMalloc((void **)a, bf), "allocateParticles");
}

void freeParticles(ParticleArrays &p)
{
    invalidate_bound(p.pos_x);
    void *all[] = {p.pos_x, p.pos_y, p.pos_z, p.vel_x, p.vel_y, p.vel_z, p.acc_x, p.acc_y,
                   p.acc_z, p.old_acc_x, p.old_acc_y, p.old_acc_z, p.mass, p.morton_codes,
                   p.morton_codes_sorted, p.particle_indices, p.particle_indices_sorted,
                   p.pos_x_sorted, p.pos_y_sorted, p.pos_z_sorted, p.mass_sorted,
                   p.acc_x_sorted, p.acc_y_sorted, p.acc_z_sorted};
    cudaDeviceSynchronize();
    for (void *a : all)
        if (a) cudaFree(a);
    std::memset(&p, 0, sizeof(p));
}

void copyParticlesToDevice(ParticleArrays &p, const double *pos_x, const double *pos_y,
                           const double *pos_z, const double *vel_x, const double *vel_y,
                           const double *vel_z, const double *mass)
{
    const size_t b = (size_t)p.num_particles * sizeof(double);
    const double *src[7] = {pos_x, pos_y, pos_z, vel_x, vel_y, vel_z, mass};
    double *dst[7] = {p.pos_x, p.pos_y, p.pos_z, p.vel_x, p.vel_y, p.vel_z, p.mass};
    for (int k = 0; k < 7; ++k)
        check_cuda(cudaMemcpy(dst[k], src[k], b, cudaMemcpyHostToDevice), "copyParticlesToDevice");
    double *zero[6] = {p.acc_x, p.acc_y, p.acc_z, p.old_acc_x, p.old_acc_y, p.old_acc_z};
    for (double *z : zero) check_cuda(cudaMemset(z, 0, b), "copyParticlesToDevice");
    invalidate_bound(p.pos_x);
}

void copyParticlesToHost(const ParticleArrays &p, double *pos_x, double *pos_y, double *pos_z,
                         double *vel_x, double *vel_y, double *vel_z, double *acc_x,
                         double *acc_y, double *acc_z, double *mass)
{
    const size_t b = (size_t)p.num_particles * sizeof(double);
    double *dst[10] = {pos_x, pos_y, pos_z, vel_x, vel_y, vel_z, acc_x, acc_y, acc_z, mass};
    const double *src[10] = {p.pos_x, p.pos_y, p.pos_z, p.vel_x, p.vel_y,
                             p.vel_z, p.acc_x, p.acc_y, p.acc_z, p.mass};
    for (int k = 0; k < 10; ++k)
        check_cuda(cudaMemcpy(dst[k], src[k], b, cudaMemcpyDeviceToHost), "copyParticlesToHost");
}

// ------------------------------------------------------------ calculators
void ForceCalculatorNaive::computeAccelerations(ParticleArrays &p)
{
    if (p.num_particles <= 0) return;
    Engine &e = engine_for(*this, p);
    total_compute_time_ms +=
        timed(e, [&] { check(nb_compute_forces(e.sim), "computeAccelerations"); });
}

std::string ForceCalculatorNaive::name() const { return "Naive-CUDA"; }

void BarnesHutForceCalculator::computeAccelerations(ParticleArrays &p)
{
    if (p.num_particles <= 0) return;
    Engine &e = engine_for(*this, p);
    check(nb_profile_enable(e.sim, 1), "nb_profile_enable");
    nb_profile prof;
    check(nb_profile_read(e.sim, &prof, 1), "nb_profile_read");
    const double ms = timed(e, [&] { check(nb_compute_forces(e.sim), "computeAccelerations"); });
    check(nb_profile_read(e.sim, &prof, 1), "nb_profile_read");
    const double walk = prof.force_kernel_ms;
    traverse_tree_time_ms += walk;
    build_tree_time_ms += ms - walk;
    total_compute_time_ms += ms;
}

void BarnesHutForceCalculator::buildTree(ParticleArrays &p)
{
    if (p.num_particles <= 0) return;
    Engine &e = engine_for(*this, p);
    build_tree_time_ms += timed(e, [&] { check(nb_bh_build(e.sim, nullptr), "buildTree"); });
}

void BarnesHutForceCalculator::computeBoundingBox(ParticleArrays &p) { buildTree(p); }
void BarnesHutForceCalculator::radixSort(ParticleArrays &p) { buildTree(p); }
void BarnesHutForceCalculator::computeMassCOM(ParticleArrays &p) { buildTree(p); }

void BarnesHutForceCalculator::buildOctree(const uint32_t *, int, TreeArrays &, int *)
{
    // the octree is built from the engine's own 63-bit codes in buildTree
}

void BarnesHutForceCalculator::destroyTree() {}

// ------------------------------------------------------------ integrators
void EulerIntegrator::step(ForceCalculator &c, ParticleArrays &p, double dt)
{
    integrate(c, p, NB_EULER, dt, nullptr, &total_compute_time_ms);
}
std::string EulerIntegrator::name() const { return "Euler Integrator"; }

void EulerCromerIntegrator::step(ForceCalculator &c, ParticleArrays &p, double dt)
{
    integrate(c, p, NB_EULER_CROMER, dt, nullptr, &total_compute_time_ms);
}
std::string EulerCromerIntegrator::name() const { return "Euler-Cromer Integrator"; }

void LeapfrogIntegrator::step(ForceCalculator &c, ParticleArrays &p, double dt)
{
    integrate(c, p, NB_LEAPFROG, dt, &is_first_step, &total_compute_time_ms);
}
std::string LeapfrogIntegrator::name() const { return "Leapfrog Integrator"; }

void VelocityVerletIntegrator::step(ForceCalculator &c, ParticleArrays &p, double dt)
{
    integrate(c, p, NB_VELOCITY_VERLET, dt, &is_first_step, &total_compute_time_ms);
}
std::string VelocityVerletIntegrator::name() const { return "Velocity Verlet"; }

void RK4Integrator::step(ForceCalculator &c, ParticleArrays &p, double dt)
{
    integrate(c, p, NB_RK4, dt, nullptr, &total_compute_time_ms);
}
std::string RK4Integrator::name() const { return "RK4"; }
