/*
 * nbody_c.h -- C ABI of the GB300 N-body engine.
 *
 * This is the drop-in boundary for the force-and-step hot path of
 * PawanKiitb/N-body-gravity-simulation.  The reference has no C ABI; its
 * boundary is the C++ host API in CUDA/include/.  Each entry point below names
 * the reference interface it replaces.  The C++ classes of that API
 * (ParticleArrays, ForceCalculatorNaive, BarnesHutForceCalculator, the
 * integrators) are re-implemented on top of this ABI by the package's compat
 * layer.
 *
 * Conventions
 *   - Every function returns nb_status; nb_last_error() gives the message of
 *     the most recent failure on the calling thread.
 *   - Arrays are structure-of-arrays FP64, one value per body, as in the
 *     reference (ParticleArrays, CUDA/include/particle_data.hpp:6-43).
 *   - Work is enqueued on the simulation's CUDA stream (the `stream`
 *     argument of nb_create; NULL = the legacy default stream, which is what
 *     the reference uses).  Functions that return host data synchronise that
 *     stream; the others are asynchronous.  nb_synchronize() waits.
 *   - A simulation object is not thread-safe; distinct objects are.
 *   - No function prints or exits.  Kernels have no failure modes of their
 *     own: the Barnes-Hut walk is stackless and its node storage is sized to
 *     an upper bound of the node count before the build, so the reference's
 *     stack and node-pool overflows cannot occur; NB_ERR_DEVICE_FAULT is
 *     reserved for device-side checks.
 */
#ifndef NBODY_C_H
#define NBODY_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum nb_status {
    NB_OK = 0,
    NB_ERR_INVALID_ARGUMENT = 1,
    NB_ERR_CUDA = 2,
    NB_ERR_OUT_OF_MEMORY = 3,
    NB_ERR_CAPACITY = 4,     /* more bodies than the object was created for */
    NB_ERR_NOT_LOADED = 5,   /* no bodies loaded yet */
    NB_ERR_DEVICE_FAULT = 6, /* a kernel reported an error status */
    NB_ERR_UNSUPPORTED = 7,
    NB_ERR_IO = 8,           /* a file could not be opened, read, parsed or written */
    NB_ERR_CANCELLED = 9     /* a serving job was cancelled before it finished */
} nb_status;

/* Force methods.
 *   NB_DIRECT_FP64  : all-pairs sum in FP64 (the 1e-12 path; the reference's
 *                     computeAccelerationNaiveKernel, force_calculator_naive.cu:4-59).
 *   NB_DIRECT_MIXED : all-pairs sum with FP32 pair arithmetic on double-single
 *                     displacements, Kahan-compensated FP32 accumulation across
 *                     j-tiles, FP64 combine (the 1e-6 path).
 *   NB_BARNES_HUT   : 63-bit Morton octree, monopole, FP32 walk, FP64 result
 *                     (replaces BarnesHutForceCalculator, force_calculator_barnes_hut.cu). */
typedef enum nb_method {
    NB_DIRECT_FP64 = 0,
    NB_DIRECT_MIXED = 1,
    NB_BARNES_HUT = 2
} nb_method;

/* Integrators, the reference's TimeIntegrator family
 * (CUDA/include/integrator.hpp:7-17, CPU/src/integrator_rk4.cpp). */
typedef enum nb_integrator {
    NB_EULER = 0,
    NB_EULER_CROMER = 1,
    NB_LEAPFROG = 2,         /* kick-drift-kick */
    NB_VELOCITY_VERLET = 3,
    NB_RK4 = 4
} nb_integrator;

typedef struct nb_config {
    int method;         /* nb_method */
    double G;           /* gravitational constant; the reference uses 4 pi^2 */
    double softening;   /* epsilon (the pair term uses epsilon^2), ForceCalculator(double softening) */
    double theta;       /* Barnes-Hut opening angle, BarnesHutForceCalculator(.., theta, ..) */
    int leaf_capacity;  /* Barnes-Hut bodies per leaf (reference default 8) */
    int flags;          /* NB_FLAG_* */
} nb_config;

/* flags */
#define NB_FLAG_NONE 0
/* Bit 0 is reserved. */
#define NB_FLAG_RESERVED 1
/* Barnes-Hut tree reuse (bits 8-15): NB_FLAG_BH_REUSE(k), k >= 2, rebuilds the
 * tree every k force evaluations; the evaluations in between keep the last
 * build's topology and body order and refit monopoles and cell sides to the
 * current positions (a cell's side becomes the larger of its cube side and its
 * bodies' bounding-box extent, so a drifted cell opens at least as readily as
 * a rebuilt one).  k = 0 or 1 (the default) rebuilds at every evaluation, as
 * BarnesHutForceCalculator::computeAccelerations does
 * (CUDA/src/force_calculator_barnes_hut.cu:625-671).  A load, a configuration
 * change or a checkpoint restore forces a rebuild. */
#define NB_FLAG_BH_REUSE(k) (((k) & 0xff) << 8)
#define NB_FLAG_BH_REUSE_OF(flags) (((flags) >> 8) & 0xff)
/* Barnes-Hut quadrupole moments: an accepted cell acts as its monopole plus its
 * traceless quadrupole about the centre of mass (from FP64 prefix sums of the
 * second moments).  The opening test is unchanged, so at the same theta the
 * force error drops (the reference is monopole-only). */
#define NB_FLAG_BH_QUADRUPOLE 2
/* Barnes-Hut opening rule.  By default a node is opened when it holds the
 * body or fails the opening test size^2 >= theta^2 d^2 (d: body to centre of
 * mass).  With this flag the walk follows the reference's own rule
 * (CPU/src/force_calculator_barnes_hut_optimized.cpp walk and
 * CUDA/src/force_calculator_barnes_hut.cu:60-73): of every node it opens, the
 * child in the body's octant relative to the node's centre is opened too,
 * whether or not it holds the body.  That opens a chain of cells toward the
 * body below every opened node -- about 2.5 times the interactions at theta
 * 0.5 -- and gives the reference's accuracy at a given theta; the default is
 * faster and, at the same theta, less accurate.  The compat
 * BarnesHutForceCalculator sets it. */
#define NB_FLAG_BH_REFERENCE_OPENING 16
/* NB_DIRECT_MIXED kernel choice.  By default systems of at least 16,384 bodies
 * take the Hilbert-sorted near/far kernel (far j-chunks in plain FP32 relative to
 * a warp-local origin, the closest pairs in double-single) and smaller ones the
 * all-pairs double-single kernel; these flags force one or the other.  The
 * sorted kernel also holds every body to |da| <= 1e-6 |a| without the
 * conditioning clause of the all-pairs kernel.  Both kernels time their CTA
 * shapes on the first evaluation of each N in a process and keep the fastest;
 * the j-segments and the bodies per warp (which set the summation order) are
 * fixed by N alone, so results are bit-identical within a process and between
 * processes on the same GPU model. */
#define NB_FLAG_MIXED_SORTED 4
#define NB_FLAG_MIXED_UNSORTED 8

typedef struct nb_sim nb_sim;

/* Energies and moments of the current state, reduced on the GPU in FP64.
 * Replaces the host loops of CUDA/src/test_common.cpp:63-182. */
typedef struct nb_diag {
    double kinetic;            /* sum 1/2 m v^2 */
    double potential;          /* -G sum_{i<j} m_i m_j / r_ij (unsoftened, as the reference) */
    double potential_softened; /* -G sum_{i<j} m_i m_j / sqrt(r_ij^2 + eps^2): conserved when eps > 0 */
    double total;              /* kinetic + potential */
    double total_softened;     /* kinetic + potential_softened */
    double angular_momentum[3];
    double center_of_mass[3];
    double momentum[3];
    double mass;
} nb_diag;

/* ---- configuration and lifetime ---------------------------------------- */

/* G = 1, softening 0, theta 0.5, leaf capacity 8, method NB_DIRECT_MIXED. */
nb_status nb_config_default(nb_config *cfg);

/* Creates a simulation able to hold up to `capacity` bodies on the current
 * CUDA device.  Replaces allocateParticles (CUDA/src/particle_data.cu:6-43)
 * together with the calculator constructors. */
nb_status nb_create(const nb_config *cfg, size_t capacity, void *stream, nb_sim **out);

/* Replaces freeParticles (CUDA/src/particle_data.cu:46-92) and the calculator
 * destructors. */
nb_status nb_destroy(nb_sim *sim);

/* Changes method / G / softening / theta / leaf capacity between steps. */
nb_status nb_set_config(nb_sim *sim, const nb_config *cfg);
nb_status nb_get_config(const nb_sim *sim, nb_config *cfg);

/* ---- particle load and readback ---------------------------------------- */

/* Copies n bodies from host FP64 arrays; zeroes accelerations.  Replaces
 * copyParticlesToDevice (CUDA/src/particle_data.cu:95-119). */
nb_status nb_load(nb_sim *sim, size_t n, const double *x, const double *y, const double *z,
                  const double *vx, const double *vy, const double *vz, const double *m);

/* Same from device pointers (device-to-device copies). */
nb_status nb_load_device(nb_sim *sim, size_t n, const double *x, const double *y,
                         const double *z, const double *vx, const double *vy, const double *vz,
                         const double *m);

/* Makes the simulation work in place on ten caller-owned device arrays of n
 * doubles (x y z vx vy vz ax ay az m), as the reference's calculators and
 * integrators work on the caller's ParticleArrays
 * (CUDA/include/particle_data.hpp:6-43); NULL restores the simulation's own
 * storage.  The caller keeps the arrays alive while they are bound. */
nb_status nb_bind_device(nb_sim *sim, size_t n, double *const *arrays10);

/* Copies the state to host arrays; any pointer may be NULL to skip that
 * field.  Replaces copyParticlesToHost (CUDA/src/particle_data.cu:122-143). */
nb_status nb_read_state(nb_sim *sim, double *x, double *y, double *z, double *vx, double *vy,
                        double *vz, double *ax, double *ay, double *az, double *m);

/* Device pointers of the FP64 state arrays (valid until nb_destroy):
 * order x y z vx vy vz ax ay az m. */
nb_status nb_device_arrays(nb_sim *sim, double **ptrs10);

nb_status nb_num_bodies(const nb_sim *sim, size_t *n);

/* ---- hot path ----------------------------------------------------------- */

/* Accelerations of the current positions into the acceleration arrays.
 * Replaces ForceCalculator::computeAccelerations
 * (CUDA/include/force_calculator.hpp:24-26; force_calculator_naive.cu:61-92;
 * force_calculator_barnes_hut.cu:625-671). */
nb_status nb_compute_forces(nb_sim *sim);

/* nsteps steps of the integrator with time step dt.  Replaces
 * TimeIntegrator::step (CUDA/include/integrator.hpp:9-13).  Leapfrog and
 * velocity Verlet reuse the acceleration of the previous step when it is
 * still valid (as integrator_leafrog.cu:59-62 does with is_first_step);
 * Euler, Euler-Cromer and RK4 evaluate it at the start of every step. */
nb_status nb_step(nb_sim *sim, int integrator, double dt, int nsteps);

/* Marks the stored accelerations stale (after the caller edited positions
 * through nb_device_arrays). */
nb_status nb_invalidate_forces(nb_sim *sim);

nb_status nb_synchronize(nb_sim *sim);

/* ---- diagnostics --------------------------------------------------------- */

/* Replaces kineticEnergy / potentialEnergy / totalEnergy / angularMomentum /
 * centerOfMass (CUDA/src/test_common.cpp:63-182). */
nb_status nb_diagnostics(nb_sim *sim, nb_diag *out);

/* ---- Barnes-Hut introspection (tests and tools) -------------------------- */

typedef struct nb_bh_info {
    int num_nodes;
    int num_leaves;
    int max_depth;
    int split_levels;   /* levels the root cube may split (<= 21) */
    double root[4];     /* centre x, y, z and side of the root cube */
    uint64_t interactions_m2p;  /* body-node (monopole) terms of the last walk */
    uint64_t interactions_p2p;  /* body-body terms of the last walk (self included) */
    uint64_t interactions_total; /* all terms of every walk of this simulation */
} nb_bh_info;

/* Builds the tree of the current positions (without a walk) and reports it. */
nb_status nb_bh_build(nb_sim *sim, nb_bh_info *info);

/* Reports the tree and the interaction counts of the last Barnes-Hut force
 * evaluation (the reference prints build/walk times only). */
nb_status nb_bh_get_info(nb_sim *sim, nb_bh_info *info);

/* After nb_bh_build or a Barnes-Hut force evaluation: the sorted 63-bit
 * Morton codes and the original index of each sorted body (host arrays of
 * n entries; either may be NULL). */
nb_status nb_bh_read_order(nb_sim *sim, uint64_t *sorted_codes, uint32_t *order);

/* Node table in depth-first preorder, children in Morton order (host arrays
 * of max_nodes entries; any may be NULL): depth, Morton prefix (top 3*depth
 * bits), first sorted body, body count, leaf flag, skip (index of the next
 * node outside the subtree; the first child of an internal node is the next
 * index); com_mass gets 4 floats per node (COM xyz, mass).  Returns
 * NB_ERR_CAPACITY when max_nodes is smaller than the node count. */
nb_status nb_bh_read_nodes(nb_sim *sim, int max_nodes, int *depth, uint64_t *prefix,
                           int *first, int *count, int *is_leaf, int *skip, float *com_mass);

/* ---- batched ensemble ------------------------------------------------------ */

/* No counterpart in the reference (one system per process there).  Many
 * independent systems of uneven N, concatenated in system order, advanced
 * together: mixed-precision direct forces of all systems in one persistent
 * launch over a per-system work queue, per-body updates over the
 * concatenation, the step loop captured in a CUDA graph and replayed.  By
 * default every system is sorted along a Hilbert curve through its own cube
 * (at the start of each nb_ensemble_step call, every 25 steps within it, and
 * in nb_ensemble_compute_forces) and far 32-body chunks take the plain FP32
 * pair term, as in the single-system sorted kernel; cfg->flags
 * NB_FLAG_MIXED_UNSORTED selects the all-pairs kernel, whose i-bodies per lane
 * are autotuned per N bucket on the loaded systems at the first evaluation (or
 * by nb_ensemble_tune).  Either way a system's result does not depend on the
 * other systems of the ensemble. */
typedef struct nb_ensemble nb_ensemble;

typedef struct nb_ensemble_info_t {
    int num_systems;
    int64_t total_bodies;
    double interactions_per_eval;   /* sum over systems of n (n - 1) */
    int work_items;
    int ipt_by_bucket[32];          /* i-bodies per lane for n in [2^b, 2^(b+1)) */
    uint64_t graph_launches;        /* replays of the captured step loop so far */
    int graph_steps;                /* steps per replay */
    uint64_t force_launches;        /* timed force launches while profiling */
    double force_kernel_ms;         /* their summed device time */
} nb_ensemble_info_t;

/* cfg->method must be NB_DIRECT_MIXED.  stream NULL: the ensemble makes its
 * own (graph capture needs a stream other than the legacy default one). */
nb_status nb_ensemble_create(const nb_config *cfg, int num_systems, const int *sizes,
                             void *stream, nb_ensemble **out);
nb_status nb_ensemble_destroy(nb_ensemble *e);
/* Host arrays of sum(sizes) bodies, systems concatenated in order. */
nb_status nb_ensemble_load(nb_ensemble *e, const double *x, const double *y, const double *z,
                           const double *vx, const double *vy, const double *vz,
                           const double *m);
nb_status nb_ensemble_read_state(nb_ensemble *e, double *x, double *y, double *z, double *vx,
                                 double *vy, double *vz, double *ax, double *ay, double *az,
                                 double *m);
nb_status nb_ensemble_compute_forces(nb_ensemble *e);
nb_status nb_ensemble_step(nb_ensemble *e, int integrator, double dt, int nsteps);
nb_status nb_ensemble_tune(nb_ensemble *e, int *ipt_by_bucket /* 32 entries or NULL */);
nb_status nb_ensemble_synchronize(nb_ensemble *e);
nb_status nb_ensemble_info(nb_ensemble *e, nb_ensemble_info_t *info);
/* Times every force launch with events (and runs steps without the graph). */
nb_status nb_ensemble_profile(nb_ensemble *e, int enable);

/* ---- serving loop ------------------------------------------------------------ */

/* No counterpart in the reference.  A continuous-batching server for
 * simulation jobs: each nb_server_tick admits queued jobs while their device
 * memory fits the HBM budget, advances every running job by one leapfrog
 * step (direct jobs together in one batched launch over a resident body
 * pool, Barnes-Hut jobs on their own streams, overlapping), and retires jobs
 * that reached their step count.  A job's result does not depend on the other
 * jobs it ran with. */
typedef struct nb_server nb_server;

typedef struct nb_server_config {
    double G;
    double softening;
    double theta;            /* Barnes-Hut jobs */
    int leaf_capacity;       /* Barnes-Hut jobs */
    int direct_max_n;        /* jobs with n < direct_max_n use the direct sum */
    double dt;               /* leapfrog step */
    size_t hbm_budget_bytes; /* device memory for job state, pool included */
    size_t pool_bodies;      /* capacity of the direct-job body pool */
} nb_server_config;

typedef struct nb_server_stats {
    uint64_t jobs_submitted, jobs_finished;
    int jobs_running, jobs_queued;
    uint64_t steps_done, ticks;
    double interactions;     /* pair (direct) + body-node and body-body (tree) terms */
    double busy_ms;          /* sum of tick device times */
    double step_ms_p50, step_ms_p99;   /* per job step: tick start -> step complete */
    double queue_ms_p50, queue_ms_p99; /* submission -> admission (wall clock) */
    int max_running;
    size_t peak_device_bytes;
    /* host wall time per tick phase, summed: admitting jobs (allocation and
     * upload), issuing the step (Barnes-Hut threads joined), waiting for the
     * device, retiring finished jobs (download and release) */
    double host_admit_ms, host_issue_ms, host_wait_ms, host_retire_ms;
    /* parts of host_issue_ms: rebuilding the direct work queue, issuing the
     * direct batch, waiting for the Barnes-Hut stream threads */
    double host_upload_ms, host_direct_ms, host_join_ms;
    /* jobs that ended without a result: a failure of their own (an allocation
     * or launch error while admitting or stepping them; the other jobs carry
     * on) or nb_server_cancel */
    uint64_t jobs_failed, jobs_cancelled;
} nb_server_stats;

/* G 1, softening 1e-3, theta 0.6, leaf 8, direct below 16384 bodies, dt 1e-3,
 * 16 GiB budget, 4 Mi-body pool. */
nb_status nb_server_config_default(nb_server_config *cfg);
nb_status nb_server_create(const nb_server_config *cfg, nb_server **out);
nb_status nb_server_destroy(nb_server *s);
/* Copies the host arrays; the job waits in the queue until admitted. */
nb_status nb_server_submit(nb_server *s, size_t n, const double *x, const double *y,
                           const double *z, const double *vx, const double *vy,
                           const double *vz, const double *m, int steps, int64_t *job_id);
/* Admits what fits, advances every running job one step, retires finished
 * jobs.  A failure that belongs to one Barnes-Hut job (its allocation, load or
 * step returned an error) ends that job alone -- its result then reports the
 * error -- and the tick still returns NB_OK; a failure of the shared direct
 * batch or of the device fails the tick. */
nb_status nb_server_tick(nb_server *s, int *running, int *queued);
/* State of a finished job (NB_ERR_NOT_LOADED until it finished; a job that
 * failed returns the status it failed with, its message in nb_last_error();
 * a cancelled one NB_ERR_CANCELLED). */
nb_status nb_server_result(nb_server *s, int64_t job_id, double *x, double *y, double *z,
                           double *vx, double *vy, double *vz, double *ax, double *ay,
                           double *az, double *m);
/* Drops a finished job's stored result. */
nb_status nb_server_release(nb_server *s, int64_t job_id);
/* Cancels a queued or running job between ticks: its device memory and pool
 * slot are freed at once and its result becomes NB_ERR_CANCELLED.  A job that
 * already finished, or an unknown id, is NB_ERR_INVALID_ARGUMENT. */
nb_status nb_server_cancel(nb_server *s, int64_t job_id);
nb_status nb_server_get_stats(nb_server *s, nb_server_stats *out);

/* ---- host-side input generators (no GPU needed) ------------------------- */

/* Equal-mass Plummer sphere (total mass M, scale radius a, G), positions and
 * velocities by the Aarseth-Henon-Wielen (1974) construction, centred on the
 * centre of mass.  Random numbers: SplitMix64 keyed by (seed, body, draw). */
nb_status nb_gen_plummer(size_t n, uint64_t seed, double total_mass, double scale, double G,
                         double *x, double *y, double *z, double *vx, double *vy, double *vz,
                         double *m);

/* Bulge (Plummer, mass fraction bulge_frac, scale bulge_scale) plus an
 * exponential disk (scale length disk_scale, sech^2 height disk_height) with
 * circular velocities from the enclosed mass plus isotropic dispersion
 * `dispersion` (in units of the local circular speed). */
nb_status nb_gen_disk_bulge(size_t n, uint64_t seed, double total_mass, double bulge_frac,
                            double bulge_scale, double disk_scale, double disk_height,
                            double dispersion, double G, double *x, double *y, double *z,
                            double *vx, double *vy, double *vz, double *m);

/* ---- files: particle lists, trajectory CSV, checkpoints (host side) ---------- */

/* Reads the reference's particle file, the format its test loader parses
 * (CUDA/tests/test3_correctness.cu:16-38, fixtures particles_{100..10000}.txt):
 * the body count N, then N records "m x y z vx vy vz", whitespace-separated.
 * With m == NULL only *n is set (a size query).  Otherwise every array must
 * hold `capacity` >= N doubles.  Errors: NB_ERR_IO (missing or malformed
 * file), NB_ERR_CAPACITY. */
nb_status nb_particles_read(const char *path, size_t capacity, size_t *n, double *m, double *x,
                            double *y, double *z, double *vx, double *vy, double *vz);
/* Writes the same format, 17 significant digits (reads back bit-exactly). */
nb_status nb_particles_write(const char *path, size_t n, const double *m, const double *x,
                             const double *y, const double *z, const double *vx,
                             const double *vy, const double *vz);
/* nb_particles_read into the simulation (nb_load of the file's bodies). */
nb_status nb_load_particles(nb_sim *sim, const char *path);

/* Appends one row of the reference's trajectory CSV (CPU/src/n-body.cpp:6-58,
 * CPU/orbit.csv): the x y z of each listed body, then kinetic, potential
 * (unsoftened) and total energy, angular momentum x y z and centre of mass
 * x y z of the simulation's current state (nb_diagnostics).  header != 0
 * first writes the header line: "<name>_x,<name>_y,<name>_z" per listed body,
 * then kinetic_energy,...,center_of_mass_z.  precision < 0 prints numbers as a
 * default C++ stream does (6 significant digits, %g); precision >= 0 prints
 * them fixed with that many decimals (the reference writes its first row the
 * first way and every later row with 15).  The file is created if missing. */
nb_status nb_csv_append(nb_sim *sim, const char *path, int nbodies, const int *bodies,
                        const char *const *names, int header, int precision);

/* Binary checkpoint of a simulation: configuration, body count, whether the
 * stored accelerations are those of the stored positions (leapfrog and
 * velocity Verlet then continue without a new force evaluation, as the
 * reference's integrators do after their first step), and the ten FP64
 * planes x y z vx vy vz ax ay az m.  Layout: 8-byte magic "NBGB3CK1", uint32
 * version 1, uint32 forces_valid, uint64 n, nb_config, then the planes
 * (native byte order).  No reference counterpart (the reference keeps no
 * state on disk). */
nb_status nb_checkpoint_save(nb_sim *sim, const char *path);
/* Restores configuration, state and the accelerations flag; n must fit the
 * simulation's capacity.  Continuing after a restore gives the same bits as
 * continuing the saved run for the FP64 and Barnes-Hut methods and for the
 * mixed method on its all-pairs kernel; the sorted kernel (NB_FLAG_MIXED_SORTED,
 * the default from 16,384 bodies) sums in the order of its last Hilbert sort,
 * which a restore into another simulation does not carry over (results stay
 * within tolerance). */
nb_status nb_checkpoint_load(nb_sim *sim, const char *path);

/* ---- all-pairs forces without device allocation ----------------------------- */

/* No counterpart in the reference: an addition of this library for callers
 * that may not allocate device memory (a host whose device memory is owned by
 * its own pool allocator, a plugin with a fixed device-memory budget, a loop
 * that cannot take the implicit synchronisation of cudaMalloc/cudaFree).
 * Computes G-scaled accelerations of n bodies with the all-pairs mixed kernels
 * (split, all-pairs sum, combine) from caller-owned DEVICE arrays x, y, z, m
 * into caller-owned DEVICE arrays ax, ay, az, on `stream` (NULL = legacy
 * default stream), asynchronously.  It never runs the Hilbert-sorted kernel
 * that NB_DIRECT_MIXED uses from 16,384 bodies, never autotunes, and caps its
 * j-split to fit its scratch, so it agrees with NB_DIRECT_MIXED to the
 * mixed-path tolerance; its bits equal those of an NB_DIRECT_MIXED evaluation
 * only when both run the same plan (the all-pairs kernel with autotuning off,
 * NB_AUTOTUNE=0, and n small enough that the j-split is not capped, about
 * n < 150,000).  It allocates nothing: its scratch is one 16 MiB array in the
 * library's device memory, present on every device that loads the library
 * until the process exits, which limits n to 262144 (larger n returns
 * NB_ERR_CAPACITY).  The first call on each device looks up that array's
 * device address (cudaGetSymbolAddress) and must run with that device current
 * and before any stream capture; the address is kept for the life of the
 * process, so the entry point must not be used on a device after
 * cudaDeviceReset.  All calls share the array: calls whose work overlaps on
 * the GPU race and must be serialised by the caller. */
nb_status nb_direct_mixed_forces_noalloc(size_t n, const double *x, const double *y,
                                         const double *z, const double *m, double G,
                                         double softening, double *ax, double *ay, double *az,
                                         void *stream);

/* ---- measurement ---------------------------------------------------------- */

/* Device time of the dominant force kernel (the all-pairs kernel or the tree
 * walk) of every evaluation while profiling is enabled, from CUDA events
 * recorded on the simulation's stream around that launch.  The reference
 * keeps the same totals in its calculators (getTotalComputeTime,
 * force_calculator_naive.hpp:23-25), but synchronises after every call. */
typedef struct nb_profile {
    uint64_t kernel_launches;  /* this library's kernel launches in the process so far */
    uint64_t force_launches;   /* timed force-kernel launches since the last reset */
    double force_kernel_ms;    /* their summed device time */
} nb_profile;

nb_status nb_profile_enable(nb_sim *sim, int enable);
/* Synchronises the stream; reset != 0 starts a new window. */
nb_status nb_profile_read(nb_sim *sim, nb_profile *out, int reset);
/* Process-wide count of kernel launches made by this library. */
uint64_t nb_kernel_launch_count(void);

/* ---- errors --------------------------------------------------------------- */

const char *nb_status_string(nb_status s);
const char *nb_last_error(void);

/* Library version string. */
const char *nb_version(void);

/* Test hook for failure handling (host side only: no CUDA call fails and the
 * device is untouched).  After `after` more successful device allocations by
 * this library, in any object of the process, the next one fails with
 * NB_ERR_OUT_OF_MEMORY and the message "injected allocation failure"; the hook
 * then disarms.  A negative value disarms it. */
nb_status nb_debug_fail_device_allocations(int after);

/* Device-side index checks.  *enabled (if not NULL) is 1 in a library built
 * with them (build.py --checks: every kernel tests the indices it is about to
 * use and skips an out-of-range access instead of making it), else 0.  Returns
 * NB_ERR_DEVICE_FAULT with the source line, index and bound of the first
 * failed check since the last call (and clears them), else NB_OK. */
nb_status nb_debug_device_checks(int *enabled);

/* Measured FP32-pipe rate of the current device: a register-only kernel of
 * independent packed (f32x2) FMAs on every SM, best of three timed launches;
 * *lane_ops_per_s = FMA lane operations per second.  A measured denominator for
 * the FP32 rooflines of the force kernels, beside the lanes x clock figure.
 * Runs on the legacy default stream and waits for it (about 1 ms).
 * Not a reference call: benchmark support. */
nb_status nb_debug_fp32_rate(double *lane_ops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* NBODY_C_H */
