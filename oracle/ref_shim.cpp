// ref_shim.cpp -- C entry points over the reference's own CPU classes.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh together with the
// reference's CPU sources (CPU/src/*.cpp of PawanKiitb/N-body-gravity-simulation,
// read in place) into oracle/_ref/libnbref.so.  The tests use it to check that
// the C restatement in nbody_oracle.c reproduces the reference bit for bit.
// Nothing here is part of the product.  G is the reference's constant::G
// (4 pi^2, CPU/include/common.hpp:28).
#include "tests_common.hpp"

#include <cstdint>
#include <vector>

namespace {

std::vector<Particle> make_particles(int n, const double *x, const double *y, const double *z,
                                     const double *vx, const double *vy, const double *vz,
                                     const double *m)
{
    std::vector<Particle> ps;
    ps.reserve(n);
    for (int i = 0; i < n; ++i)
        ps.emplace_back(m[i], Vector3D(x[i], y[i], z[i]),
                        Vector3D(vx ? vx[i] : 0.0, vy ? vy[i] : 0.0, vz ? vz[i] : 0.0));
    return ps;
}

void read_back(const std::vector<Particle> &ps, double *x, double *y, double *z, double *vx,
               double *vy, double *vz, double *ax, double *ay, double *az)
{
    for (size_t i = 0; i < ps.size(); ++i) {
        if (x) { x[i] = ps[i].position.x; y[i] = ps[i].position.y; z[i] = ps[i].position.z; }
        if (vx) { vx[i] = ps[i].velocity.x; vy[i] = ps[i].velocity.y; vz[i] = ps[i].velocity.z; }
        if (ax) { ax[i] = ps[i].acceleration.x; ay[i] = ps[i].acceleration.y; az[i] = ps[i].acceleration.z; }
    }
}

// Exposes the protected node pool of the reference's node-pool tree.
struct DumpableBH : public ForceCalculatorBarnesHutOptimized {
    using ForceCalculatorBarnesHutOptimized::ForceCalculatorBarnesHutOptimized;
    int dump(std::vector<Particle> &ps, int max_out, int *depth, int *count, int *is_leaf,
             int64_t *cx, int64_t *cy, int64_t *cz)
    {
        particles_ = &ps;
        buildTree(ps);
        int nn = (int)nextFreeNode;
        if (nn > max_out) return -1;
        std::vector<int> q{rootIndex}, dep(nn, 0), cnt(nn, 0);
        std::vector<int64_t> c(3 * (size_t)nn, 0);
        for (size_t h = 0; h < q.size(); ++h) {
            int v = q[h];
            const Node &nd = nodePool[v];
            if (nd.firstChild >= 0)
                for (int i = 0; i < 8; ++i) {
                    int k = nd.firstChild + i;
                    dep[k] = dep[v] + 1;
                    c[3 * k + 0] = 2 * c[3 * v + 0] + ((i & 1) ? 1 : 0);
                    c[3 * k + 1] = 2 * c[3 * v + 1] + ((i & 2) ? 1 : 0);
                    c[3 * k + 2] = 2 * c[3 * v + 2] + ((i & 4) ? 1 : 0);
                    q.push_back(k);
                }
        }
        for (size_t h = q.size(); h-- > 0;) {
            int v = q[h];
            const Node &nd = nodePool[v];
            if (nd.firstChild < 0) cnt[v] = (int)nd.particleIndices.size();
            else {
                int s = 0;
                for (int i = 0; i < 8; ++i) s += cnt[nd.firstChild + i];
                cnt[v] = s;
            }
        }
        for (int v = 0; v < nn; ++v) {
            depth[v] = dep[v];
            count[v] = cnt[v];
            is_leaf[v] = nodePool[v].firstChild < 0;
            cx[v] = c[3 * v + 0];
            cy[v] = c[3 * v + 1];
            cz[v] = c[3 * v + 2];
        }
        destroyTree();
        return nn;
    }
};

} // namespace

extern "C" {

double ref_G() { return constant::G; }

void ref_forces(int method, int n, const double *x, const double *y, const double *z,
                const double *m, double softening, double theta, int leaf_capacity, double *ax,
                double *ay, double *az)
{
    std::vector<Particle> ps = make_particles(n, x, y, z, nullptr, nullptr, nullptr, m);
    if (method == 0) {
        ForceCalculatorNaive c(softening);
        c.computeAccelerations(ps);
    } else if (method == 1) {
        ForceCalculatorBarnesHutOptimized c(softening, theta, leaf_capacity);
        c.computeAccelerations(ps);
    } else {
        ForceCalculatorBarnesHut c(softening, theta);
        c.computeAccelerations(ps);
    }
    read_back(ps, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, ax, ay, az);
}

// integrator: 0 Euler, 1 Euler-Cromer, 2 Leapfrog, 3 Velocity-Verlet, 4 RK4.
void ref_run(int integrator, int method, int n, double *x, double *y, double *z, double *vx,
             double *vy, double *vz, const double *m, double *ax, double *ay, double *az,
             double softening, double theta, int leaf_capacity, double dt, int nsteps)
{
    std::vector<Particle> ps = make_particles(n, x, y, z, vx, vy, vz, m);
    std::unique_ptr<TimeIntegrator> integ;
    switch (integrator) {
    case 0: integ = std::make_unique<EulerIntegrator>(); break;
    case 1: integ = std::make_unique<EulerCromerIntegrator>(); break;
    case 2: integ = std::make_unique<LeapfrogIntegrator>(); break;
    case 3: integ = std::make_unique<VelocityVerletIntegrator>(); break;
    default: integ = std::make_unique<RK4Integrator>(); break;
    }
    std::unique_ptr<ForceCalculator> calc;
    if (method == 0) calc = std::make_unique<ForceCalculatorNaive>(softening);
    else if (method == 1)
        calc = std::make_unique<ForceCalculatorBarnesHutOptimized>(softening, theta, leaf_capacity);
    else calc = std::make_unique<ForceCalculatorBarnesHut>(softening, theta);
    for (int s = 0; s < nsteps; ++s) integ->step(ps, *calc, dt);
    read_back(ps, x, y, z, vx, vy, vz, ax, ay, az);
}

// out: KE, PE (unsoftened), E, Lx, Ly, Lz, COMx, COMy, COMz
void ref_diagnostics(int n, const double *x, const double *y, const double *z, const double *vx,
                     const double *vy, const double *vz, const double *m, double *out)
{
    std::vector<Particle> ps = make_particles(n, x, y, z, vx, vy, vz, m);
    out[0] = kineticEnergy(ps);
    out[1] = potentialEnergy(ps);
    out[2] = totalEnergy(ps);
    Vector3D L = angularMomentum(ps);
    Vector3D c = centerOfMass(ps);
    out[3] = L.x; out[4] = L.y; out[5] = L.z;
    out[6] = c.x; out[7] = c.y; out[8] = c.z;
}

int ref_bh_opt_dump(int n, const double *x, const double *y, const double *z, const double *m,
                    int leaf_capacity, int max_out, int *depth, int *count, int *is_leaf,
                    int64_t *cx, int64_t *cy, int64_t *cz)
{
    std::vector<Particle> ps = make_particles(n, x, y, z, nullptr, nullptr, nullptr, m);
    DumpableBH bh(0.0, 0.5, leaf_capacity);
    return bh.dump(ps, max_out, depth, count, is_leaf, cx, cy, cz);
}

} // extern "C"
