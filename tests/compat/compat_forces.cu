// compat_forces.cu -- uses the reference's CUDA host API, as implemented by
// libnbody_compat.so, the way the reference's force benchmark does
// (CUDA/tests/test2_ForceBenchmark.cu): a uniform cube drawn from
// std::mt19937(seed) in x, y, z, mass order, the all-pairs and Barnes-Hut
// calculators, readback with copyParticlesToHost.  Writes n, the inputs and
// both acceleration sets as raw doubles to argv[3].
#include "force_calculator_barnes_hut.hpp"
#include "force_calculator_naive.hpp"

#include <cstdio>
#include <random>
#include <vector>

int main(int argc, char **argv)
{
    if (argc < 4) return 2;
    const int n = std::atoi(argv[1]);
    const unsigned seed = (unsigned)std::atoi(argv[2]);
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> position(-100.0, 100.0), massDist(0.5, 2.0);
    std::vector<double> x(n), y(n), z(n), vx(n, 0.0), vy(n, 0.0), vz(n, 0.0), m(n);
    for (int i = 0; i < n; ++i) {
        x[i] = position(rng);
        y[i] = position(rng);
        z[i] = position(rng);
        m[i] = massDist(rng);
    }
    ParticleArrays p;
    allocateParticles(p, n);
    copyParticlesToDevice(p, x.data(), y.data(), z.data(), vx.data(), vy.data(), vz.data(),
                          m.data());
    std::vector<double> t(n), a1(3 * n), a2(3 * n);
    ForceCalculatorNaive naive(0.0);
    naive.computeAccelerations(p);
    copyParticlesToHost(p, t.data(), t.data(), t.data(), t.data(), t.data(), t.data(), a1.data(),
                        a1.data() + n, a1.data() + 2 * n, t.data());
    BarnesHutForceCalculator bh(0.0, 0.5);
    for (int k = 0; k < 3; ++k) bh.computeAccelerations(p);
    copyParticlesToHost(p, t.data(), t.data(), t.data(), t.data(), t.data(), t.data(), a2.data(),
                        a2.data() + n, a2.data() + 2 * n, t.data());
    FILE *f = std::fopen(argv[3], "wb");
    if (!f) return 3;
    const double dn = n;
    std::fwrite(&dn, sizeof(double), 1, f);
    for (auto *v : {&x, &y, &z, &m, &a1, &a2}) std::fwrite(v->data(), sizeof(double), v->size(), f);
    const double times[4] = {naive.getTotalComputeTime(), bh.getTotalComputeTime(),
                             bh.getBuildTreeTime(), bh.getTraversalTime()};
    std::fwrite(times, sizeof(double), 4, f);
    std::fclose(f);
    freeParticles(p);
    std::printf("%s %s %.3f ms, %s %.3f ms (build %.3f, walk %.3f)\n", naive.name().c_str(), "",
                times[0], bh.name().c_str(), times[1], times[2], times[3]);
    return 0;
}
