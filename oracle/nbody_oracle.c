/*
 * nbody_oracle.c -- CPU restatement of the reference's force-and-step path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: it is linked by the tests,
 * by the package's smoke check and by the CPU-baseline leg of the benchmark, and
 * nowhere else.  The GPU product never calls it.
 *
 * Every routine restates, in plain C and FP64, the arithmetic of the reference
 * (PawanKiitb/N-body-gravity-simulation) in the same operation order, so that
 * with -ffp-contract=off the results are bit-identical to the reference's own
 * CPU build.  The parity of this restatement is pinned two ways (see the tests):
 *   - against the reference's published seed-42 error tables
 *     (CPU/outputs/output2_4.txt) and the Earth-Sun trajectory CPU/orbit.csv;
 *   - against the reference's CPU sources compiled in this checkout
 *     (oracle/_ref, built by oracle/build_ref.sh when the sources are present).
 *
 * Units: G is a parameter (the reference hard-codes G = 4 pi^2,
 * CPU/include/common.hpp:28; the Plummer/disk workloads use G = 1).
 *
 * Sections:
 *   1. MT19937 + libstdc++ uniform_real_distribution (input generation of the
 *      reference's tests, CPU/tests/test2_ForceBenchmark.cpp:8,20-21,46-58).
 *   2. Direct FP64 sum           CPU/src/force_calculator_naive.cpp:3-35
 *   3. Node-pool Barnes-Hut      CPU/src/force_calculator_barnes_hut_optimized.cpp:6-236
 *   4. Pointer Barnes-Hut        CPU/src/force_calculator_barnes_hut.cpp:5-217
 *   5. Integrators               CPU/src/integrator_{euler,euler-cromer,leapfrog,
 *                                velocity_verlet,rk4}.cpp
 *   6. Diagnostics               CPU/include/tests_common.hpp:33-101
 *   7. The 63-bit Morton / sort / octree topology rule that the GPU Barnes-Hut
 *      build must reproduce bit for bit.  It generalises
 *      CUDA/src/force_calculator_barnes_hut.cu:217-251 (Morton interleave,
 *      x in the high bit of each triple) to 21 bits per axis, and takes the
 *      root cube and the per-level cell split from the CPU tree
 *      (CPU/src/force_calculator_barnes_hut_optimized.cpp:105-124,206-231), so
 *      that the octree it describes is the CPU tree's set of non-empty cells.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_API __attribute__((visibility("default")))

static void orc_set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

ORC_API int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* 1. MT19937 (Matsumoto & Nishimura 1998) and libstdc++'s                   */
/*    generate_canonical<double,53> / uniform_real_distribution<double>.     */
/* ------------------------------------------------------------------------- */
typedef struct {
    uint32_t mt[624];
    int idx;
} orc_mt;

ORC_API size_t orc_mt_size(void) { return sizeof(orc_mt); }

ORC_API void orc_mt_seed(orc_mt *g, uint32_t seed)
{
    g->mt[0] = seed;
    for (int i = 1; i < 624; ++i)
        g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->idx = 624;
}

static void orc_mt_twist(orc_mt *g)
{
    for (int i = 0; i < 624; ++i) {
        uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
        uint32_t v = g->mt[(i + 397) % 624] ^ (y >> 1);
        if (y & 1u) v ^= 0x9908b0dfu;
        g->mt[i] = v;
    }
    g->idx = 0;
}

ORC_API uint32_t orc_mt_u32(orc_mt *g)
{
    if (g->idx >= 624) orc_mt_twist(g);
    uint32_t y = g->mt[g->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* generate_canonical with a 32-bit engine and 53 bits: two draws, the first
 * one in the low word; the sum is formed in double, divided by 2^64, and a
 * result that rounds up to 1 is replaced by the largest double below 1. */
ORC_API double orc_mt_canonical(orc_mt *g)
{
    double sum = 0.0, tmp = 1.0;
    for (int k = 0; k < 2; ++k) {
        sum += (double)orc_mt_u32(g) * tmp;
        tmp *= 4294967296.0;
    }
    double r = sum / tmp;
    if (r >= 1.0) r = nextafter(1.0, 0.0);
    return r;
}

ORC_API double orc_mt_uniform(orc_mt *g, double a, double b)
{
    return orc_mt_canonical(g) * (b - a) + a;
}

/* Uniform cube of the reference's force benchmark: position U(-100,100)^3,
 * mass U(0.5,2), zero velocity.
 * order == 0: CPU test order.  CPU/tests/test2_ForceBenchmark.cpp:48-57 passes
 *   mass(rng) and Vector3D(position(rng) x3) as constructor arguments; g++
 *   evaluates those right to left, so the draws are z, y, x, then mass.
 * order == 1: CUDA test order, CUDA/tests/test2_ForceBenchmark.cu:61-67:
 *   x, y, z, mass in statement order. */
ORC_API void orc_gen_uniform_cube(orc_mt *g, int n, int order,
                                  double *x, double *y, double *z, double *m)
{
    for (int i = 0; i < n; ++i) {
        if (order == 0) {
            z[i] = orc_mt_uniform(g, -100.0, 100.0);
            y[i] = orc_mt_uniform(g, -100.0, 100.0);
            x[i] = orc_mt_uniform(g, -100.0, 100.0);
            m[i] = orc_mt_uniform(g, 0.5, 2.0);
        } else {
            x[i] = orc_mt_uniform(g, -100.0, 100.0);
            y[i] = orc_mt_uniform(g, -100.0, 100.0);
            z[i] = orc_mt_uniform(g, -100.0, 100.0);
            m[i] = orc_mt_uniform(g, 0.5, 2.0);
        }
    }
}

/* ------------------------------------------------------------------------- */
/* 2. Direct FP64 sum, CPU/src/force_calculator_naive.cpp:9-30.              */
/*    a_i = sum_{j != i} r_ij * (G * m_j * (1/sqrt(r_ij.r_ij + eps2))^3)     */
/* ------------------------------------------------------------------------- */
ORC_API void orc_forces_naive(int n, const double *x, const double *y, const double *z,
                              const double *m, double G, double eps2,
                              double *ax, double *ay, double *az, int nthreads)
{
    orc_set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        const double xi = x[i], yi = y[i], zi = z[i];
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            double rx = x[j] - xi, ry = y[j] - yi, rz = z[j] - zi;
            double d2 = rx * rx + ry * ry + rz * rz + eps2;
            double inv = 1 / sqrt(d2);
            double inv3 = inv * inv * inv;
            double f = G * m[j] * inv3;
            sx += rx * f;
            sy += ry * f;
            sz += rz * f;
        }
        ax[i] = sx;
        ay[i] = sy;
        az[i] = sz;
    }
}

/* Sum of the magnitudes of the pair terms, s_i = sum_{j != i} |G m_j r_ij| /
 * (r_ij^2 + eps2)^(3/2): the scale of the rounding error of any finite-precision
 * evaluation of a_i.  s_i / |a_i| is the condition number of body i's sum (not a
 * reference quantity: used by the tests to state error bounds). */
ORC_API void orc_forces_naive_abs(int n, const double *x, const double *y, const double *z,
                                  const double *m, double G, double eps2, double *sabs,
                                  int nthreads)
{
    orc_set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            double rx = x[j] - x[i], ry = y[j] - y[i], rz = z[j] - z[i];
            double r2 = rx * rx + ry * ry + rz * rz;
            double d2 = r2 + eps2;
            s += G * m[j] * sqrt(r2) / (d2 * sqrt(d2));
        }
        sabs[i] = s;
    }
}

/* Rows [i0, i1) of the direct sum (the bounded CPU-baseline sample). */
ORC_API void orc_forces_naive_rows(int n, int i0, int i1, const double *x, const double *y,
                                   const double *z, const double *m, double G, double eps2,
                                   double *ax, double *ay, double *az, int nthreads)
{
    orc_set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int i = i0; i < i1; ++i) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        const double xi = x[i], yi = y[i], zi = z[i];
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            double rx = x[j] - xi, ry = y[j] - yi, rz = z[j] - zi;
            double d2 = rx * rx + ry * ry + rz * rz + eps2;
            double inv = 1 / sqrt(d2);
            double inv3 = inv * inv * inv;
            double f = G * m[j] * inv3;
            sx += rx * f;
            sy += ry * f;
            sz += rz * f;
        }
        ax[i - i0] = sx;
        ay[i - i0] = sy;
        az[i - i0] = sz;
    }
}

/* ------------------------------------------------------------------------- */
/* 3. Node-pool Barnes-Hut with a leaf capacity,                             */
/*    CPU/src/force_calculator_barnes_hut_optimized.cpp.                     */
/*    Octant bits x=1, y=2, z=4 (:75-77); root cube centred on the bounding  */
/*    box, side = max extent + 1e-9 (:117-124); a full leaf splits on the    */
/*    next insertion unless the half size is below 1e-9 (:138-173,206-211).  */
/*    COM is updated incrementally on every insertion (:133-134).            */
/* ------------------------------------------------------------------------- */
typedef struct {
    double cx, cy, cz;
    double size, size_sqr;
    double mass;
    double comx, comy, comz;
    int first_child;
    int np, cap;
    int *idx;
} orc_pnode;

typedef struct {
    orc_pnode *pool;
    int nnodes, max_nodes;
    const double *x, *y, *z, *m;
    int leaf_capacity;
    double epsilon;
} orc_ptree;

static int orc_ptree_alloc(orc_ptree *t)
{
    if (t->nnodes >= t->max_nodes) return -1;
    orc_pnode *nd = &t->pool[t->nnodes];
    free(nd->idx);
    memset(nd, 0, sizeof(*nd));
    nd->first_child = -1;
    return t->nnodes++;
}

static void orc_pnode_push(orc_pnode *nd, int p)
{
    if (nd->np == nd->cap) {
        nd->cap = nd->cap ? 2 * nd->cap : 8;
        nd->idx = (int *)realloc(nd->idx, sizeof(int) * (size_t)nd->cap);
    }
    nd->idx[nd->np++] = p;
}

static int orc_ptree_subdivide(orc_ptree *t, int ni)
{
    double half = t->pool[ni].size / 2.0;
    if (half < t->epsilon) return 0;
    t->pool[ni].first_child = t->nnodes;
    for (int i = 0; i < 8; ++i) {
        int c = orc_ptree_alloc(t);
        if (c < 0) return -1;
        orc_pnode *ch = &t->pool[c];
        const orc_pnode *nd = &t->pool[ni];
        ch->size = half;
        ch->size_sqr = half * half;
        double ox = (i & 1) ? half / 2.0 : -half / 2.0;
        double oy = (i & 2) ? half / 2.0 : -half / 2.0;
        double oz = (i & 4) ? half / 2.0 : -half / 2.0;
        ch->cx = nd->cx + ox;
        ch->cy = nd->cy + oy;
        ch->cz = nd->cz + oz;
    }
    return 1;
}

static int orc_octant_xlow(double px, double py, double pz, const orc_pnode *nd)
{
    int c = 0;
    if (px >= nd->cx) c |= 1;
    if (py >= nd->cy) c |= 2;
    if (pz >= nd->cz) c |= 4;
    return c;
}

static int orc_ptree_insert(orc_ptree *t, int ni, int p)
{
    orc_pnode *nd = &t->pool[ni];
    const double mp = t->m[p], px = t->x[p], py = t->y[p], pz = t->z[p];
    nd->mass += mp;
    {
        double w = nd->mass - mp;
        nd->comx = (nd->comx * w + px * mp) / nd->mass;
        nd->comy = (nd->comy * w + py * mp) / nd->mass;
        nd->comz = (nd->comz * w + pz * mp) / nd->mass;
    }
    if (nd->first_child == -1) {
        if (nd->np < t->leaf_capacity) {
            orc_pnode_push(nd, p);
            return 0;
        }
        int s = orc_ptree_subdivide(t, ni);
        nd = &t->pool[ni];
        if (s < 0) return -1;
        if (s == 0) {
            orc_pnode_push(nd, p);
            return 0;
        }
        int *old = nd->idx;
        int nold = nd->np;
        nd->idx = NULL;
        nd->np = nd->cap = 0;
        for (int k = 0; k < nold; ++k) {
            int q = old[k];
            const orc_pnode *nn = &t->pool[ni];
            int c = orc_octant_xlow(t->x[q], t->y[q], t->z[q], nn);
            if (orc_ptree_insert(t, nn->first_child + c, q) < 0) {
                free(old);
                return -1;
            }
        }
        free(old);
        const orc_pnode *nn = &t->pool[ni];
        int c = orc_octant_xlow(px, py, pz, nn);
        return orc_ptree_insert(t, nn->first_child + c, p);
    }
    int c = orc_octant_xlow(px, py, pz, nd);
    return orc_ptree_insert(t, nd->first_child + c, p);
}

static void orc_ptree_free(orc_ptree *t)
{
    if (!t->pool) return;
    for (int i = 0; i < t->max_nodes; ++i) free(t->pool[i].idx);
    free(t->pool);
    t->pool = NULL;
}

/* Builds the node-pool tree.  Returns the node count, or -1 when max_nodes
 * is exceeded (the reference asserts, :188-193). */
static int orc_ptree_build(orc_ptree *t, int n, const double *x, const double *y,
                           const double *z, const double *m, int leaf_capacity, int max_nodes)
{
    memset(t, 0, sizeof(*t));
    t->x = x; t->y = y; t->z = z; t->m = m;
    t->leaf_capacity = leaf_capacity;
    t->epsilon = 1e-9;
    t->max_nodes = max_nodes;
    t->pool = (orc_pnode *)calloc((size_t)max_nodes, sizeof(orc_pnode));
    if (n <= 0) return 0;
    double minx = DBL_MAX, miny = DBL_MAX, minz = DBL_MAX;
    double maxx = -DBL_MAX, maxy = -DBL_MAX, maxz = -DBL_MAX;
    for (int i = 0; i < n; ++i) {
        /* std::min(a,b) = (b < a) ? b : a ; std::max(a,b) = (a < b) ? b : a */
        minx = (x[i] < minx) ? x[i] : minx;
        maxx = (maxx < x[i]) ? x[i] : maxx;
        miny = (y[i] < miny) ? y[i] : miny;
        maxy = (maxy < y[i]) ? y[i] : maxy;
        minz = (z[i] < minz) ? z[i] : minz;
        maxz = (maxz < z[i]) ? z[i] : maxz;
    }
    double ey = maxy - miny, ez = maxz - minz, ex = maxx - minx;
    double eyz = (ey < ez) ? ez : ey;
    double size = (ex < eyz) ? eyz : ex;
    size += t->epsilon;
    int root = orc_ptree_alloc(t);
    t->pool[root].cx = (minx + maxx) / 2;
    t->pool[root].cy = (miny + maxy) / 2;
    t->pool[root].cz = (minz + maxz) / 2;
    t->pool[root].size = size;
    t->pool[root].size_sqr = size * size;
    for (int i = 0; i < n; ++i)
        if (orc_ptree_insert(t, root, i) < 0) return -1;
    return t->nnodes;
}

static void orc_ptree_walk(const orc_ptree *t, int p, double G, double eps2, double theta_sqr,
                           double *oax, double *oay, double *oaz)
{
    const double px = t->x[p], py = t->y[p], pz = t->z[p];
    double ax = 0.0, ay = 0.0, az = 0.0;
    int stack[64];
    int top = 0;
    stack[top++] = 0;
    while (top > 0) {
        const orc_pnode *nd = &t->pool[stack[--top]];
        if (nd->first_child == -1) {
            for (int k = 0; k < nd->np; ++k) {
                int q = nd->idx[k];
                if (q == p) continue;
                double rx = t->x[q] - px, ry = t->y[q] - py, rz = t->z[q] - pz;
                double d2 = rx * rx + ry * ry + rz * rz + eps2;
                double inv = 1.0 / sqrt(d2);
                double inv3 = inv * inv * inv;
                double s = t->m[q] * inv3;
                ax += (rx * G) * s;
                ay += (ry * G) * s;
                az += (rz * G) * s;
            }
            continue;
        }
        int cc = orc_octant_xlow(px, py, pz, nd);
        const orc_pnode *ch = &t->pool[nd->first_child];
        for (int i = 0; i < 8; ++i) {
            if (i == cc) {
                stack[top++] = nd->first_child + i;
                continue;
            }
            double rx = ch[i].comx - px, ry = ch[i].comy - py, rz = ch[i].comz - pz;
            double d2 = rx * rx + ry * ry + rz * rz;
            if (ch[i].size_sqr < theta_sqr * d2) {
                double d2s = d2 + eps2;
                double inv = 1.0 / sqrt(d2s);
                double inv3 = inv * inv * inv;
                double s = ch[i].mass * inv3;
                ax += (rx * G) * s;
                ay += (ry * G) * s;
                az += (rz * G) * s;
            } else {
                stack[top++] = nd->first_child + i;
            }
        }
    }
    *oax = ax;
    *oay = ay;
    *oaz = az;
}

/* Returns the node count, or -1 if the node pool overflowed. */
ORC_API int orc_forces_bh_opt(int n, const double *x, const double *y, const double *z,
                              const double *m, double G, double eps2, double theta,
                              int leaf_capacity, double *ax, double *ay, double *az,
                              int nthreads)
{
    orc_ptree t;
    int max_nodes = 8 * n + 64;
    if (max_nodes < 1000) max_nodes = 1000;
    int nn = orc_ptree_build(&t, n, x, y, z, m, leaf_capacity, max_nodes);
    if (nn < 0) {
        orc_ptree_free(&t);
        return -1;
    }
    double theta_sqr = theta * theta;
    orc_set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) orc_ptree_walk(&t, i, G, eps2, theta_sqr, &ax[i], &ay[i], &az[i]);
    orc_ptree_free(&t);
    return nn;
}

/* Node dump of the node-pool tree, for the topology comparison: for every
 * node, its depth, particle count (bodies under it), leaf flag and the
 * per-axis cell index at its depth relative to the root cube (x, y, z, each
 * in [0, 2^depth)).  Returns the node count or -1. */
ORC_API int orc_bh_opt_dump(int n, const double *x, const double *y, const double *z,
                            const double *m, int leaf_capacity, int max_out, int *depth,
                            int *count, int *is_leaf, int64_t *cell_x, int64_t *cell_y,
                            int64_t *cell_z)
{
    orc_ptree t;
    int max_nodes = 8 * n + 64;
    if (max_nodes < 1000) max_nodes = 1000;
    int nn = orc_ptree_build(&t, n, x, y, z, m, leaf_capacity, max_nodes);
    if (nn < 0 || nn > max_out) {
        orc_ptree_free(&t);
        return -1;
    }
    /* BFS from the root assigning depth / cell coordinates; count bodies. */
    int *queue = (int *)malloc(sizeof(int) * (size_t)nn);
    int *cnt = (int *)calloc((size_t)nn, sizeof(int));
    int64_t *cxs = (int64_t *)calloc((size_t)nn * 3, sizeof(int64_t));
    int *dep = (int *)calloc((size_t)nn, sizeof(int));
    int head = 0, tail = 0;
    queue[tail++] = 0;
    while (head < tail) {
        int v = queue[head++];
        const orc_pnode *nd = &t.pool[v];
        if (nd->first_child >= 0) {
            for (int i = 0; i < 8; ++i) {
                int c = nd->first_child + i;
                dep[c] = dep[v] + 1;
                cxs[3 * c + 0] = 2 * cxs[3 * v + 0] + ((i & 1) ? 1 : 0);
                cxs[3 * c + 1] = 2 * cxs[3 * v + 1] + ((i & 2) ? 1 : 0);
                cxs[3 * c + 2] = 2 * cxs[3 * v + 2] + ((i & 4) ? 1 : 0);
                queue[tail++] = c;
            }
        }
    }
    /* Body counts bottom-up: leaves own their bodies; visit in reverse BFS. */
    for (int k = tail - 1; k >= 0; --k) {
        int v = queue[k];
        const orc_pnode *nd = &t.pool[v];
        if (nd->first_child < 0) cnt[v] = nd->np;
        else {
            int s = 0;
            for (int i = 0; i < 8; ++i) s += cnt[nd->first_child + i];
            cnt[v] = s;
        }
    }
    for (int v = 0; v < nn; ++v) {
        depth[v] = dep[v];
        count[v] = cnt[v];
        is_leaf[v] = t.pool[v].first_child < 0;
        cell_x[v] = cxs[3 * v + 0];
        cell_y[v] = cxs[3 * v + 1];
        cell_z[v] = cxs[3 * v + 2];
    }
    free(queue);
    free(cnt);
    free(cxs);
    free(dep);
    orc_ptree_free(&t);
    return nn;
}

/* ------------------------------------------------------------------------- */
/* 4. Pointer Barnes-Hut (one body per leaf), CPU/src/force_calculator_      */
/*    barnes_hut.cpp.  Insertion :133-174, octant :177-183 (x=1,y=2,z=4),    */
/*    subdivision :186-209, recursive walk :47-92.                           */
/* ------------------------------------------------------------------------- */
typedef struct orc_qnode {
    double cx, cy, cz, size, size_sqr, mass, comx, comy, comz;
    struct orc_qnode *ch[8];
    int *idx;
    int np, cap;
    int is_leaf;
} orc_qnode;

typedef struct {
    const double *x, *y, *z, *m;
    double epsilon;
} orc_qctx;

static orc_qnode *orc_qnode_new(void)
{
    orc_qnode *q = (orc_qnode *)calloc(1, sizeof(orc_qnode));
    q->is_leaf = 1;
    return q;
}

static void orc_qnode_free(orc_qnode *q)
{
    if (!q) return;
    for (int i = 0; i < 8; ++i) orc_qnode_free(q->ch[i]);
    free(q->idx);
    free(q);
}

static void orc_qnode_push(orc_qnode *q, int p)
{
    if (q->np == q->cap) {
        q->cap = q->cap ? 2 * q->cap : 2;
        q->idx = (int *)realloc(q->idx, sizeof(int) * (size_t)q->cap);
    }
    q->idx[q->np++] = p;
}

static int orc_qoct(const orc_qnode *q, double px, double py, double pz)
{
    int c = 0;
    if (px >= q->cx) c |= 1;
    if (py >= q->cy) c |= 2;
    if (pz >= q->cz) c |= 4;
    return c;
}

static int orc_qsubdivide(const orc_qctx *c, orc_qnode *q)
{
    double half = q->size / 2.0;
    if (half < c->epsilon) return 0;
    for (int i = 0; i < 8; ++i) {
        orc_qnode *k = orc_qnode_new();
        k->size = half;
        k->size_sqr = half * half;
        double ox = (i & 1) ? half / 2.0 : -half / 2.0;
        double oy = (i & 2) ? half / 2.0 : -half / 2.0;
        double oz = (i & 4) ? half / 2.0 : -half / 2.0;
        k->cx = q->cx + ox;
        k->cy = q->cy + oy;
        k->cz = q->cz + oz;
        q->ch[i] = k;
    }
    return 1;
}

static void orc_qinsert(const orc_qctx *c, orc_qnode *q, int p)
{
    const double mp = c->m[p], px = c->x[p], py = c->y[p], pz = c->z[p];
    if (q->is_leaf && q->np == 0) {
        orc_qnode_push(q, p);
        q->mass = mp;
        q->comx = px;
        q->comy = py;
        q->comz = pz;
        return;
    } else if (q->is_leaf) {
        if (!orc_qsubdivide(c, q)) {
            q->mass += mp;
            double w = q->mass - mp;
            q->comx = (q->comx * w + px * mp) / q->mass;
            q->comy = (q->comy * w + py * mp) / q->mass;
            q->comz = (q->comz * w + pz * mp) / q->mass;
            orc_qnode_push(q, p);
            return;
        }
        int e = q->idx[0];
        q->is_leaf = 0;
        q->np = 0;
        orc_qinsert(c, q->ch[orc_qoct(q, c->x[e], c->y[e], c->z[e])], e);
        orc_qinsert(c, q->ch[orc_qoct(q, px, py, pz)], p);
        const double me = c->m[e];
        q->mass = me + mp;
        q->comx = (c->x[e] * me + px * mp) / q->mass;
        q->comy = (c->y[e] * me + py * mp) / q->mass;
        q->comz = (c->z[e] * me + pz * mp) / q->mass;
    } else {
        orc_qinsert(c, q->ch[orc_qoct(q, px, py, pz)], p);
        q->mass += mp;
        double w = q->mass - mp;
        q->comx = (q->comx * w + px * mp) / q->mass;
        q->comy = (q->comy * w + py * mp) / q->mass;
        q->comz = (q->comz * w + pz * mp) / q->mass;
    }
}

typedef struct {
    double ax, ay, az;
} orc_acc3;

static void orc_qwalk(const orc_qctx *c, const orc_qnode *q, int p, double G, double eps2,
                      double theta_sqr, orc_acc3 *a)
{
    if (!q) return;
    const double px = c->x[p], py = c->y[p], pz = c->z[p];
    if (q->is_leaf) {
        for (int k = 0; k < q->np; ++k) {
            int o = q->idx[k];
            if (o == p) continue;
            double rx = c->x[o] - px, ry = c->y[o] - py, rz = c->z[o] - pz;
            double d2 = rx * rx + ry * ry + rz * rz + eps2;
            double inv = 1.0 / sqrt(d2);
            double inv3 = inv * inv * inv;
            double s = c->m[o] * inv3;
            a->ax += (rx * G) * s;
            a->ay += (ry * G) * s;
            a->az += (rz * G) * s;
        }
        return;
    }
    int cc = orc_qoct(q, px, py, pz);
    for (int i = 0; i < 8; ++i) {
        const orc_qnode *k = q->ch[i];
        if (!k) continue;
        if (i == cc) {
            orc_qwalk(c, k, p, G, eps2, theta_sqr, a);
        } else {
            double rx = k->comx - px, ry = k->comy - py, rz = k->comz - pz;
            double d2 = rx * rx + ry * ry + rz * rz;
            if (k->size_sqr < theta_sqr * d2) {
                double d2s = d2 + eps2;
                double inv = 1.0 / sqrt(d2s);
                double inv3 = inv * inv * inv;
                double s = k->mass * inv3;
                a->ax += (rx * G) * s;
                a->ay += (ry * G) * s;
                a->az += (rz * G) * s;
            } else {
                orc_qwalk(c, k, p, G, eps2, theta_sqr, a);
            }
        }
    }
}

ORC_API void orc_forces_bh_ptr(int n, const double *x, const double *y, const double *z,
                               const double *m, double G, double eps2, double theta,
                               double *ax, double *ay, double *az, int nthreads)
{
    if (n <= 0) return;
    orc_qctx c = {x, y, z, m, 1e-9};
    double minx = DBL_MAX, miny = DBL_MAX, minz = DBL_MAX;
    double maxx = -DBL_MAX, maxy = -DBL_MAX, maxz = -DBL_MAX;
    for (int i = 0; i < n; ++i) {
        minx = (x[i] < minx) ? x[i] : minx;
        maxx = (maxx < x[i]) ? x[i] : maxx;
        miny = (y[i] < miny) ? y[i] : miny;
        maxy = (maxy < y[i]) ? y[i] : maxy;
        minz = (z[i] < minz) ? z[i] : minz;
        maxz = (maxz < z[i]) ? z[i] : maxz;
    }
    double ey = maxy - miny, ez = maxz - minz, ex = maxx - minx;
    double eyz = (ey < ez) ? ez : ey;
    double size = ((ex < eyz) ? eyz : ex) + c.epsilon;
    orc_qnode *root = orc_qnode_new();
    root->cx = (minx + maxx) / 2;
    root->cy = (miny + maxy) / 2;
    root->cz = (minz + maxz) / 2;
    root->size = size;
    root->size_sqr = size * size;
    for (int i = 0; i < n; ++i) orc_qinsert(&c, root, i);
    double theta_sqr = theta * theta;
    orc_set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        orc_acc3 a = {0.0, 0.0, 0.0};
        orc_qwalk(&c, root, i, G, eps2, theta_sqr, &a);
        ax[i] = a.ax;
        ay[i] = a.ay;
        az[i] = a.az;
    }
    orc_qnode_free(root);
}

/* ------------------------------------------------------------------------- */
/* 5. Integrators, CPU/src/integrator_*.cpp.  The state arrays play the role */
/*    of the reference's Particle vector: acceleration persists between      */
/*    steps like Particle::acceleration.  Force methods: 0 direct,           */
/*    1 node-pool BH, 2 pointer BH.                                          */
/* ------------------------------------------------------------------------- */
enum { ORC_EULER = 0, ORC_EULER_CROMER = 1, ORC_LEAPFROG = 2, ORC_VERLET = 3, ORC_RK4 = 4 };

typedef struct {
    int method;
    double G, eps2, theta;
    int leaf_capacity;
    int nthreads;
} orc_force_cfg;

static int orc_force(const orc_force_cfg *f, int n, const double *x, const double *y,
                     const double *z, const double *m, double *ax, double *ay, double *az)
{
    if (f->method == 0) {
        orc_forces_naive(n, x, y, z, m, f->G, f->eps2, ax, ay, az, f->nthreads);
        return 0;
    }
    if (f->method == 1)
        return orc_forces_bh_opt(n, x, y, z, m, f->G, f->eps2, f->theta, f->leaf_capacity, ax,
                                 ay, az, f->nthreads) < 0 ? -1 : 0;
    orc_forces_bh_ptr(n, x, y, z, m, f->G, f->eps2, f->theta, ax, ay, az, f->nthreads);
    return 0;
}

/* One reference step() of the chosen integrator, nsteps times.  Returns 0,
 * or -1 on a tree overflow / bad integrator. */
ORC_API int orc_step(int integrator, int method, int n, double *x, double *y, double *z,
                     double *vx, double *vy, double *vz, const double *m, double *ax,
                     double *ay, double *az, double G, double eps2, double theta,
                     int leaf_capacity, double dt, int nsteps, int nthreads)
{
    orc_force_cfg f = {method, G, eps2, theta, leaf_capacity, nthreads};
    size_t bytes = sizeof(double) * (size_t)(n > 0 ? n : 1);
    double *buf = NULL;
    if (integrator == ORC_VERLET) buf = (double *)malloc(3 * bytes);
    if (integrator == ORC_RK4) buf = (double *)malloc(18 * bytes);
    for (int s = 0; s < nsteps; ++s) {
        switch (integrator) {
        case ORC_EULER: /* integrator_euler.cpp:3-20 */
            if (orc_force(&f, n, x, y, z, m, ax, ay, az)) goto fail;
            for (int i = 0; i < n; ++i) {
                x[i] = x[i] + vx[i] * dt;
                y[i] = y[i] + vy[i] * dt;
                z[i] = z[i] + vz[i] * dt;
            }
            for (int i = 0; i < n; ++i) {
                vx[i] = vx[i] + ax[i] * dt;
                vy[i] = vy[i] + ay[i] * dt;
                vz[i] = vz[i] + az[i] * dt;
            }
            break;
        case ORC_EULER_CROMER: /* integrator_euler-cromer.cpp:3-20 */
            if (orc_force(&f, n, x, y, z, m, ax, ay, az)) goto fail;
            for (int i = 0; i < n; ++i) {
                vx[i] = vx[i] + ax[i] * dt;
                vy[i] = vy[i] + ay[i] * dt;
                vz[i] = vz[i] + az[i] * dt;
            }
            for (int i = 0; i < n; ++i) {
                x[i] = x[i] + vx[i] * dt;
                y[i] = y[i] + vy[i] * dt;
                z[i] = z[i] + vz[i] * dt;
            }
            break;
        case ORC_LEAPFROG: { /* integrator_leapfrog.cpp:3-26 */
            double h = dt / 2.0;
            if (orc_force(&f, n, x, y, z, m, ax, ay, az)) goto fail;
            for (int i = 0; i < n; ++i) {
                vx[i] += ax[i] * h;
                vy[i] += ay[i] * h;
                vz[i] += az[i] * h;
            }
            for (int i = 0; i < n; ++i) {
                x[i] += vx[i] * dt;
                y[i] += vy[i] * dt;
                z[i] += vz[i] * dt;
            }
            if (orc_force(&f, n, x, y, z, m, ax, ay, az)) goto fail;
            for (int i = 0; i < n; ++i) {
                vx[i] += ax[i] * h;
                vy[i] += ay[i] * h;
                vz[i] += az[i] * h;
            }
            break;
        }
        case ORC_VERLET: { /* integrator_velocity_verlet.cpp:3-26 */
            double *oax = buf, *oay = buf + n, *oaz = buf + 2 * n;
            if (orc_force(&f, n, x, y, z, m, ax, ay, az)) goto fail;
            for (int i = 0; i < n; ++i) {
                /* p.position += p.velocity*dt + 0.5*p.acceleration*dt*dt */
                x[i] += vx[i] * dt + ((ax[i] * 0.5) * dt) * dt;
                y[i] += vy[i] * dt + ((ay[i] * 0.5) * dt) * dt;
                z[i] += vz[i] * dt + ((az[i] * 0.5) * dt) * dt;
            }
            for (int i = 0; i < n; ++i) {
                oax[i] = ax[i];
                oay[i] = ay[i];
                oaz[i] = az[i];
            }
            if (orc_force(&f, n, x, y, z, m, ax, ay, az)) goto fail;
            for (int i = 0; i < n; ++i) {
                double h = 0.5 * dt;
                vx[i] += (oax[i] + ax[i]) * h;
                vy[i] += (oay[i] + ay[i]) * h;
                vz[i] += (oaz[i] + az[i]) * h;
            }
            break;
        }
        case ORC_RK4: { /* integrator_rk4.cpp:3-47 */
            double *k2x = buf, *k2y = buf + n, *k2z = buf + 2 * n;
            double *k2vx = buf + 3 * n, *k2vy = buf + 4 * n, *k2vz = buf + 5 * n;
            double *k3x = buf + 6 * n, *k3y = buf + 7 * n, *k3z = buf + 8 * n;
            double *k3vx = buf + 9 * n, *k3vy = buf + 10 * n, *k3vz = buf + 11 * n;
            double *k4x = buf + 12 * n, *k4y = buf + 13 * n, *k4z = buf + 14 * n;
            double *k4vx = buf + 15 * n, *k4vy = buf + 16 * n, *k4vz = buf + 17 * n;
            double *a2 = (double *)malloc(9 * bytes);
            double *a2x = a2, *a2y = a2 + n, *a2z = a2 + 2 * n;
            double *a3x = a2 + 3 * n, *a3y = a2 + 4 * n, *a3z = a2 + 5 * n;
            double *a4x = a2 + 6 * n, *a4y = a2 + 7 * n, *a4z = a2 + 8 * n;
            double h = dt / 2.0;
            if (orc_force(&f, n, x, y, z, m, ax, ay, az)) { free(a2); goto fail; }
            for (int i = 0; i < n; ++i) {
                k2x[i] = x[i] + vx[i] * h;
                k2y[i] = y[i] + vy[i] * h;
                k2z[i] = z[i] + vz[i] * h;
                k2vx[i] = vx[i] + ax[i] * h;
                k2vy[i] = vy[i] + ay[i] * h;
                k2vz[i] = vz[i] + az[i] * h;
            }
            if (orc_force(&f, n, k2x, k2y, k2z, m, a2x, a2y, a2z)) { free(a2); goto fail; }
            for (int i = 0; i < n; ++i) {
                k3x[i] = x[i] + k2vx[i] * h;
                k3y[i] = y[i] + k2vy[i] * h;
                k3z[i] = z[i] + k2vz[i] * h;
                k3vx[i] = vx[i] + a2x[i] * h;
                k3vy[i] = vy[i] + a2y[i] * h;
                k3vz[i] = vz[i] + a2z[i] * h;
            }
            if (orc_force(&f, n, k3x, k3y, k3z, m, a3x, a3y, a3z)) { free(a2); goto fail; }
            for (int i = 0; i < n; ++i) {
                k4x[i] = x[i] + k3vx[i] * dt;
                k4y[i] = y[i] + k3vy[i] * dt;
                k4z[i] = z[i] + k3vz[i] * dt;
                k4vx[i] = vx[i] + a3x[i] * dt;
                k4vy[i] = vy[i] + a3y[i] * dt;
                k4vz[i] = vz[i] + a3z[i] * dt;
            }
            if (orc_force(&f, n, k4x, k4y, k4z, m, a4x, a4y, a4z)) { free(a2); goto fail; }
            double w = dt / 6.0;
            for (int i = 0; i < n; ++i) {
                /* (v + 2*K2.v + 2*K3.v + K4.v) * (dt/6), left to right */
                x[i] += (((vx[i] + k2vx[i] * 2.0) + k3vx[i] * 2.0) + k4vx[i]) * w;
                y[i] += (((vy[i] + k2vy[i] * 2.0) + k3vy[i] * 2.0) + k4vy[i]) * w;
                z[i] += (((vz[i] + k2vz[i] * 2.0) + k3vz[i] * 2.0) + k4vz[i]) * w;
                vx[i] += (((ax[i] + a2x[i] * 2.0) + a3x[i] * 2.0) + a4x[i]) * w;
                vy[i] += (((ay[i] + a2y[i] * 2.0) + a3y[i] * 2.0) + a4y[i]) * w;
                vz[i] += (((az[i] + a2z[i] * 2.0) + a3z[i] * 2.0) + a4z[i]) * w;
            }
            free(a2);
            break;
        }
        default:
            goto fail;
        }
    }
    free(buf);
    return 0;
fail:
    free(buf);
    return -1;
}

/* ------------------------------------------------------------------------- */
/* 6. Diagnostics, CPU/include/tests_common.hpp:33-75 (and the same          */
/*    quantities in CUDA/src/test_common.cpp:63-182).                        */
/*    out[0] KE, out[1] PE (unsoftened, as the reference), out[2] PE         */
/*    softened with eps2 (the conserved quantity when eps > 0),              */
/*    out[3..5] L, out[6..8] COM, out[9..11] linear momentum, out[12] M.     */
/* ------------------------------------------------------------------------- */
ORC_API void orc_diagnostics(int n, const double *x, const double *y, const double *z,
                             const double *vx, const double *vy, const double *vz,
                             const double *m, double G, double eps2, double *out, int nthreads)
{
    double ke = 0.0;
    for (int i = 0; i < n; ++i) {
        double vv = vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
        ke += 0.5 * m[i] * vv;
    }
    double pe = 0.0, pes = 0.0;
    orc_set_threads(nthreads);
    /* Each row's partial is summed in row order afterwards, so the result is
     * the reference's sequential i<j sum regrouped by row (the regrouping only
     * moves the rounding; the reference's own loop is a single running sum). */
    double *rowu = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    double *rows = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
        double su = 0.0, ss = 0.0;
        for (int j = i + 1; j < n; ++j) {
            double rx = x[j] - x[i], ry = y[j] - y[i], rz = z[j] - z[i];
            double r2 = rx * rx + ry * ry + rz * rz;
            double d = sqrt(r2);
            su -= G * m[i] * m[j] / d;
            ss -= G * m[i] * m[j] / sqrt(r2 + eps2);
        }
        rowu[i] = su;
        rows[i] = ss;
    }
    for (int i = 0; i < n; ++i) {
        pe += rowu[i];
        pes += rows[i];
    }
    free(rowu);
    free(rows);
    double Lx = 0.0, Ly = 0.0, Lz = 0.0;
    double cx = 0.0, cy = 0.0, cz = 0.0, M = 0.0;
    double Px = 0.0, Py = 0.0, Pz = 0.0;
    for (int i = 0; i < n; ++i) {
        double crx = y[i] * vz[i] - z[i] * vy[i];
        double cry = z[i] * vx[i] - x[i] * vz[i];
        double crz = x[i] * vy[i] - y[i] * vx[i];
        Lx += crx * m[i];
        Ly += cry * m[i];
        Lz += crz * m[i];
        cx += x[i] * m[i];
        cy += y[i] * m[i];
        cz += z[i] * m[i];
        M += m[i];
        Px += vx[i] * m[i];
        Py += vy[i] * m[i];
        Pz += vz[i] * m[i];
    }
    out[0] = ke;
    out[1] = pe;
    out[2] = pes;
    out[3] = Lx;
    out[4] = Ly;
    out[5] = Lz;
    out[6] = cx / M;
    out[7] = cy / M;
    out[8] = cz / M;
    out[9] = Px;
    out[10] = Py;
    out[11] = Pz;
    out[12] = M;
}

/* The reference's single running PE sum (tests_common.hpp:42-53), exactly,
 * for small-N bit-exact checks. */
ORC_API double orc_potential_energy_seq(int n, const double *x, const double *y, const double *z,
                                        const double *m, double G)
{
    double pe = 0.0;
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            double rx = x[j] - x[i], ry = y[j] - y[i], rz = z[j] - z[i];
            double d = sqrt(rx * rx + ry * ry + rz * rz);
            pe -= G * m[i] * m[j] / d;
        }
    return pe;
}

/* ------------------------------------------------------------------------- */
/* 7. 63-bit Morton codes, stable sort and octree topology (GPU BH rule).    */
/* ------------------------------------------------------------------------- */

/* Root cube of the CPU tree (:105-124): centre of the bounding box, side =
 * max extent + 1e-9.  root[0..2] centre, root[3] side. */
ORC_API void orc_root_cube(int n, const double *x, const double *y, const double *z,
                           double *root)
{
    double minx = DBL_MAX, miny = DBL_MAX, minz = DBL_MAX;
    double maxx = -DBL_MAX, maxy = -DBL_MAX, maxz = -DBL_MAX;
    for (int i = 0; i < n; ++i) {
        minx = (x[i] < minx) ? x[i] : minx;
        maxx = (maxx < x[i]) ? x[i] : maxx;
        miny = (y[i] < miny) ? y[i] : miny;
        maxy = (maxy < y[i]) ? y[i] : maxy;
        minz = (z[i] < minz) ? z[i] : minz;
        maxz = (maxz < z[i]) ? z[i] : maxz;
    }
    double ey = maxy - miny, ez = maxz - minz, ex = maxx - minx;
    double eyz = (ey < ez) ? ez : ey;
    root[0] = (minx + maxx) / 2;
    root[1] = (miny + maxy) / 2;
    root[2] = (minz + maxz) / 2;
    root[3] = ((ex < eyz) ? eyz : ex) + 1e-9;
}

/* Number of levels the CPU tree may split below the root: a node of side s
 * splits only while s/2 >= 1e-9 (:208-211), and the 63-bit code holds 21. */
ORC_API int orc_split_levels(double size)
{
    int lv = 0;
    double s = size;
    while (lv < 21) {
        double half = s / 2.0;
        if (half < 1e-9) break;
        s = half;
        ++lv;
    }
    return lv;
}

/* Code of one body: at each level compare against the running cell centre
 * exactly as the CPU tree's subdivision does (child centre = centre +/-
 * (size/2)/2), x in the high bit of each 3-bit digit.  Levels beyond the
 * split limit contribute zero digits. */
static uint64_t orc_code_of(double px, double py, double pz, const double *root, int levels)
{
    double cx = root[0], cy = root[1], cz = root[2], s = root[3];
    uint64_t code = 0;
    for (int l = 0; l < 21; ++l) {
        uint64_t d = 0;
        if (l < levels) {
            int bx = px >= cx, by = py >= cy, bz = pz >= cz;
            d = ((uint64_t)bx << 2) | ((uint64_t)by << 1) | (uint64_t)bz;
            double half = s / 2.0;
            double off = half / 2.0;
            cx = cx + (bx ? off : -off);
            cy = cy + (by ? off : -off);
            cz = cz + (bz ? off : -off);
            s = half;
        }
        code = (code << 3) | d;
    }
    return code;
}

ORC_API void orc_morton63(int n, const double *x, const double *y, const double *z,
                          uint64_t *codes, double *root_out)
{
    double root[4];
    orc_root_cube(n, x, y, z, root);
    int levels = orc_split_levels(root[3]);
    for (int i = 0; i < n; ++i) codes[i] = orc_code_of(x[i], y[i], z[i], root, levels);
    if (root_out) memcpy(root_out, root, sizeof(root));
}

typedef struct {
    uint64_t k;
    uint32_t v;
} orc_kv;

static int orc_kv_cmp(const void *a, const void *b)
{
    const orc_kv *p = (const orc_kv *)a, *q = (const orc_kv *)b;
    if (p->k != q->k) return p->k < q->k ? -1 : 1;
    return p->v < q->v ? -1 : (p->v > q->v);
}

/* Stable sort by code: ties keep the original index order. */
ORC_API void orc_sort_codes(int n, const uint64_t *codes, uint64_t *sorted_codes,
                            uint32_t *order)
{
    orc_kv *a = (orc_kv *)malloc(sizeof(orc_kv) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) {
        a[i].k = codes[i];
        a[i].v = (uint32_t)i;
    }
    qsort(a, (size_t)n, sizeof(orc_kv), orc_kv_cmp);
    for (int i = 0; i < n; ++i) {
        sorted_codes[i] = a[i].k;
        order[i] = a[i].v;
    }
    free(a);
}

static int orc_lower_bound(const uint64_t *c, int lo, int hi, uint64_t key)
{
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (c[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* Octree over sorted codes in breadth-first order: a cell with more than
 * leaf_capacity bodies splits while its depth is below `levels`; only the
 * non-empty children are kept, in digit order.  Node arrays: depth, prefix
 * (code >> (63 - 3*depth)), first body, body count, leaf flag, first child,
 * child count.  Returns the node count, or -1 if max_nodes is too small. */
ORC_API int orc_octree(int n, const uint64_t *sc, int leaf_capacity, int levels, int max_nodes,
                       int *depth, uint64_t *prefix, int *first, int *count, int *is_leaf,
                       int *first_child, int *nchild)
{
    if (n <= 0) return 0;
    int nn = 1;
    depth[0] = 0;
    prefix[0] = 0;
    first[0] = 0;
    count[0] = n;
    for (int v = 0; v < nn; ++v) {
        int d = depth[v];
        int split = count[v] > leaf_capacity && d < levels;
        is_leaf[v] = !split;
        first_child[v] = -1;
        nchild[v] = 0;
        if (!split) continue;
        int shift = 63 - 3 * (d + 1);
        int lo = first[v], hi = first[v] + count[v];
        first_child[v] = nn;
        for (int k = 0; k < 8; ++k) {
            uint64_t p = (prefix[v] << 3) | (uint64_t)k;
            int a = orc_lower_bound(sc, lo, hi, p << shift);
            int b = (k == 7) ? hi : orc_lower_bound(sc, lo, hi, (p + 1) << shift);
            if (b > a) {
                if (nn >= max_nodes) return -1;
                depth[nn] = d + 1;
                prefix[nn] = p;
                first[nn] = a;
                count[nn] = b - a;
                ++nn;
                ++nchild[v];
            }
        }
    }
    return nn;
}

/* ------------------------------------------------------------------------
 * 8. Synthetic workload generators.
 *
 * The benchmark configurations (Plummer spheres, the disk + bulge system)
 * have no reference code.  This section restates the engine's own seeded
 * generators (n-body-gravity-simulation_gb300/csrc/nb_gen.cpp) in C so that
 * the CPU arms of the benchmark can build their inputs without loading the
 * engine library; a test checks that both give the same bits.
 *   - SplitMix64 (Steele, Lea & Flood 2014), one stream per body keyed by
 *     (seed, body index); uniform draws on (0, 1) from the top 53 bits.
 *   - Plummer: Aarseth, Henon & Wielen (1974): radius from the cumulative
 *     mass truncated at 99.9 %, speed by von Neumann rejection on
 *     q^2 (1 - q^2)^(7/2) in units of the local escape speed.
 *   - Exponential disk: radius by inverting 1 - (1 + y) e^-y = u
 *     (bracketed Newton), sech^2 vertical profile, circular speed of the
 *     enclosed bulge + disk mass with a Gaussian dispersion.
 * All arithmetic is FP64 with the same operation order as the engine's. */
#define ORC_PI 3.14159265358979323846

typedef struct {
    uint64_t s;
} orc_sm64;

static uint64_t orc_sm64_next(orc_sm64 *r)
{
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void orc_sm64_init(orc_sm64 *r, uint64_t seed, uint64_t body)
{
    r->s = seed * 0xD1B54A32D192ED03ull ^ (body + 1) * 0x9E3779B97F4A7C15ull;
    (void)orc_sm64_next(r);
}

static double orc_sm64_u(orc_sm64 *r)
{
    return ((double)(orc_sm64_next(r) >> 11) + 0.5) * 0x1.0p-53;
}

static double orc_sm64_normal(orc_sm64 *r)
{
    const double a = orc_sm64_u(r), b = orc_sm64_u(r);
    return sqrt(-2.0 * log(a)) * cos(2.0 * ORC_PI * b);
}

static void orc_isotropic(orc_sm64 *r, double len, double *x, double *y, double *z)
{
    const double c = 1.0 - 2.0 * orc_sm64_u(r);
    const double one_c2 = 1.0 - c * c;
    const double s = sqrt(one_c2 > 0.0 ? one_c2 : 0.0);
    const double phi = 2.0 * ORC_PI * orc_sm64_u(r);
    *x = len * s * cos(phi);
    *y = len * s * sin(phi);
    *z = len * c;
}

static void orc_plummer_body(orc_sm64 *r, double M, double a, double G, double *p, double *v)
{
    const double X1 = 0.999 * orc_sm64_u(r);
    const double rad = a / sqrt(pow(X1, -2.0 / 3.0) - 1.0);
    orc_isotropic(r, rad, &p[0], &p[1], &p[2]);
    double q = 0.0;
    for (int it = 0; it < 100000; ++it) {
        q = orc_sm64_u(r);
        const double g = 0.1 * orc_sm64_u(r);
        if (g < q * q * pow(1.0 - q * q, 3.5)) break;
    }
    const double ve = sqrt(2.0 * G * M / a) * pow(1.0 + rad * rad / (a * a), -0.25);
    orc_isotropic(r, q * ve, &v[0], &v[1], &v[2]);
}

static void orc_to_com_frame(int n, const double *m, double *x, double *y, double *z,
                             double *vx, double *vy, double *vz)
{
    double M = 0, c[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; ++i) {
        M += m[i];
        c[0] += m[i] * x[i]; c[1] += m[i] * y[i]; c[2] += m[i] * z[i];
        c[3] += m[i] * vx[i]; c[4] += m[i] * vy[i]; c[5] += m[i] * vz[i];
    }
    if (!(M > 0)) return;
    for (int k = 0; k < 6; ++k) c[k] /= M;
    for (int i = 0; i < n; ++i) {
        x[i] -= c[0]; y[i] -= c[1]; z[i] -= c[2];
        vx[i] -= c[3]; vy[i] -= c[4]; vz[i] -= c[5];
    }
}

static double orc_disk_radius(double u)
{
    double lo = 0.0, hi = 50.0, y = 1.0;
    for (int it = 0; it < 200; ++it) {
        const double f = 1.0 - (1.0 + y) * exp(-y) - u;
        if (f > 0) hi = y; else lo = y;
        const double df = y * exp(-y);
        double yn = (df > 0) ? y - f / df : 0.5 * (lo + hi);
        if (!(yn > lo && yn < hi)) yn = 0.5 * (lo + hi);
        if (fabs(yn - y) < 1e-15 * (1.0 + y)) { y = yn; break; }
        y = yn;
    }
    return y;
}

ORC_API void orc_gen_plummer(int n, uint64_t seed, double total_mass, double scale, double G,
                             double *x, double *y, double *z, double *vx, double *vy, double *vz,
                             double *m)
{
    for (int i = 0; i < n; ++i) {
        orc_sm64 r;
        orc_sm64_init(&r, seed, (uint64_t)i);
        double p[3], v[3];
        orc_plummer_body(&r, total_mass, scale, G, p, v);
        x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
        vx[i] = v[0]; vy[i] = v[1]; vz[i] = v[2];
        m[i] = total_mass / (double)n;
    }
    orc_to_com_frame(n, m, x, y, z, vx, vy, vz);
}

ORC_API void orc_gen_disk_bulge(int n, uint64_t seed, double total_mass, double bulge_frac,
                                double bulge_scale, double disk_scale, double disk_height,
                                double dispersion, double G, double *x, double *y, double *z,
                                double *vx, double *vy, double *vz, double *m)
{
    const int nbulge = (int)llround(bulge_frac * (double)n);
    const double Mb = total_mass * bulge_frac, Md = total_mass - Mb;
    for (int i = 0; i < n; ++i) {
        orc_sm64 r;
        orc_sm64_init(&r, seed, (uint64_t)i);
        m[i] = total_mass / (double)n;
        double p[3], v[3];
        if (i < nbulge) {
            orc_plummer_body(&r, Mb, bulge_scale, G, p, v);
        } else {
            const double R = disk_scale * orc_disk_radius(0.999 * orc_sm64_u(&r));
            const double phi = 2.0 * ORC_PI * orc_sm64_u(&r);
            double uz = orc_sm64_u(&r);
            uz = uz < 5e-4 ? 5e-4 : uz;
            uz = uz > 1.0 - 5e-4 ? 1.0 - 5e-4 : uz;
            p[0] = R * cos(phi);
            p[1] = R * sin(phi);
            p[2] = disk_height * atanh(2.0 * uz - 1.0);
            const double rs = sqrt(R * R + p[2] * p[2]);
            const double yd = R / disk_scale;
            const double menc = Mb * rs * rs * rs / pow(rs * rs + bulge_scale * bulge_scale, 1.5) +
                                Md * (1.0 - (1.0 + yd) * exp(-yd));
            const double vc = (R > 0) ? sqrt(G * menc / (rs > 1e-12 ? rs : 1e-12)) : 0.0;
            const double sig = dispersion * vc;
            v[0] = -vc * sin(phi) + sig * orc_sm64_normal(&r);
            v[1] = vc * cos(phi) + sig * orc_sm64_normal(&r);
            v[2] = sig * orc_sm64_normal(&r);
        }
        x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
        vx[i] = v[0]; vy[i] = v[1]; vz[i] = v[2];
    }
    orc_to_com_frame(n, m, x, y, z, vx, vy, vz);
}
