// nb_io.cpp -- host-side files: the reference's particle lists, its trajectory
// CSV, and binary checkpoints of a simulation.
//
// Particle files follow the loader of CUDA/tests/test3_correctness.cu:16-38
// (N, then N records "m x y z vx vy vz"), the format of the reference's
// particles_{100..10000}.txt fixtures.  The CSV row is the one
// CPU/src/n-body.cpp:6-58 writes per step (body positions, energies, angular
// momentum, centre of mass).  Checkpoints have no reference counterpart.
#include "nb_internal.h"

#include <cerrno>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using nb::fail;

namespace {

struct File {
    FILE *f = nullptr;
    File(const char *path, const char *mode) : f(std::fopen(path, mode)) {}
    ~File()
    {
        if (f) std::fclose(f);
    }
    File(const File &) = delete;
    File &operator=(const File &) = delete;
};

std::string io_msg(const char *what, const char *path)
{
    std::string m = std::string(what) + " '" + path + "'";
    if (errno) m += std::string(": ") + std::strerror(errno);
    return m;
}

bool read_all(const char *path, std::string &out)
{
    errno = 0;
    File fh(path, "rb");
    if (!fh.f) return false;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, fh.f)) > 0) out.append(buf, got);
    return !std::ferror(fh.f);
}

// Whitespace-separated tokens, as an istream >> reads them.
struct Tokens {
    const char *p, *end;
    bool next_double(double &v)
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
        if (p >= end) return false;
        char *q = nullptr;
        v = std::strtod(p, &q);
        if (q == p) return false;
        p = q;
        return true;
    }
};

nb_status parse_particles(const char *path, size_t capacity, size_t *n, double *const *cols)
{
    std::string text;
    if (!read_all(path, text)) return fail(NB_ERR_IO, io_msg("cannot read particle file", path));
    Tokens tk{text.data(), text.data() + text.size()};
    double count = 0.0;
    // the range test comes first: converting a double beyond long long's
    // range is undefined, and no file holds 2^53 bodies
    if (!tk.next_double(count) || !(count >= 0.0 && count <= 9.0e15) ||
        count != (double)(long long)count)
        return fail(NB_ERR_IO, std::string("particle file '") + path +
                                   "': the first token is not a body count");
    const size_t N = (size_t)count;
    *n = N;
    if (!cols[0]) return NB_OK;  // size query
    if (N > capacity) return fail(NB_ERR_CAPACITY, "particle file holds more bodies than capacity");
    for (size_t i = 0; i < N; ++i)
        for (int c = 0; c < 7; ++c)
            if (!tk.next_double(cols[c][i]))
                return fail(NB_ERR_IO, std::string("particle file '") + path +
                                           "': record " + std::to_string(i) +
                                           " is missing or malformed");
    return NB_OK;
}

void put_number(std::string &out, double v, int precision)
{
    char buf[64];
    if (precision < 0)
        std::snprintf(buf, sizeof buf, "%g", v);
    else
        std::snprintf(buf, sizeof buf, "%.*f", precision, v);
    out += buf;
}

constexpr char kMagic[8] = {'N', 'B', 'G', 'B', '3', 'C', 'K', '1'};
constexpr uint32_t kVersion = 1;

} // namespace

extern "C" {

nb_status nb_particles_read(const char *path, size_t capacity, size_t *n, double *m, double *x,
                            double *y, double *z, double *vx, double *vy, double *vz)
{
    if (!path || !n) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    double *cols[7] = {m, x, y, z, vx, vy, vz};
    if (m)
        for (double *c : cols)
            if (!c) return fail(NB_ERR_INVALID_ARGUMENT, "NULL output array");
    return parse_particles(path, capacity, n, cols);
}

nb_status nb_particles_write(const char *path, size_t n, const double *m, const double *x,
                             const double *y, const double *z, const double *vx,
                             const double *vy, const double *vz)
{
    if (!path) return fail(NB_ERR_INVALID_ARGUMENT, "NULL path");
    const double *cols[7] = {m, x, y, z, vx, vy, vz};
    for (const double *c : cols)
        if (n > 0 && !c) return fail(NB_ERR_INVALID_ARGUMENT, "NULL input array");
    errno = 0;
    File fh(path, "wb");
    if (!fh.f) return fail(NB_ERR_IO, io_msg("cannot create particle file", path));
    std::fprintf(fh.f, "%zu\n", n);
    for (size_t i = 0; i < n; ++i)
        std::fprintf(fh.f, "%.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", m[i], x[i], y[i],
                     z[i], vx[i], vy[i], vz[i]);
    if (std::ferror(fh.f)) return fail(NB_ERR_IO, io_msg("write failed on", path));
    return NB_OK;
}

nb_status nb_load_particles(nb_sim *s, const char *path)
{
    if (!s || !path) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    size_t n = 0;
    NB_TRY(nb_particles_read(path, 0, &n, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                             nullptr));
    if (n > s->capacity) return fail(NB_ERR_CAPACITY, "n exceeds the capacity of the simulation");
    std::vector<double> buf(7 * std::max<size_t>(n, 1));
    double *c[7];
    for (int k = 0; k < 7; ++k) c[k] = buf.data() + k * n;
    NB_TRY(nb_particles_read(path, n, &n, c[0], c[1], c[2], c[3], c[4], c[5], c[6]));
    return nb_load(s, n, c[1], c[2], c[3], c[4], c[5], c[6], c[0]);
}

nb_status nb_csv_append(nb_sim *s, const char *path, int nbodies, const int *bodies,
                        const char *const *names, int header, int precision)
{
    if (!s || !path || nbodies < 0 || (nbodies > 0 && (!bodies || (header && !names))))
        return fail(NB_ERR_INVALID_ARGUMENT, "NULL or negative argument");
    if (s->n == 0) return fail(NB_ERR_NOT_LOADED, "no bodies loaded");
    for (int b = 0; b < nbodies; ++b)
        if (bodies[b] < 0 || (size_t)bodies[b] >= s->n)
            return fail(NB_ERR_INVALID_ARGUMENT, "body index out of range");
    // positions of the listed bodies, then the diagnostics of the state
    std::vector<double> pos(3 * (size_t)nbodies);
    for (int b = 0; b < nbodies; ++b)
        for (int c = 0; c < 3; ++c)
            NB_CUDA_TRY(cudaMemcpyAsync(&pos[3 * b + c], s->f[c] + bodies[b], sizeof(double),
                                        cudaMemcpyDeviceToHost, s->stream));
    nb_diag d{};
    NB_TRY(nb_diagnostics(s, &d));  // synchronises the stream
    std::string row;
    if (header) {
        for (int b = 0; b < nbodies; ++b)
            for (const char *ax : {"_x,", "_y,", "_z,"}) {
                row += names[b] ? names[b] : "";
                row += ax;
            }
        row += "kinetic_energy,potential_energy,total_energy,angular_momentum_x,"
               "angular_momentum_y,angular_momentum_z,center_of_mass_x,center_of_mass_y,"
               "center_of_mass_z\n";
    }
    const double vals[9] = {d.kinetic,
                            d.potential,
                            d.total,
                            d.angular_momentum[0],
                            d.angular_momentum[1],
                            d.angular_momentum[2],
                            d.center_of_mass[0],
                            d.center_of_mass[1],
                            d.center_of_mass[2]};
    for (double v : pos) {
        put_number(row, v, precision);
        row += ',';
    }
    for (int k = 0; k < 9; ++k) {
        put_number(row, vals[k], precision);
        row += k < 8 ? ',' : '\n';
    }
    errno = 0;
    File fh(path, "ab");
    if (!fh.f) return fail(NB_ERR_IO, io_msg("cannot open CSV file", path));
    if (std::fwrite(row.data(), 1, row.size(), fh.f) != row.size())
        return fail(NB_ERR_IO, io_msg("write failed on", path));
    return NB_OK;
}

nb_status nb_checkpoint_save(nb_sim *s, const char *path)
{
    if (!s || !path) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    const size_t n = s->n;
    std::vector<double> plane(std::max<size_t>(n, 1));
    errno = 0;
    File fh(path, "wb");
    if (!fh.f) return fail(NB_ERR_IO, io_msg("cannot create checkpoint", path));
    const uint32_t version = kVersion, valid = s->forces_valid ? 1u : 0u;
    const uint64_t n64 = n;
    bool ok = std::fwrite(kMagic, 1, 8, fh.f) == 8 &&
              std::fwrite(&version, sizeof version, 1, fh.f) == 1 &&
              std::fwrite(&valid, sizeof valid, 1, fh.f) == 1 &&
              std::fwrite(&n64, sizeof n64, 1, fh.f) == 1 &&
              std::fwrite(&s->cfg, sizeof(nb_config), 1, fh.f) == 1;
    for (int k = 0; k < 10 && ok && n > 0; ++k) {
        NB_CUDA_TRY(cudaMemcpyAsync(plane.data(), s->f[k], n * sizeof(double),
                                    cudaMemcpyDeviceToHost, s->stream));
        NB_CUDA_TRY(cudaStreamSynchronize(s->stream));
        ok = std::fwrite(plane.data(), sizeof(double), n, fh.f) == n;
    }
    if (!ok) return fail(NB_ERR_IO, io_msg("write failed on", path));
    return NB_OK;
}

nb_status nb_checkpoint_load(nb_sim *s, const char *path)
{
    if (!s || !path) return fail(NB_ERR_INVALID_ARGUMENT, "NULL argument");
    errno = 0;
    File fh(path, "rb");
    if (!fh.f) return fail(NB_ERR_IO, io_msg("cannot open checkpoint", path));
    char magic[8];
    uint32_t version = 0, valid = 0;
    uint64_t n64 = 0;
    nb_config cfg{};
    const bool ok = std::fread(magic, 1, 8, fh.f) == 8 &&
                    std::fread(&version, sizeof version, 1, fh.f) == 1 &&
                    std::fread(&valid, sizeof valid, 1, fh.f) == 1 &&
                    std::fread(&n64, sizeof n64, 1, fh.f) == 1 &&
                    std::fread(&cfg, sizeof cfg, 1, fh.f) == 1;
    if (!ok || std::memcmp(magic, kMagic, 8) != 0 || version != kVersion)
        return fail(NB_ERR_IO, std::string("'") + path + "' is not a version-1 checkpoint");
    if (n64 > s->capacity) return fail(NB_ERR_CAPACITY, "checkpoint holds more bodies than capacity");
    const size_t n = (size_t)n64;
    std::vector<double> planes(10 * std::max<size_t>(n, 1));
    if (n > 0 && std::fread(planes.data(), sizeof(double), 10 * n, fh.f) != 10 * n)
        return fail(NB_ERR_IO, std::string("checkpoint '") + path + "' is truncated");
    NB_TRY(nb_set_config(s, &cfg));
    for (int k = 0; k < 10 && n > 0; ++k)
        NB_CUDA_TRY(cudaMemcpyAsync(s->f[k], planes.data() + k * n, n * sizeof(double),
                                    cudaMemcpyHostToDevice, s->stream));
    NB_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->n = n;
    s->forces_valid = valid != 0;
    nb::bh_invalidate(s->bh);
    nb::reset_step_graph(s);
    return NB_OK;
}

} // extern "C"
