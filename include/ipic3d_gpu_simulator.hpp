/*
 * C++ drop-in for the reference's timestep loop: simulateSteps over a
 * Universe (simulator.h:42-47,127-242; universe.h:12-51), running on the GB300
 * path behind the C ABI of ipic3d_gpu.h.
 *
 * Header-only, C++14. Everything is templated on the Universe type, so the
 * same code serves the reference's own ipic3d::Universe (see
 * ipic3d_gpu_reference.hpp, which adds explicit specializations of
 * ipic3d::simulateSteps for the policy tags below) and any structure with the
 * same members:
 *
 *   universe.properties   size (.x .y .z), cellWidth, dt, speedOfLight,
 *                         planetRadius, objectCenter, origin,
 *                         externalMagneticField            (universe_properties.h:52-123)
 *   universe.cells[c]     .particles: a std::vector of {position, velocity,
 *                         q, qom}                          (cell.h:31-36, particle.h:9-17)
 *   universe.field[n]     .E .B .Bext on (size+3)^3        (field.h:14-18)
 *   universe.bcfield[n]   .Bc on (size+2)^3                (field.h:20-23)
 *   universe.currentDensity[n]  .J on (size+1)^3           (field.h:25-27)
 *
 * where c and n are coordinates with .x .y .z members (utils::Coordinate<3>)
 * and grid.size() returns one.
 *
 * Ownership follows the reference: the Universe owns the state; a call
 * moves it to the device, runs the steps and writes particles, fields and
 * current density back. Errors, which the reference answers with assert
 * aborts, are thrown as ipic3d_gpu::Error with the C ABI's status.
 */
#ifndef IPIC3D_GPU_SIMULATOR_HPP
#define IPIC3D_GPU_SIMULATOR_HPP

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ipic3d_gpu.h"

namespace ipic3d_gpu {

/* ---- policy tags: the simulateSteps template arguments ------------------ */
/* projectors (ParticleToFieldProjector, simulator.h:244-250) */
struct no_projector {};           // the reference's active loop: no projection step
struct cic_projector {};          // projectToDensityField (cell.h:787-824) every step
/* field solvers (FieldSolver, simulator.h:252-268) */
struct static_field_solver {};    // default_field_solver: solveFieldStatically, a no-op
struct leapfrog_field_solver {};  // leapfrog_field_solver: solveFieldLeapfrog
struct forward_field_solver {};   // forward_field_solver: solveFieldForward
/* particle movers (ParticleMover, simulator.h:270-275) */
struct dipole_particle_mover {};  // default_particle_mover: moveParticles + exportParticles
struct field_particle_mover {};   // the field-gather mover (cell.h:905-937, 867-885)

/* Settings the policy types do not carry; read at every call. */
struct Options {
    int precision = IPIC3D_FP64;              // IPIC3D_FP64 / IPIC3D_FP32
    int bc_low[3] = {IPIC3D_BC_REFLECT, IPIC3D_BC_REFLECT, IPIC3D_BC_REFLECT};
    int bc_high[3] = {IPIC3D_BC_REFLECT, IPIC3D_BC_REFLECT, IPIC3D_BC_REFLECT};
    uint32_t flags = IPIC3D_F_USE_GRAPH;      // IPIC3D_F_* (J_DIV8, GATHER_DIV_VOL, ...)
    // The reference's debug-build trace (ENABLE_DEBUG_OUTPUT: writeOutputHeader
    // and writeOutputData, simulator.h:65-90): when set, the header and the
    // conserved quantities before every trace_every-th cycle and before the
    // last are written to *trace, from the device's reductions. The steps then
    // run one call per cycle.
    std::ostream* trace = nullptr;
    int trace_every = 1;
    // With the trace: the per-cell particle counts before cycle 0 and before
    // every cycle i with (i + 1) % density_every == 0, written to
    // density_prefix + "%06d" (t = (i + 1) / density_every) as the
    // reference's "t,x,y,z,density" files (simulator.h:92-113), from the
    // device's cell counts. Off when density_every is 0.
    std::string density_prefix;
    int density_every = 0;
};

inline Options& options() {
    static Options o;
    return o;
}

class Error : public std::runtime_error {
   public:
    Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }

   private:
    int status_;
};

/* Wall-clock split of the reference's DurationMeasurement (simulator.h:36-39),
 * in seconds: the first step (including the transfer to the device) and the
 * remaining ones (including the transfer back). */
struct Durations {
    double firstStep;
    double remainingSteps;
};

namespace detail {

inline void check(int rc, const char* what) {
    if (rc == IPIC3D_OK) return;
    char buf[512];
    ipic3d_gpu_last_error(buf, sizeof buf);
    throw Error(rc, std::string(what) + ": " + buf);
}

template <class P> struct projector;
template <> struct projector<no_projector> { static constexpr int value = IPIC3D_PROJECT_NONE; };
template <> struct projector<cic_projector> { static constexpr int value = IPIC3D_PROJECT_CIC; };
template <class F> struct solver;
template <> struct solver<static_field_solver> { static constexpr int value = IPIC3D_SOLVER_STATIC; };
template <> struct solver<leapfrog_field_solver> { static constexpr int value = IPIC3D_SOLVER_LEAPFROG; };
template <> struct solver<forward_field_solver> { static constexpr int value = IPIC3D_SOLVER_FORWARD; };
template <class M> struct mover;
template <> struct mover<dipole_particle_mover> { static constexpr int value = IPIC3D_MOVER_DIPOLE; };
template <> struct mover<field_particle_mover> { static constexpr int value = IPIC3D_MOVER_FIELD; };

template <class Coord>
Coord coord(const Coord& like, int64_t x, int64_t y, int64_t z) {
    Coord c = like;
    c.x = x;
    c.y = y;
    c.z = z;
    return c;
}

template <class Props>
ipic3d_props props_of(const Props& p) {
    ipic3d_props o;
    o.size[0] = p.size.x;
    o.size[1] = p.size.y;
    o.size[2] = p.size.z;
    o.cell_width[0] = p.cellWidth.x;
    o.cell_width[1] = p.cellWidth.y;
    o.cell_width[2] = p.cellWidth.z;
    o.dt = p.dt;
    o.speed_of_light = p.speedOfLight;
    o.planet_radius = p.planetRadius;
    o.object_center[0] = p.objectCenter.x;
    o.object_center[1] = p.objectCenter.y;
    o.object_center[2] = p.objectCenter.z;
    o.origin[0] = p.origin.x;
    o.origin[1] = p.origin.y;
    o.origin[2] = p.origin.z;
    o.external_b[0] = p.externalMagneticField.x;
    o.external_b[1] = p.externalMagneticField.y;
    o.external_b[2] = p.externalMagneticField.z;
    return o;
}

/* Universe::cells -> particles grouped by cell (row-major, x slowest) */
template <class Universe>
void pack_particles(const Universe& u, std::vector<ipic3d_particle>& parts, std::vector<uint64_t>& counts) {
    const auto s = u.cells.size();
    parts.clear();
    counts.assign((size_t)(s.x * s.y * s.z), 0);
    size_t k = 0;
    for (int64_t x = 0; x < s.x; ++x)
        for (int64_t y = 0; y < s.y; ++y)
            for (int64_t z = 0; z < s.z; ++z, ++k) {
                const auto& cell = u.cells[coord(s, x, y, z)];
                counts[k] = cell.particles.size();
                for (const auto& p : cell.particles) {
                    ipic3d_particle q;
                    q.position[0] = p.position.x;
                    q.position[1] = p.position.y;
                    q.position[2] = p.position.z;
                    q.velocity[0] = p.velocity.x;
                    q.velocity[1] = p.velocity.y;
                    q.velocity[2] = p.velocity.z;
                    q.q = p.q;
                    q.qom = p.qom;
                    parts.push_back(q);
                }
            }
}

template <class Universe>
void unpack_particles(Universe& u, const std::vector<ipic3d_particle>& parts, const std::vector<uint64_t>& counts) {
    const auto s = u.cells.size();
    size_t k = 0, i = 0;
    for (int64_t x = 0; x < s.x; ++x)
        for (int64_t y = 0; y < s.y; ++y)
            for (int64_t z = 0; z < s.z; ++z, ++k) {
                auto& v = u.cells[coord(s, x, y, z)].particles;
                v.resize((size_t)counts[k]);
                for (auto& p : v) {
                    const ipic3d_particle& q = parts[i++];
                    p.position.x = q.position[0];
                    p.position.y = q.position[1];
                    p.position.z = q.position[2];
                    p.velocity.x = q.velocity[0];
                    p.velocity.y = q.velocity[1];
                    p.velocity.z = q.velocity[2];
                    p.q = q.q;
                    p.qom = q.qom;
                }
            }
}

/* Visits every node of a grid in row-major order with its flat index. */
template <class Grid, class Fn>
void for_nodes(Grid& g, Fn fn) {
    const auto s = g.size();
    size_t k = 0;
    for (int64_t x = 0; x < s.x; ++x)
        for (int64_t y = 0; y < s.y; ++y)
            for (int64_t z = 0; z < s.z; ++z, ++k) fn(g[coord(s, x, y, z)], k);
}

template <class V>
void put3(double* d, const V& v) {
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
}
template <class V>
void get3(V& v, const double* d) {
    v.x = d[0];
    v.y = d[1];
    v.z = d[2];
}

template <class Universe>
void pack_fields(const Universe& u, std::vector<double>& field, std::vector<double>& bc, std::vector<double>& j) {
    const auto fs = u.field.size(), bs = u.bcfield.size(), js = u.currentDensity.size();
    field.assign((size_t)(fs.x * fs.y * fs.z) * IPIC3D_FIELD_NODE_DOUBLES, 0.0);
    bc.assign((size_t)(bs.x * bs.y * bs.z) * IPIC3D_BC_CELL_DOUBLES, 0.0);
    j.assign((size_t)(js.x * js.y * js.z) * IPIC3D_DENSITY_NODE_DOUBLES, 0.0);
    for_nodes(u.field, [&](const auto& n, size_t k) {
        put3(&field[9 * k], n.E);
        put3(&field[9 * k + 3], n.B);
        put3(&field[9 * k + 6], n.Bext);
    });
    for_nodes(u.bcfield, [&](const auto& n, size_t k) { put3(&bc[3 * k], n.Bc); });
    for_nodes(u.currentDensity, [&](const auto& n, size_t k) { put3(&j[3 * k], n.J); });
}

template <class Universe>
void unpack_fields(Universe& u, const std::vector<double>& field, const std::vector<double>& bc,
                   const std::vector<double>& j) {
    for_nodes(u.field, [&](auto& n, size_t k) {
        get3(n.E, &field[9 * k]);
        get3(n.B, &field[9 * k + 3]);
        get3(n.Bext, &field[9 * k + 6]);
    });
    for_nodes(u.bcfield, [&](auto& n, size_t k) { get3(n.Bc, &bc[3 * k]); });
    for_nodes(u.currentDensity, [&](auto& n, size_t k) { get3(n.J, &j[3 * k]); });
}

/* Closes the context on every exit path. */
struct Context {
    ipic3d_ctx* ctx = nullptr;
    ~Context() {
        if (ctx) ipic3d_gpu_destroy(ctx);
    }
};

// One "t,x,y,z,density" file of the reference's debug output
// (simulator.h:92-113): per cell, its corner (cell index times width) and
// its particle count, from the device's cell counts.
template <class Props>
void write_density(ipic3d_ctx* ctx, const Props& p, int t, const std::string& prefix) {
    const int64_t sx = p.size.x, sy = p.size.y, sz = p.size.z;
    std::vector<uint64_t> counts((size_t)(sx * sy * sz));
    check(ipic3d_gpu_cell_counts(ctx, counts.data()), "ipic3d_gpu_cell_counts");
    char name[32];
    std::snprintf(name, sizeof name, "%06d", t);
    std::ofstream out(prefix + name);
    out << "t,x,y,z,density\n";
    for (int64_t x = 0; x < sx; x++)
        for (int64_t y = 0; y < sy; y++)
            for (int64_t z = 0; z < sz; z++) {
                const double dx = x * p.cellWidth.x, dy = y * p.cellWidth.y, dz = z * p.cellWidth.z;
                out << t << "," << dx << "," << dy << "," << dz << "," << counts[(size_t)((x * sy + y) * sz + z)]
                    << "\n";
            }
}

}  // namespace detail

/* simulateSteps<Projector, FieldSolver, Mover>(numSteps, universe) on the
 * GPU, updating the universe in place. The reference's loop runs only the
 * mover and the import (its projection and field-solver steps are commented
 * out, simulator.h:189-209): no_projector + static_field_solver is exactly
 * that loop; cic_projector and the leapfrog / forward solvers run the steps
 * those lines describe (project, ghost copy, solve) before the mover. Particles come back grouped by
 * cell; their order inside a cell is unspecified (the reference's is the
 * order of its mailbox imports, cell.h:1272-1306). */
template <class Projector, class FieldSolver, class Mover, class Universe>
Durations simulate(std::uint64_t numSteps, Universe& universe) {
    using clock = std::chrono::high_resolution_clock;
    const Options& opt = options();
    ipic3d_config cfg;
    ipic3d_gpu_config_default(&cfg);
    cfg.precision = opt.precision;
    cfg.mover = detail::mover<Mover>::value;
    cfg.solver = detail::solver<FieldSolver>::value;
    cfg.projector = detail::projector<Projector>::value;
    for (int a = 0; a < 3; ++a) {
        cfg.bc_low[a] = opt.bc_low[a];
        cfg.bc_high[a] = opt.bc_high[a];
    }
    cfg.flags = opt.flags;
    const ipic3d_props props = detail::props_of(universe.properties);

    const auto start = clock::now();
    detail::Context c;
    detail::check(ipic3d_gpu_create(&props, &cfg, &c.ctx), "ipic3d_gpu_create");
    std::vector<ipic3d_particle> parts;
    std::vector<uint64_t> counts;
    std::vector<double> field, bc, j;
    detail::pack_particles(universe, parts, counts);
    detail::pack_fields(universe, field, bc, j);
    detail::check(ipic3d_gpu_upload_fields(c.ctx, field.data(), bc.data(), j.data()), "ipic3d_gpu_upload_fields");
    detail::check(ipic3d_gpu_upload_particles(c.ctx, parts.empty() ? nullptr : parts.data(), counts.data(), nullptr),
                  "ipic3d_gpu_upload_particles");
    auto end_first = start;
    if (opt.trace) {
        *opt.trace << "Cycle \t Total Moment \t E energy \t B energy \t Total KE \n";
        for (std::uint64_t i = 0; i < numSteps; ++i) {
            if (opt.trace_every > 0 && (i % (std::uint64_t)opt.trace_every == 0 || i + 1 == numSteps)) {
                ipic3d_conserved q;
                detail::check(ipic3d_gpu_conserved(c.ctx, &q), "ipic3d_gpu_conserved");
                *opt.trace << i << "\t" << q.total_momentum << "\t" << q.e_energy << "\t" << q.b_energy << "\t"
                           << q.kinetic_energy << "\n";
            }
            if (opt.density_every > 0 && (i == 0 || (i + 1) % (std::uint64_t)opt.density_every == 0))
                detail::write_density(c.ctx, universe.properties, (int)((i + 1) / (std::uint64_t)opt.density_every),
                                      opt.density_prefix);
            detail::check(ipic3d_gpu_step(c.ctx, 1), "ipic3d_gpu_step");
            if (i == 0) {
                detail::check(ipic3d_gpu_synchronize(c.ctx), "ipic3d_gpu_synchronize");
                end_first = clock::now();
            }
        }
    } else if (numSteps > 0) {
        detail::check(ipic3d_gpu_step(c.ctx, 1), "ipic3d_gpu_step");
        detail::check(ipic3d_gpu_synchronize(c.ctx), "ipic3d_gpu_synchronize");
        end_first = clock::now();
        if (numSteps > 1) detail::check(ipic3d_gpu_step(c.ctx, numSteps - 1), "ipic3d_gpu_step");
    }
    uint64_t n = 0;
    detail::check(ipic3d_gpu_particle_count(c.ctx, &n), "ipic3d_gpu_particle_count");
    parts.resize((size_t)n);
    detail::check(ipic3d_gpu_download_particles(c.ctx, parts.empty() ? nullptr : parts.data(), n, counts.data(),
                                                nullptr),
                  "ipic3d_gpu_download_particles");
    detail::check(ipic3d_gpu_download_fields(c.ctx, field.data(), bc.data(), j.data(), nullptr),
                  "ipic3d_gpu_download_fields");
    detail::unpack_particles(universe, parts, counts);
    detail::unpack_fields(universe, field, bc, j);
    const auto end = clock::now();
    return {std::chrono::duration<double>(end_first - start).count(),
            std::chrono::duration<double>(end - end_first).count()};
}

/* traceParticle (pic_tracer.cxx:77-148) on the GPU for every particle of a
 * range of the reference's Particle objects (anything with position,
 * velocity, q and qom members), `steps` steps each (pic_tracer's main passes
 * T + 1), counting into `counts`, the ParticleCount vector (num_frames x
 * cells uint32, row-major, frame slowest), which is added to as traceParticle
 * increments it. `config` is the UniverseProperties the tracer runs with.
 * Throws Error on failure. */
template <class Props, class Particles>
void trace_particles(const Props& config, const Particles& particles, int steps, int frame_interval, int num_frames,
                     std::uint32_t* counts) {
    std::vector<ipic3d_particle> buf;
    buf.reserve(particles.size());
    for (const auto& p : particles) {
        ipic3d_particle q;
        q.position[0] = p.position.x;
        q.position[1] = p.position.y;
        q.position[2] = p.position.z;
        q.velocity[0] = p.velocity.x;
        q.velocity[1] = p.velocity.y;
        q.velocity[2] = p.velocity.z;
        q.q = p.q;
        q.qom = p.qom;
        buf.push_back(q);
    }
    const ipic3d_props props = detail::props_of(config);
    detail::check(ipic3d_gpu_trace(&props, buf.data(), buf.size(), steps, frame_interval, num_frames, counts),
                  "ipic3d_gpu_trace");
}

}  // namespace ipic3d_gpu

#endif /* IPIC3D_GPU_SIMULATOR_HPP */
