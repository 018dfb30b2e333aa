// The C++ drop-in against the reference's own types: a Universe built by the
// reference's constructors (universe.h:34-40) goes through the adapter's
// pack/unpack unchanged, and simulateSteps with the GPU policy tags resolves
// to the GPU path (on a machine without an sm_103 GPU it throws
// ipic3d_gpu::Error with IPIC3D_E_NODEVICE).
#include <cstdio>

#include "ipic3d_gpu_reference.hpp"

using namespace ipic3d;

static double val(int64_t a, int64_t b, int64_t c, int k) { return 0.25 * a - 0.5 * b + 0.125 * c + 0.01 * k; }

int main(int argc, char** argv) {
    const int64_t n = 4;
    UniverseProperties props(UseCase::Dipole, {n, n, n}, {1.0, 2.0, 0.5}, 0.1, 1.0, 0.0, {0, 0, 0}, {-1, -2, -3},
                             {0, 0, 1e-4});
    Universe u(props);
    const auto s = u.cells.size();
    for (int64_t x = 0; x < s.x; ++x)
        for (int64_t y = 0; y < s.y; ++y)
            for (int64_t z = 0; z < s.z; ++z) {
                auto& cell = u.cells[utils::Coordinate<3>{x, y, z}];
                for (int k = 0; k < (int)((x + 2 * y + 3 * z) % 4); ++k) {
                    Particle p;
                    p.position = {props.origin.x + (x + 0.3) * props.cellWidth.x,
                                  props.origin.y + (y + 0.1 * k) * props.cellWidth.y,
                                  props.origin.z + (z + 0.7) * props.cellWidth.z};
                    p.velocity = {val(x, y, z, k), val(y, z, x, k), val(z, x, y, k)};
                    p.q = 1.0 + k;
                    p.qom = -1.0;
                    cell.particles.push_back(p);
                }
            }
    auto fill = [](auto& grid, auto fn) {
        const auto g = grid.size();
        for (int64_t x = 0; x < g.x; ++x)
            for (int64_t y = 0; y < g.y; ++y)
                for (int64_t z = 0; z < g.z; ++z) fn(grid[utils::Coordinate<3>{x, y, z}], x, y, z);
    };
    fill(u.field, [](FieldNode& f, int64_t x, int64_t y, int64_t z) {
        f.E = {val(x, y, z, 1), val(x, y, z, 2), val(x, y, z, 3)};
        f.B = {val(x, y, z, 4), val(x, y, z, 5), val(x, y, z, 6)};
        f.Bext = {val(x, y, z, 7), val(x, y, z, 8), val(x, y, z, 9)};
    });
    fill(u.bcfield, [](BcFieldCell& f, int64_t x, int64_t y, int64_t z) {
        f.Bc = {val(x, y, z, 10), val(x, y, z, 11), val(x, y, z, 12)};
    });
    fill(u.currentDensity, [](DensityNode& f, int64_t x, int64_t y, int64_t z) {
        f.J = {val(x, y, z, 13), val(x, y, z, 14), val(x, y, z, 15)};
    });

    // pack: row-major order and the flat layouts of ipic3d_types.h
    std::vector<ipic3d_particle> parts;
    std::vector<uint64_t> counts;
    std::vector<double> field, bc, j;
    ipic3d_gpu::detail::pack_particles(u, parts, counts);
    ipic3d_gpu::detail::pack_fields(u, field, bc, j);
    int bad = 0;
    size_t i = 0;
    for (int64_t x = 0; x < s.x; ++x)
        for (int64_t y = 0; y < s.y; ++y)
            for (int64_t z = 0; z < s.z; ++z) {
                const auto& v = u.cells[utils::Coordinate<3>{x, y, z}].particles;
                if (counts[(x * s.y + y) * s.z + z] != v.size()) ++bad;
                for (const auto& p : v) {
                    const auto& q = parts[i++];
                    bad += q.position[0] != p.position.x || q.position[1] != p.position.y ||
                           q.position[2] != p.position.z || q.velocity[0] != p.velocity.x ||
                           q.velocity[1] != p.velocity.y || q.velocity[2] != p.velocity.z || q.q != p.q ||
                           q.qom != p.qom;
                }
            }
    const int64_t f1 = n + 3;
    bad += field[9 * ((1 * f1 + 2) * f1 + 3) + 4] != val(1, 2, 3, 5);  // B.y at node (1,2,3)
    bad += bc[3 * ((2 * (n + 2) + 0) * (n + 2) + 1) + 2] != val(2, 0, 1, 12);
    bad += j[3 * ((3 * (n + 1) + 1) * (n + 1) + 4) + 0] != val(3, 1, 4, 13);
    const ipic3d_props pp = ipic3d_gpu::detail::props_of(u.properties);
    bad += pp.size[1] != n || pp.cell_width[1] != 2.0 || pp.origin[2] != -3 || pp.external_b[2] != 1e-4;

    // unpack into a fresh universe: equal to the original
    Universe w(props);
    ipic3d_gpu::detail::unpack_particles(w, parts, counts);
    ipic3d_gpu::detail::unpack_fields(w, field, bc, j);
    for (int64_t x = 0; x < s.x; ++x)
        for (int64_t y = 0; y < s.y; ++y)
            for (int64_t z = 0; z < s.z; ++z) {
                const auto& a = u.cells[utils::Coordinate<3>{x, y, z}].particles;
                const auto& b = w.cells[utils::Coordinate<3>{x, y, z}].particles;
                if (a.size() != b.size()) {
                    ++bad;
                    continue;
                }
                for (size_t k = 0; k < a.size(); ++k)
                    bad += a[k].position.x != b[k].position.x || a[k].velocity.z != b[k].velocity.z ||
                           a[k].q != b[k].q;
            }
    fill(w.field, [&](FieldNode& f, int64_t x, int64_t y, int64_t z) {
        bad += f.E.x != val(x, y, z, 1) || f.Bext.z != val(x, y, z, 9);
    });
    std::printf("roundtrip mismatches %d\n", bad);

    // the GPU policy tags select the explicit specialization
    try {
        DurationMeasurement d = simulateSteps<ipic3d_gpu::no_projector, ipic3d_gpu::static_field_solver,
                                              ipic3d_gpu::dipole_particle_mover>(2, u);
        std::printf("stepped %.3f %.3f\n", d.firstStep, d.remainingSteps);
    } catch (const ipic3d_gpu::Error& e) {
        std::printf("status %d\n", e.status());
    }
    // the tracer helper over the reference's Particle and UniverseProperties
    std::vector<Particle> tracer_particles;
    for (const auto& q : parts) {
        Particle p;
        p.position = {q.position[0], q.position[1], q.position[2]};
        p.velocity = {q.velocity[0], q.velocity[1], q.velocity[2]};
        p.q = q.q;
        p.qom = q.qom;
        tracer_particles.push_back(p);
    }
    std::vector<std::uint32_t> frames(3 * n * n * n, 0);
    try {
        ipic3d_gpu::trace_particles(props, tracer_particles, 21, 10, 3, frames.data());
        std::printf("traced\n");
    } catch (const ipic3d_gpu::Error& e) {
        std::printf("trace status %d\n", e.status());
    }
    (void)argc;
    (void)argv;
    return bad ? 1 : 0;
}
