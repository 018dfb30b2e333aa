// The C++ drop-in (include/ipic3d_gpu_simulator.hpp) on a stand-in Universe
// with the reference's member names (universe.h:12-51): writes the initial
// particles and the ones after `steps` GPU steps, for the Python test to
// compare with the C ABI path.
//
//   adapter_standin <policy 0|1> <precision 0|1> <steps> <out prefix>
//   policy 0: no_projector + static_field_solver + dipole_particle_mover
//   policy 1: cic_projector + leapfrog_field_solver + field_particle_mover
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "ipic3d_gpu_simulator.hpp"

namespace standin {

struct Coord {
    int64_t x, y, z;
};
struct Vec {
    double x, y, z;
};
template <class T>
struct Grid {
    Coord s;
    std::vector<T> data;
    explicit Grid(Coord size) : s(size), data((size_t)(size.x * size.y * size.z)) {}
    Coord size() const { return s; }
    T& operator[](const Coord& c) { return data[(size_t)((c.x * s.y + c.y) * s.z + c.z)]; }
    const T& operator[](const Coord& c) const { return data[(size_t)((c.x * s.y + c.y) * s.z + c.z)]; }
};
struct Particle {
    Vec position, velocity;
    double q, qom;
};
struct Cell {
    std::vector<Particle> particles;
};
struct FieldNode {
    Vec E, B, Bext;
};
struct BcFieldCell {
    Vec Bc;
};
struct DensityNode {
    Vec J;
};
struct Properties {
    Coord size;
    Vec cellWidth;
    double dt, speedOfLight, planetRadius;
    Vec objectCenter, origin, externalMagneticField;
};
struct Universe {
    Properties properties;
    Grid<Cell> cells;
    Grid<FieldNode> field;
    Grid<BcFieldCell> bcfield;
    Grid<DensityNode> currentDensity;
    explicit Universe(const Properties& p)
        : properties(p),
          cells(p.size),
          field({p.size.x + 3, p.size.y + 3, p.size.z + 3}),
          bcfield({p.size.x + 2, p.size.y + 2, p.size.z + 2}),
          currentDensity({p.size.x + 1, p.size.y + 1, p.size.z + 1}) {}
};

}  // namespace standin

static uint64_t g_state = 0x2545F4914F6CDD1DULL;
static double uni() {  // xorshift64*, uniform in [0, 1)
    g_state ^= g_state >> 12;
    g_state ^= g_state << 25;
    g_state ^= g_state >> 27;
    return (double)((g_state * 0x2545F4914F6CDD1DULL) >> 11) * (1.0 / 9007199254740992.0);
}

static void dump(const char* path, const standin::Universe& u) {
    std::vector<ipic3d_particle> parts;
    std::vector<uint64_t> counts;
    ipic3d_gpu::detail::pack_particles(u, parts, counts);
    FILE* f = std::fopen(path, "wb");
    const uint64_t n = parts.size(), nc = counts.size();
    std::fwrite(&n, 8, 1, f);
    std::fwrite(&nc, 8, 1, f);
    std::fwrite(counts.data(), 8, nc, f);
    std::fwrite(parts.data(), sizeof(ipic3d_particle), n, f);
    std::fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    const int policy = std::atoi(argv[1]);
    ipic3d_gpu::options().precision = std::atoi(argv[2]) ? IPIC3D_FP32 : IPIC3D_FP64;
    const uint64_t steps = std::strtoull(argv[3], nullptr, 10);
    const std::string prefix = argv[4];
    standin::Properties p{};
    p.size = {6, 6, 6};
    p.cellWidth = {1.0, 1.0, 1.0};
    p.dt = 0.1;
    p.speedOfLight = 1.0;
    if (policy == 0) {  // the reference's dipole loop: planet at the centre
        p.cellWidth = {10.0, 10.0, 10.0};
        p.origin = {-30.0, -30.0, -30.0};
        p.planetRadius = 8.0;
        p.externalMagneticField = {0.0, 0.0, 1e-4};
        p.dt = 0.15;
    } else {
        for (int a = 0; a < 3; ++a) ipic3d_gpu::options().bc_low[a] = ipic3d_gpu::options().bc_high[a] = IPIC3D_BC_PERIODIC;
        ipic3d_gpu::options().flags = IPIC3D_F_USE_GRAPH | IPIC3D_F_REFRESH_NODE_B;
    }
    standin::Universe u(p);
    for (int64_t x = 0; x < 6; ++x)
        for (int64_t y = 0; y < 6; ++y)
            for (int64_t z = 0; z < 6; ++z) {
                auto& cell = u.cells[{x, y, z}];
                const int n = 4 + (int)(uni() * 12);
                for (int k = 0; k < n; ++k) {
                    standin::Particle q;
                    q.position = {p.origin.x + (x + uni()) * p.cellWidth.x, p.origin.y + (y + uni()) * p.cellWidth.y,
                                  p.origin.z + (z + uni()) * p.cellWidth.z};
                    q.velocity = {0.4 * (uni() - 0.5), 0.4 * (uni() - 0.5), 0.4 * (uni() - 0.5)};
                    const bool ion = k & 1;
                    q.q = ion ? 0.05 : -0.05;
                    q.qom = ion ? 0.01 : -1.0;
                    cell.particles.push_back(q);
                }
            }
    if (policy == 1) {  // uniform E, B
        for (auto& f : u.field.data) {
            f.E = {0.0, 0.01, 0.0};
            f.B = {0.0, 0.0, 0.1};
        }
        for (auto& b : u.bcfield.data) b.Bc = {0.0, 0.0, 0.1};
    }
    dump((prefix + "_in.bin").c_str(), u);
    std::ofstream trace;
    if (argc > 5) {  // the debug-build trace of the conserved quantities and the density files
        trace.open(argv[5]);
        ipic3d_gpu::options().trace = &trace;
        ipic3d_gpu::options().density_prefix = std::string(argv[5]) + ".csv.";
        ipic3d_gpu::options().density_every = 2;
    }
    try {
        if (policy == 0)
            ipic3d_gpu::simulate<ipic3d_gpu::no_projector, ipic3d_gpu::static_field_solver,
                                 ipic3d_gpu::dipole_particle_mover>(steps, u);
        else
            ipic3d_gpu::simulate<ipic3d_gpu::cic_projector, ipic3d_gpu::leapfrog_field_solver,
                                 ipic3d_gpu::field_particle_mover>(steps, u);
    } catch (const ipic3d_gpu::Error& e) {
        std::printf("status %d: %s\n", e.status(), e.what());
        return 1;
    }
    dump((prefix + "_out.bin").c_str(), u);
    std::printf("ok\n");
    return 0;
}
