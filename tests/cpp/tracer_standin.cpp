// ipic3d_gpu::trace_particles (include/ipic3d_gpu_simulator.hpp) on stand-in
// types with the reference's member names (UniverseProperties,
// universe_properties.h:52-123; Particle, particle.h:9-60): pic_tracer's
// configuration for an R^3 grid (pic_tracer.cxx:196-214), particles read
// from a file of 64-byte records, the histogram written to a file, for the
// Python test to compare with the C ABI path.
//
//   tracer_standin <R> <steps> <frame interval> <frames> <particles.bin> <counts.bin>
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
struct Particle {
    Vec position, velocity;
    double q, qom;
};
struct Properties {
    Coord size;
    Vec cellWidth;
    double dt, speedOfLight, planetRadius;
    Vec objectCenter, origin, externalMagneticField;
};

}  // namespace standin

int main(int argc, char** argv) {
    if (argc < 7) return 2;
    const int R = std::atoi(argv[1]), steps = std::atoi(argv[2]), S = std::atoi(argv[3]), F = std::atoi(argv[4]);
    standin::Properties config;
    config.dt = 0.01;
    config.speedOfLight = 299792458;
    config.size = {R, R, R};
    config.planetRadius = 6378137;
    const double w = (20.0 / config.size.x) * config.planetRadius;
    config.cellWidth = {w, w, w};
    config.objectCenter = {0.0, 0.0, 0.0};
    config.origin = {config.objectCenter.x - config.size.x * config.cellWidth.x / 2.0,
                     config.objectCenter.y - config.size.y * config.cellWidth.y / 2.0,
                     config.objectCenter.z - config.size.z * config.cellWidth.z / 2.0};
    config.externalMagneticField = {0.0, 0.0, 3.07e-5};

    std::ifstream in(argv[5], std::ios::binary);
    std::vector<standin::Particle> particles;
    double rec[8];
    while (in.read(reinterpret_cast<char*>(rec), sizeof rec))
        particles.push_back({{rec[0], rec[1], rec[2]}, {rec[3], rec[4], rec[5]}, rec[6], rec[7]});
    std::vector<std::uint32_t> counts((size_t)F * R * R * R, 0);
    try {
        ipic3d_gpu::trace_particles(config, particles, steps, S, F, counts.data());
    } catch (const ipic3d_gpu::Error& e) {
        std::printf("status %d\n", e.status());
        return 1;
    }
    std::ofstream out(argv[6], std::ios::binary);
    out.write(reinterpret_cast<const char*>(counts.data()), (std::streamsize)(counts.size() * sizeof(std::uint32_t)));
    std::printf("traced %zu\n", particles.size());
    return 0;
}
