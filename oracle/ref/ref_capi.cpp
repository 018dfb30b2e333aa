// C-callable wrappers around the reference's own per-phase functions,
// compiled from the reference's headers in place (code/app/include) against
// the AllScale shim. Built into oracle/_ref/libipic3d_ref.so by ref/Makefile.
//
// TEST INFRASTRUCTURE ONLY. Used on the build machine (where the reference
// sources exist) to pin the CPU restatement in oracle/ipic3d_oracle.cpp and
// to generate the fixtures under tests/golden/. Nothing on the product path
// links it.
#include <cstring>
#include <vector>

#include "ipic3d/app/cell.h"
#include "ipic3d/app/field.h"
#include "ipic3d/app/parameters.h"
#include "ipic3d/app/simulator.h"
#include "ipic3d/app/universe.h"

#include "../../include/ipic3d_types.h"

using namespace ipic3d;

namespace {

UniverseProperties to_props(const ipic3d_props* p) {
    UniverseProperties u;
    u.size = {p->size[0], p->size[1], p->size[2]};
    u.cellWidth = {p->cell_width[0], p->cell_width[1], p->cell_width[2]};
    u.dt = p->dt;
    u.speedOfLight = p->speed_of_light;
    u.planetRadius = p->planet_radius;
    u.objectCenter = {p->object_center[0], p->object_center[1], p->object_center[2]};
    u.origin = {p->origin[0], p->origin[1], p->origin[2]};
    u.externalMagneticField = {p->external_b[0], p->external_b[1], p->external_b[2]};
    u.useCase = UseCase::Dipole;
    return u;
}

void from_props(const UniverseProperties& u, ipic3d_props* p) {
    for (int i = 0; i < 3; ++i) {
        p->size[i] = u.size[i];
        p->cell_width[i] = u.cellWidth[i];
        p->object_center[i] = u.objectCenter[i];
        p->origin[i] = u.origin[i];
        p->external_b[i] = u.externalMagneticField[i];
    }
    p->dt = u.dt;
    p->speed_of_light = u.speedOfLight;
    p->planet_radius = u.planetRadius;
}

Particle to_particle(const ipic3d_particle& a) {
    Particle p;
    p.position = {a.position[0], a.position[1], a.position[2]};
    p.velocity = {a.velocity[0], a.velocity[1], a.velocity[2]};
    p.q = a.q;
    p.qom = a.qom;
    return p;
}

ipic3d_particle from_particle(const Particle& p) {
    ipic3d_particle a;
    for (int i = 0; i < 3; ++i) {
        a.position[i] = p.position[i];
        a.velocity[i] = p.velocity[i];
    }
    a.q = p.q;
    a.qom = p.qom;
    return a;
}

void fill_cells(Cells& cells, const ipic3d_particle* in, const uint64_t* counts) {
    auto s = cells.size();
    uint64_t k = 0, c = 0;
    for (int64_t x = 0; x < s.x; ++x)
        for (int64_t y = 0; y < s.y; ++y)
            for (int64_t z = 0; z < s.z; ++z, ++c)
                for (uint64_t i = 0; i < counts[c]; ++i) cells[{x, y, z}].particles.push_back(to_particle(in[k++]));
}

int drain_cells(const Cells& cells, ipic3d_particle* out, uint64_t cap, uint64_t* counts) {
    auto s = cells.size();
    uint64_t k = 0, c = 0;
    for (int64_t x = 0; x < s.x; ++x)
        for (int64_t y = 0; y < s.y; ++y)
            for (int64_t z = 0; z < s.z; ++z, ++c) {
                const auto& v = cells[{x, y, z}].particles;
                counts[c] = v.size();
                for (const auto& p : v) {
                    if (k >= cap) return -1;
                    out[k++] = from_particle(p);
                }
            }
    return 0;
}

template <typename G>
void grid_in(G& g, const double* a, int per) {
    std::memcpy((void*)g.raw(), a, sizeof(double) * per * (size_t)(g.size().x * g.size().y * g.size().z));
}
template <typename G>
void grid_out(const G& g, double* a, int per) {
    std::memcpy(a, (const void*)g.raw(), sizeof(double) * per * (size_t)(g.size().x * g.size().y * g.size().z));
}

}  // namespace

static_assert(sizeof(FieldNode) == 9 * sizeof(double), "FieldNode layout");
static_assert(sizeof(BcFieldCell) == 3 * sizeof(double), "BcFieldCell layout");
static_assert(sizeof(DensityNode) == 3 * sizeof(double), "DensityNode layout");

extern "C" {

// simulateSteps with the reference's default policies (simulator.h:127-242):
// per step, moveParticles + exportParticles over all cells, then
// importParticles. Particles are grouped by cell (row-major), counts[c] each.
// Each particle's q is replaced by its input index while the loop runs (the
// default mover, export and import never read q) so the caller can follow
// particles; ids_out receives those indices and q is restored.
int ref_simulate_default(const ipic3d_props* props, const ipic3d_particle* in, const uint64_t* counts, uint64_t steps,
                         ipic3d_particle* out, uint64_t out_cap, uint64_t* out_counts, uint32_t* ids_out) {
    Universe u(to_props(props));
    auto s = u.cells.size();
    uint64_t ncells = (uint64_t)(s.x * s.y * s.z), n = 0;
    for (uint64_t c = 0; c < ncells; ++c) n += counts[c];
    std::vector<double> q(n);
    std::vector<ipic3d_particle> tagged(in, in + n);
    for (uint64_t i = 0; i < n; ++i) {
        q[i] = tagged[i].q;
        tagged[i].q = (double)i;
    }
    fill_cells(u.cells, tagged.data(), counts);
    simulateSteps(steps, u);
    if (drain_cells(u.cells, out, out_cap, out_counts)) return -1;
    uint64_t m = 0;
    for (uint64_t c = 0; c < ncells; ++c) m += out_counts[c];
    for (uint64_t i = 0; i < m; ++i) {
        uint64_t id = (uint64_t)out[i].q;
        if (ids_out) ids_out[i] = (uint32_t)id;
        out[i].q = q[id];
    }
    return 0;
}

// One call of moveParticles (cell.h:896-964) on a list of particles located
// in cell `pos` (no export): the analytic dipole mover with sub-cycling.
int ref_move_particles(const ipic3d_props* props, const int64_t pos[3], ipic3d_particle* ps, uint64_t n) {
    UniverseProperties u = to_props(props);
    Cell cell;
    for (uint64_t i = 0; i < n; ++i) cell.particles.push_back(to_particle(ps[i]));
    Field dummy(coordinate_type(1));
    moveParticles(u, cell, {pos[0], pos[1], pos[2]}, dummy);
    for (uint64_t i = 0; i < n; ++i) ps[i] = from_particle(cell.particles[i]);
    return 0;
}

// Particle::updateVelocity then updatePosition (particle.h:24-49), nsteps times.
int ref_boris(ipic3d_particle* p, const double E[3], const double B[3], double dt, uint64_t nsteps, int push_position) {
    Particle q = to_particle(*p);
    Vector3<double> e{E[0], E[1], E[2]}, b{B[0], B[1], B[2]};
    for (uint64_t i = 0; i < nsteps; ++i) {
        q.updateVelocity(e, b, dt);
        if (push_position) q.updatePosition(dt);
    }
    *p = from_particle(q);
    return 0;
}

// projectToDensityField (cell.h:787-824) for every node of the
// (size+1)^3 CurrentDensity grid; J receives 3 doubles per node.
int ref_project_current(const ipic3d_props* props, const ipic3d_particle* in, const uint64_t* counts, double* J) {
    Universe u(to_props(props));
    fill_cells(u.cells, in, counts);
    auto sz = u.currentDensity.size();
    for (int64_t x = 0; x < sz.x; ++x)
        for (int64_t y = 0; y < sz.y; ++y)
            for (int64_t z = 0; z < sz.z; ++z) projectToDensityField(u.properties, u.cells, {x, y, z}, u.currentDensity);
    grid_out(u.currentDensity, J, 3);
    return 0;
}

// aggregateDensityContributions (cell.h:835-855) for every node of the
// (size+1)^3 CurrentDensity grid from a (2 size)^3 contribution grid (the
// buffer of simulator.h:156); J (3 doubles per node) is read and updated in
// place, as the reference adds into the node's J.
int ref_aggregate_contributions(const ipic3d_props* props, const double* contrib, double* J) {
    Universe u(to_props(props));
    CurrentDensity c(u.properties.size * 2);
    grid_in(c, contrib, 3);
    grid_in(u.currentDensity, J, 3);
    auto sz = u.currentDensity.size();
    for (int64_t x = 0; x < sz.x; ++x)
        for (int64_t y = 0; y < sz.y; ++y)
            for (int64_t z = 0; z < sz.z; ++z)
                aggregateDensityContributions(u.properties, c, {x, y, z}, u.currentDensity[{x, y, z}]);
    grid_out(u.currentDensity, J, 3);
    return 0;
}

// updateFieldsOnBoundaries (field.h:407-440) on a (size+3)^3 Field and a
// (size+2)^3 BcField.
int ref_update_boundaries(const ipic3d_props* props, double* field, double* bcfield) {
    Universe u(to_props(props));
    grid_in(u.field, field, 9);
    grid_in(u.bcfield, bcfield, 3);
    updateFieldsOnBoundaries(u.field, u.bcfield);
    grid_out(u.field, field, 9);
    grid_out(u.bcfield, bcfield, 3);
    return 0;
}

// solveFieldLeapfrog (field.h:342-402) over the box [1, size+2)^3 that the
// commented step uses (simulator.h:146-147,207-209). The per-node function
// updates E at pos and then Bc at pos from E at pos+e_i, so its result
// depends on the visiting order. Visiting nodes in reverse row-major order
// makes every E read by a Bc update already new and every Bc read by an E
// update still old: the two-phase (all E, then all Bc) leapfrog.
int ref_leapfrog_two_phase(const ipic3d_props* props, double* field, double* bcfield, const double* J) {
    Universe u(to_props(props));
    grid_in(u.field, field, 9);
    grid_in(u.bcfield, bcfield, 3);
    grid_in(u.currentDensity, const_cast<double*>(J), 3);
    auto fs = u.field.size();
    for (int64_t x = fs.x - 2; x >= 1; --x)
        for (int64_t y = fs.y - 2; y >= 1; --y)
            for (int64_t z = fs.z - 2; z >= 1; --z)
                solveFieldLeapfrog(u.properties, {x, y, z}, u.currentDensity, u.field, u.bcfield);
    grid_out(u.field, field, 9);
    grid_out(u.bcfield, bcfield, 3);
    return 0;
}

// solveFieldForward (field.h:294-337) at one node (the reference's tests call
// it node by node, field_test.cc:453,502).
int ref_solve_forward_at(const ipic3d_props* props, const int64_t pos[3], double* field, double* bcfield, const double* J) {
    Universe u(to_props(props));
    grid_in(u.field, field, 9);
    grid_in(u.bcfield, bcfield, 3);
    grid_in(u.currentDensity, const_cast<double*>(J), 3);
    solveFieldForward(u.properties, {pos[0], pos[1], pos[2]}, u.currentDensity, u.field, u.bcfield);
    grid_out(u.field, field, 9);
    grid_out(u.bcfield, bcfield, 3);
    return 0;
}

// trilinearInterpolationF2P (cell.h:867-885) on a scalar corner set.
double ref_trilinear(const double corners[8], const double pos[3], double vol) {
    double c[2][2][2];
    std::memcpy(c, corners, sizeof(c));
    return trilinearInterpolationF2P(c, Vector3<double>{pos[0], pos[1], pos[2]}, vol);
}

// Conserved quantities as writeOutputData computes them (simulator.h:76-83).
int ref_conserved(const ipic3d_props* props, const ipic3d_particle* in, const uint64_t* counts, const double* field,
                  ipic3d_conserved* out) {
    Universe u(to_props(props));
    fill_cells(u.cells, in, counts);
    grid_in(u.field, field, 9);
    auto getE = [](const auto& f, const auto& index) { return f[index].E; };
    auto getB = [](const auto& f, const auto& index) { return (f[index].B + f[index].Bext); };
    out->e_energy = getFieldEnergy(u.field, u.properties, getE);
    out->b_energy = getFieldEnergy(u.field, u.properties, getB);
    out->total_momentum = getTotalParticlesEnergy(u.cells, getParticlesMomentum);
    out->kinetic_energy = getTotalParticlesEnergy(u.cells, getParticlesKineticEnergy);
    out->particles = countParticlesInDomain(u.cells);
    double q = 0;
    for (uint64_t i = 0; i < out->particles; ++i) q += in[i].q;
    out->total_charge = q;
    return 0;
}

// outputParticlePositions (cell.h:1400-1429) of the given particles (grouped
// by cell) into the file `path`.
int ref_write_particle_positions(const ipic3d_props* props, const ipic3d_particle* in, const uint64_t* counts,
                                 const char* path) {
    Universe u(to_props(props));
    fill_cells(u.cells, in, counts);
    outputParticlePositions(u.cells, std::string(path));
    return 0;
}

// outputFieldGrids (field.h:464-530) of the given Field ((size+3)^3 x 9) and
// BcField ((size+2)^3 x 3) into the file `path`.
int ref_write_field_grids(const ipic3d_props* props, const double* field, const double* bcfield, const char* path) {
    Universe u(to_props(props));
    grid_in(u.field, const_cast<double*>(field), 9);
    grid_in(u.bcfield, const_cast<double*>(bcfield), 3);
    outputFieldGrids(u.field, u.bcfield, std::string(path));
    return 0;
}

// The .inp driver's set-up (src/ipic3d.cxx:30-83): parse, apply the driver's
// overrides, build the universe with createUniverseFromDistribution. Returns
// props, the field grid, the particles grouped by cell and ncycles. Call with
// out == NULL to query n_out first.
int ref_init_from_inp(const char* path, ipic3d_props* props_out, uint64_t* ncycles, ipic3d_particle* out,
                      uint64_t cap, uint64_t* counts, uint64_t* n_out, double* field_out) {
    auto params = Parameters(path);
    InitProperties initProperties = InitProperties(params);
    UniverseProperties universeProperties = UniverseProperties(params);
    universeProperties.dt = 0.01;
    universeProperties.speedOfLight = 299792458;
    universeProperties.planetRadius = 6378137;
    universeProperties.cellWidth *= universeProperties.planetRadius;
    auto universeSize = elementwiseProduct(universeProperties.cellWidth, universeProperties.size);
    universeProperties.objectCenter = {0.0, 0.0, 0.0};
    universeProperties.origin = universeProperties.objectCenter - universeSize / 2.0;
    universeProperties.externalMagneticField = {0.0, 0.0, 3.07e-5};
    universeProperties.useCase = UseCase::Dipole;
    int numParticles = universeProperties.size.x * universeProperties.size.y * universeProperties.size.z;
    numParticles = numParticles * initProperties.particlesPerCell[0].x * initProperties.particlesPerCell[0].y *
                   initProperties.particlesPerCell[0].z;
    double e = 1.602176565e-19;
    double K = 1e7 * e;
    double m = 1.672621777e-27;
    double v_mod = universeProperties.speedOfLight /
                   sqrt(1.0 + (m * universeProperties.speedOfLight * universeProperties.speedOfLight) / K);
    auto low = universeProperties.origin + 0.125 * universeSize;
    auto hig = low + 0.75 * universeSize;
    auto dist = distribution::uniform_pos_normal_speed<>(low, hig, Vector3<double>{0, 0, 0},
                                                         Vector3<double>{v_mod, v_mod, v_mod});
    auto universe = createUniverseFromDistribution(universeProperties, initProperties, numParticles, dist);
    from_props(universe.properties, props_out);
    *ncycles = params.ncycles;
    *n_out = countParticlesInDomain(universe.cells);
    if (!out) return 0;
    if (field_out) grid_out(universe.field, field_out, 9);
    return drain_cells(universe.cells, out, cap, counts);
}

}  // extern "C"
