/*
 * Plain-C data types shared by the GB300 particle path's C ABI
 * (ipic3d_gpu.h), its CPU oracle and the tests.
 *
 * Every type mirrors a structure of the AllScale iPIC3D reference
 * (paths relative to code/app/include/ipic3d/app/):
 *   ipic3d_props     <- UniverseProperties   (universe_properties.h:52-123)
 *   ipic3d_particle  <- Particle              (particle.h:9-60), same 64-byte layout
 *   field arrays     <- Field / BcField / CurrentDensity (field.h:14-38)
 */
#ifndef IPIC3D_TYPES_H
#define IPIC3D_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* UniverseProperties (universe_properties.h:52-123). Only the members the
 * timestep reads; the output-cycle members and file base name stay on the
 * host driver. The reference requires a cubic grid (universe_properties.h:81);
 * this layer accepts any positive size. */
typedef struct ipic3d_props {
    int64_t size[3];        /* cells per axis                        */
    double cell_width[3];   /* cellWidth                             */
    double dt;              /* dt                                    */
    double speed_of_light;  /* speedOfLight                          */
    double planet_radius;   /* planetRadius                          */
    double object_center[3];/* objectCenter                          */
    double origin[3];       /* origin (front lower left corner)      */
    double external_b[3];   /* externalMagneticField                 */
} ipic3d_props;

/* Particle (particle.h:9-60): absolute position, velocity, charge q and
 * charge-over-mass qom, all FP64: 64 bytes, same order as the reference. */
typedef struct ipic3d_particle {
    double position[3];
    double velocity[3];
    double q;
    double qom;
} ipic3d_particle;

/* Field grid node (field.h:14-18): E, B, Bext, 9 doubles per node, on a
 * (size+3)^3 grid with one ghost layer (universe.h:36). BcFieldCell
 * (field.h:20-23): Bc, 3 doubles per cell centre on (size+2)^3.
 * DensityNode (field.h:25-27): J, 3 doubles per node on (size+1)^3.
 * All grids are row-major with x slowest (the Grid flatten of cell.h:521). */
#define IPIC3D_FIELD_NODE_DOUBLES 9
#define IPIC3D_BC_CELL_DOUBLES 3
#define IPIC3D_DENSITY_NODE_DOUBLES 3

/* Conserved quantities written by writeOutputData (simulator.h:73-91),
 * plus total charge and particle count. */
typedef struct ipic3d_conserved {
    double total_momentum;   /* sum (q/qom) |v|          cell.h:1329-1338 */
    double e_energy;         /* sum vol/2 |E|^2 / 4pi     field.h:443-459  */
    double b_energy;         /* same over |B + Bext|^2                      */
    double kinetic_energy;   /* sum 1/2 (q/qom) |v|^2     cell.h:1315-1324 */
    double total_charge;     /* sum q (not in the reference)                */
    uint64_t particles;      /* countParticlesInDomain    cell.h:87-100    */
} ipic3d_conserved;

#ifdef __cplusplus
}
#endif

#endif /* IPIC3D_TYPES_H */
