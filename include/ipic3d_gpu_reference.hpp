/*
 * The GB300 path behind the reference's own entry point: explicit
 * specializations of ipic3d::simulateSteps (simulator.h:42-47) for the
 * policy tags of ipic3d_gpu_simulator.hpp. A caller of the reference
 * switches a run to the GPU by naming the tags, e.g. in ipic3d.cxx:94
 *
 *   auto duration = simulateSteps<ipic3d_gpu::no_projector,
 *                                 ipic3d_gpu::static_field_solver,
 *                                 ipic3d_gpu::dipole_particle_mover>(params.ncycles, universe);
 *
 * and links libipic3d_gb300.so; Universe, Cell, Field, UniverseProperties and
 * the .inp driver stay the reference's. Include this header after the
 * reference's simulator.h is reachable on the include path
 * (code/app/include).
 */
#ifndef IPIC3D_GPU_REFERENCE_HPP
#define IPIC3D_GPU_REFERENCE_HPP

#include "ipic3d/app/simulator.h"
#include "ipic3d_gpu_simulator.hpp"

namespace ipic3d {

#define IPIC3D_GPU_SIMULATE_STEPS(P, F, M)                                                                  \
    template <>                                                                                             \
    inline DurationMeasurement simulateSteps<ipic3d_gpu::P, ipic3d_gpu::F, ipic3d_gpu::M>(std::uint64_t n, \
                                                                                         Universe& u) {     \
        const ipic3d_gpu::Durations d = ipic3d_gpu::simulate<ipic3d_gpu::P, ipic3d_gpu::F, ipic3d_gpu::M>(n, u); \
        return {d.firstStep, d.remainingSteps};                                                             \
    }
#define IPIC3D_GPU_SIMULATE_STEPS_SOLVERS(P, M)                 \
    IPIC3D_GPU_SIMULATE_STEPS(P, static_field_solver, M)        \
    IPIC3D_GPU_SIMULATE_STEPS(P, leapfrog_field_solver, M)      \
    IPIC3D_GPU_SIMULATE_STEPS(P, forward_field_solver, M)

IPIC3D_GPU_SIMULATE_STEPS_SOLVERS(no_projector, dipole_particle_mover)
IPIC3D_GPU_SIMULATE_STEPS_SOLVERS(no_projector, field_particle_mover)
IPIC3D_GPU_SIMULATE_STEPS_SOLVERS(cic_projector, dipole_particle_mover)
IPIC3D_GPU_SIMULATE_STEPS_SOLVERS(cic_projector, field_particle_mover)

#undef IPIC3D_GPU_SIMULATE_STEPS_SOLVERS
#undef IPIC3D_GPU_SIMULATE_STEPS

}  // namespace ipic3d

#endif /* IPIC3D_GPU_REFERENCE_HPP */
