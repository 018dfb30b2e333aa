// FP64 particle kernels: absolute positions, the reference's arithmetic
// order. Built with -fmad=false: no product-sum is fused, as on the
// reference's x86 build (explicit __fma_rn calls stay fused on purpose).
#include "particles_impl.cuh"

namespace ipg {
template <>
int launch_push<double>(const Geom& g, const PopSet<double>& S, int mode, const PushShape&, cudaStream_t st) {
    return launch_push_generic<double>(g, S, mode, st);
}
template <>
int launch_push_pending<double>(const Geom& g, const PopSet<double>& S, cudaStream_t st) {
    return launch_push_pending_generic<double>(g, S, st);
}
template int launch_inject<double>(const Geom&, const Pop<double>&, double, const double*, const double*, uint64_t,
                                   const uint64_t*, cudaStream_t);
template int launch_place<double>(const Geom&, const PopSet<double>&, cudaStream_t);
template int launch_pending_rotate<double>(const PopSet<double>&, uint64_t*, cudaStream_t);
template int launch_relayout<double>(const Pop<double>&, const Pop<double>&, int, int32_t*, cudaStream_t);
template int launch_pending_count<double>(const Pop<double>&, int32_t*, cudaStream_t);

template <>
int launch_push_batch<double>(const PopJob<double>* jobs, const int2* cta_job, int64_t nctas, int mode,
                              const Geom&, const PushShape&, cudaStream_t st) {
    return launch_push_batch_generic<double>(jobs, cta_job, nctas, mode, st);
}
template <>
int launch_push_pending_batch<double>(const PopJob<double>* jobs, int njobs, cudaStream_t st) {
    return launch_push_pending_batch_generic<double>(jobs, njobs, st);
}
template int launch_place_batch<double>(const PopJob<double>*, const int2*, int64_t, cudaStream_t);
template int launch_pending_rotate_batch<double>(const PopJob<double>*, int, cudaStream_t);
template int launch_batch_begin<double>(const PopJob<double>*, int, const InstJob*, int, int64_t, int, uint32_t*,
                                        cudaStream_t);
template int launch_batch_end<double>(const PopJob<double>*, const InstJob*, int, uint32_t*, cudaStream_t);
template int launch_batch_status<double>(const PopJob<double>*, int, JobStatus*, cudaStream_t);
}  // namespace ipg

#include "../../include/ipic3d_types.h"

namespace ipg {

// Particle::updateVelocity + updatePosition (particle.h:24-49), nsteps times,
// uniform E and B: the element kernel behind the Boris known-answer tests.
__global__ void k_boris(ipic3d_particle* p, uint64_t n, double ex, double ey, double ez, double bx, double by,
                        double bz, double dt, uint64_t nsteps, int push_position) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    ipic3d_particle q = p[i];
    for (uint64_t t = 0; t < nsteps; ++t) {
        boris<double>(q.velocity[0], q.velocity[1], q.velocity[2], ex, ey, ez, bx, by, bz, q.qom, dt);
        if (push_position) {
            q.position[0] = q.position[0] + q.velocity[0] * dt;
            q.position[1] = q.position[1] + q.velocity[1] * dt;
            q.position[2] = q.position[2] + q.velocity[2] * dt;
        }
    }
    p[i] = q;
}

int launch_boris(const void* parts, uint64_t n, const double E[3], const double B[3], double dt, uint64_t nsteps,
                 int push_position, void* out, cudaStream_t st) {
    (void)parts;
    k_boris<<<(unsigned)((n + 127) / 128), 128, 0, st>>>((ipic3d_particle*)out, n, E[0], E[1], E[2], B[0], B[1], B[2],
                                                          dt, nsteps, push_position);
    return 1;
}

}  // namespace ipg
