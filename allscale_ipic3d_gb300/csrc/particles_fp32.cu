// FP32 particle kernels: positions relative to the cell origin, FP32 push
// with fused multiply-adds, FP64 node accumulation of the deposit.
#include "particles_impl.cuh"
#include "push32.cuh"

namespace ipg {

Push32Const push32_const(const Geom& g, const Pop<float>& P) {
    Push32Const pc;
    pc.qom = (float)P.qom;
    pc.k_sub = (float)(g.dt * 4.0 * fabs(P.qom) / (3.14159265358979323846 * g.c));
    pc.dt = (float)g.dt;
    pc.mft = (float)g.mft;
    pc.planet_r2 = (float)g.planet_r2;
    for (int a = 0; a < 3; ++a) {
        pc.w[a] = (float)g.w[a];
        pc.inv_w[a] = (float)g.inv_w[a];
        pc.origin[a] = (float)g.origin[a];
        pc.center[a] = (float)g.object_center[a];
    }
    pc.inv_sy = 1.0f / (float)g.sy;
    pc.inv_sz = 1.0f / (float)g.sz;
    return pc;
}

// the FP32 step uses the lean kernels of push32.cuh
template <>
int launch_push<float>(const Geom& g, const Pop<float>& P, int mode, cudaStream_t st) {
    if (P.capacity <= 0) return 0;
    const int64_t blocks = (P.capacity + kSlotsPerCta - 1) / kSlotsPerCta;
    k_push32<3><<<(unsigned)blocks, kPushThreads, 0, st>>>(g, P, push32_const(g, P), mode);
    return 1;
}

template <>
int launch_push_pending<float>(const Geom& g, const Pop<float>& P, cudaStream_t st) {
    k_push_pending32<<<152, 128, 0, st>>>(g, P, push32_const(g, P));
    return 1;
}

int launch_cell_coef(const Geom& g, float* coef, cudaStream_t st) {
    const int64_t n = (int64_t)g.sx * g.sy * g.sz;
    int64_t blocks = (n + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    const double scale = (g.flags & 2u) ? 1.0 / g.vol : 1.0;
    k_cell_coef<<<(unsigned)blocks, 128, 0, st>>>(g.field, g.sx, g.sy, g.sz, scale, coef);
    return 1;
}

template <>
int launch_push_batch<float>(const PopJob<float>* jobs, const int2* cta_job, int64_t nctas, int mode,
                             cudaStream_t st) {
    if (nctas <= 0) return 0;
    k_push32_batch<3><<<(unsigned)nctas, kPushThreads, 0, st>>>(jobs, cta_job, mode);
    return 1;
}

template <>
int launch_push_pending_batch<float>(const PopJob<float>* jobs, int njobs, cudaStream_t st) {
    k_push_pending32_batch<<<dim3(2, njobs), 128, 0, st>>>(jobs);
    return 1;
}

int launch_cell_coef_batch(const InstJob* inst, int ninst, int64_t max_cells, cudaStream_t st) {
    int64_t blocks = (max_cells + 127) / 128;
    if (blocks > 64) blocks = 64;
    k_cell_coef_batch<<<dim3((unsigned)blocks, ninst), 128, 0, st>>>(inst);
    return 1;
}

template int launch_place_batch<float>(const PopJob<float>*, const int2*, int64_t, cudaStream_t);
template int launch_pending_rotate_batch<float>(const PopJob<float>*, int, cudaStream_t);
template int launch_batch_begin<float>(const PopJob<float>*, int, const InstJob*, int, int64_t, int, uint32_t*,
                                       cudaStream_t);
template int launch_batch_end<float>(const PopJob<float>*, const InstJob*, int, uint32_t*, cudaStream_t);
template int launch_batch_status<float>(const PopJob<float>*, int, JobStatus*, cudaStream_t);
template int launch_inject<float>(const Geom&, const Pop<float>&, double, const double*, const double*, uint64_t,
                                  const uint64_t*, cudaStream_t);
template int launch_place<float>(const Geom&, const Pop<float>&, int32_t*, cudaStream_t);
template int launch_pending_rotate<float>(const Pop<float>&, uint32_t*, cudaStream_t);
template int launch_relayout<float>(const Pop<float>&, const Pop<float>&, int, int32_t*, cudaStream_t);
template int launch_pending_count<float>(const Pop<float>&, int32_t*, cudaStream_t);
}  // namespace ipg
