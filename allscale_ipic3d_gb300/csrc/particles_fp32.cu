// FP32 particle kernels: positions relative to the cell origin, FP32 push
// with fused multiply-adds, FP64 node accumulation of the deposit.
#include <algorithm>
#include <mutex>

#include "particles_impl.cuh"
#include "push32.cuh"
#include "push32_pipe.cuh"

namespace ipg {

namespace {
constexpr int kMaxDevices = 64;
constexpr int kPipeStages = 3;  // shared-memory stages per CTA (2 CTAs per SM)
std::mutex g_pipe_mu;
bool g_pipe_ready[kMaxDevices] = {};
int g_pipe_per_sm[kMaxDevices] = {};  // resident blocks per SM of the pipelined push
int g_pipe_sms[kMaxDevices] = {};

using PipeFn = void (*)(Geom, PopSet<float>, Push32Set, TileMap, PushShape);
using PipeJobsFn = void (*)(const PopJob<float>*, const int2*, int, PushShape);

// The compile-time policies that are instantiated (kPipe* bit sets): the
// step with the dipole mover, the field-gather mover with or without the
// dipole term, each with or without the deposit; and the deposit alone.
constexpr int kPipeVariants[] = {
    kPipeStep | kPipeDipole,
    kPipeStep | kPipeDipole | kPipeDeposit,
    kPipeStep | kPipeGather,
    kPipeStep | kPipeGather | kPipeDeposit,
    kPipeStep | kPipeGather | kPipeDipole,
    kPipeStep | kPipeGather | kPipeDipole | kPipeDeposit,
    kPipeDeposit,
};

template <int kF>
constexpr PipeFn pipe_fn() {
    return k_push32_pipe<kPipeStages, 2, kF>;
}

template <int kF>
constexpr PipeJobsFn pipe_jobs_fn() {
    return k_push32_pipe_jobs<kPipeStages, 2, kF>;
}

PipeJobsFn pipe_jobs_kernel(int f) {
    switch (f) {
        case kPipeStep | kPipeDipole: return pipe_jobs_fn<kPipeStep | kPipeDipole>();
        case kPipeStep | kPipeDipole | kPipeDeposit: return pipe_jobs_fn<kPipeStep | kPipeDipole | kPipeDeposit>();
        case kPipeStep | kPipeGather: return pipe_jobs_fn<kPipeStep | kPipeGather>();
        case kPipeStep | kPipeGather | kPipeDeposit: return pipe_jobs_fn<kPipeStep | kPipeGather | kPipeDeposit>();
        case kPipeStep | kPipeGather | kPipeDipole: return pipe_jobs_fn<kPipeStep | kPipeGather | kPipeDipole>();
        case kPipeStep | kPipeGather | kPipeDipole | kPipeDeposit:
            return pipe_jobs_fn<kPipeStep | kPipeGather | kPipeDipole | kPipeDeposit>();
        case kPipeDeposit: return pipe_jobs_fn<kPipeDeposit>();
        default: return nullptr;
    }
}

// The policy bits of a launch: mode 0 = step, 1 = deposit only.
int pipe_policy(const Geom& g, int mode) {
    int f = g.deposit ? kPipeDeposit : 0;
    if (mode == 0) {
        f |= kPipeStep;
        if (g.mover == 1) f |= kPipeGather;
        if (g.mover != 1 || (g.flags & 4u)) f |= kPipeDipole;
    }
    return f;
}

PipeFn pipe_kernel(int f) {
    switch (f) {
        case kPipeStep | kPipeDipole: return pipe_fn<kPipeStep | kPipeDipole>();
        case kPipeStep | kPipeDipole | kPipeDeposit: return pipe_fn<kPipeStep | kPipeDipole | kPipeDeposit>();
        case kPipeStep | kPipeGather: return pipe_fn<kPipeStep | kPipeGather>();
        case kPipeStep | kPipeGather | kPipeDeposit: return pipe_fn<kPipeStep | kPipeGather | kPipeDeposit>();
        case kPipeStep | kPipeGather | kPipeDipole: return pipe_fn<kPipeStep | kPipeGather | kPipeDipole>();
        case kPipeStep | kPipeGather | kPipeDipole | kPipeDeposit:
            return pipe_fn<kPipeStep | kPipeGather | kPipeDipole | kPipeDeposit>();
        case kPipeDeposit: return pipe_fn<kPipeDeposit>();
        default: return nullptr;
    }
}
}  // namespace

// Once per device (the device current): shared-memory opt-in and persistent
// grid size of the pipelined push kernels. Called when a context is created,
// before any stream capture.
cudaError_t init_push32(int dev) {
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_pipe_mu);
    if (g_pipe_ready[dev]) return cudaSuccess;
    const int bytes = (int)pipe_smem_bytes<kPipeStages>();
    int min_per_sm = 1 << 30;
    for (int f : kPipeVariants) {
        PipeFn fn = pipe_kernel(f);
        PipeJobsFn fj = pipe_jobs_kernel(f);
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(fj, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        int per_sm = 0, per_sm_j = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kPipeThreads, bytes);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_j, fj, kPipeThreads, bytes);
        if (e != cudaSuccess) return e;
        min_per_sm = std::min(min_per_sm, std::min(per_sm, per_sm_j));
    }
    int sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    g_pipe_per_sm[dev] = min_per_sm > 0 ? min_per_sm : 1;
    g_pipe_sms[dev] = sms;
    g_pipe_ready[dev] = true;
    return cudaSuccess;
}

int push32_blocks_per_sm(int dev) {
    if (dev < 0 || dev >= kMaxDevices) return 1;
    std::lock_guard<std::mutex> lock(g_pipe_mu);
    return g_pipe_per_sm[dev] > 0 ? g_pipe_per_sm[dev] : 1;
}

namespace {
// Persistent grid of the pipelined push on the current device: shp.per_sm
// blocks per SM (at most the resident count), no more than the tiles.
// Without init_push32 on this device the launch fails (no shared-memory
// opt-in) and the caller reports it.
int pipe_grid(const PushShape& shp, int64_t tiles) {
    int dev = 0;
    cudaGetDevice(&dev);
    int per_sm = 1, sms = 1;
    if (dev >= 0 && dev < kMaxDevices && g_pipe_sms[dev] > 0) {
        per_sm = std::max(1, std::min(shp.per_sm, g_pipe_per_sm[dev]));
        sms = g_pipe_sms[dev];
    }
    return (int)std::min<int64_t>((int64_t)per_sm * sms, tiles);
}

// the device-side limits of a shape (item a power of two from 32 to a
// tile, item mode only where the cells' coefficients fit the stage)
PushShape clamp_shape(PushShape s) {
    int item = 32;
    while (item * 2 <= std::min(kTileSlots, s.item)) item *= 2;
    s.item = item;
    s.item_cells = std::max(0, std::min(kItemMaxCells, s.item_cells));
    return s;
}
}  // namespace

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
    // the one-sub-cycle constants, rounded as the kernel's general path
    // rounds them for ns = 1 (dts = dt): qom * 0.5f * dt and dt * inv_w
    pc.k1 = pc.qom * 0.5f * pc.dt;
    for (int a = 0; a < 3; ++a) pc.a1[a] = pc.dt * pc.inv_w[a];
    return pc;
}

// the FP32 step: the pipelined persistent push (push32_pipe.cuh), the
// instance of the step's policies, one launch for all populations of S
template <>
int launch_push<float>(const Geom& g, const PopSet<float>& S, int mode, const PushShape& shp, cudaStream_t st) {
    if (mode != 0 && !g.deposit) return 0;  // nothing to deposit
    PipeFn fn = pipe_kernel(pipe_policy(g, mode));
    if (!fn || S.n <= 0) return 0;
    TileMap tm{};
    tm.n = S.n;
    Push32Set pcs{};
    for (int i = 0; i < S.n; ++i) {
        tm.first[i + 1] = tm.first[i] + (int)((S.p[i].capacity + kTileSlots - 1) / kTileSlots);
        pcs.c[i] = push32_const(g, S.p[i]);
    }
    const int tiles = tm.first[S.n];
    if (tiles <= 0) return 0;
    fn<<<pipe_grid(shp, tiles), kPipeThreads, pipe_smem_bytes<kPipeStages>(), st>>>(g, S, pcs, tm,
                                                                                    clamp_shape(shp));
    return 1;
}

template <>
int launch_push_pending<float>(const Geom& g, const PopSet<float>& S, cudaStream_t st) {
    if (S.n <= 0) return 0;
    Push32Set pcs{};
    for (int i = 0; i < S.n; ++i) pcs.c[i] = push32_const(g, S.p[i]);
    k_push_pending32<<<dim3(152, S.n), 128, 0, st>>>(g, S, pcs);
    return 1;
}

int launch_cell_coef(const Geom& g, float* coef, cudaStream_t st) {
    const float scale = (g.flags & 2u) ? (float)(1.0 / g.vol) : 1.0f;
    if (g.node32) {
        const int64_t n = (int64_t)g.sx * g.sy * g.sz;
        int64_t blocks = (n + 127) / 128;
        if (blocks > 152 * 16) blocks = 152 * 16;
        k_cell_coef32<<<(unsigned)blocks, 128, 0, st>>>(g.node32, g.sx, g.sy, g.sz, scale, coef);
        return 1;
    }
    const int64_t n = (int64_t)g.sx * g.sy * g.sz * 6;
    int64_t blocks = (n + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_cell_coef<<<(unsigned)blocks, 128, 0, st>>>(g.field, g.sx, g.sy, g.sz, (g.flags & 2u) ? 1.0 / g.vol : 1.0, coef);
    return 1;
}

// the batched FP32 step: the pipelined push over every job's tiles
template <>
int launch_push_batch<float>(const PopJob<float>* jobs, const int2* cta_job, int64_t nctas, int mode,
                             const Geom& g0, const PushShape& shp, cudaStream_t st) {
    if (nctas <= 0) return 0;
    if (mode != 0 && !g0.deposit) return 0;
    PipeJobsFn fn = pipe_jobs_kernel(pipe_policy(g0, mode));
    if (!fn) return 0;
    fn<<<pipe_grid(shp, nctas), kPipeThreads, pipe_smem_bytes<kPipeStages>(), st>>>(jobs, cta_job, (int)nctas,
                                                                                    clamp_shape(shp));
    return 1;
}

template <>
int launch_push_pending_batch<float>(const PopJob<float>* jobs, int njobs, cudaStream_t st) {
    k_push_pending32_batch<<<dim3(2, njobs), 128, 0, st>>>(jobs);
    return 1;
}

int launch_cell_coef_batch(const InstJob* inst, int ninst, int64_t max_cells, cudaStream_t st) {
    int64_t blocks = (max_cells * 6 + 127) / 128;
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
template int launch_place<float>(const Geom&, const PopSet<float>&, cudaStream_t);
template int launch_pending_rotate<float>(const PopSet<float>&, uint64_t*, cudaStream_t);
template int launch_relayout<float>(const Pop<float>&, const Pop<float>&, int, int32_t*, cudaStream_t);
template int launch_pending_count<float>(const Pop<float>&, int32_t*, cudaStream_t);
}  // namespace ipg
