// Launchers of the particle kernels for one storage type; included once per
// type by particles_fp64.cu and particles_fp32.cu.
#pragma once

#include "launch.h"
#include "particle_kernels.cuh"

namespace ipg {

// generic versions (the FP64 path); particles_fp32.cu specialises both
template <typename T>
int launch_push_generic(const Geom& g, const PopSet<T>& S, int mode, cudaStream_t st) {
    int n = 0;
    for (int i = 0; i < S.n; ++i) {
        const Pop<T>& P = S.p[i];
        if (P.capacity <= 0) continue;
        const int64_t blocks = (P.capacity + kSlotsPerCta - 1) / kSlotsPerCta;
        k_push<T><<<(unsigned)blocks, kPushThreads, 0, st>>>(g, P, mode);
        ++n;
    }
    return n;
}

template <typename T>
int launch_push_pending_generic(const Geom& g, const PopSet<T>& S, cudaStream_t st) {
    if (S.n <= 0) return 0;
    k_push_pending<T><<<dim3(152, S.n), 128, 0, st>>>(g, S);
    return 1;
}

template <typename T>
int launch_inject(const Geom& g, const Pop<T>& P, double per_cell, const double drift[3], const double vth[3],
                  uint64_t seed, const uint64_t* d_step, cudaStream_t st) {
    InjectParams ip;
    ip.per_cell = per_cell;
    for (int a = 0; a < 3; ++a) {
        ip.drift[a] = drift[a];
        ip.vth[a] = vth[a];
    }
    ip.seed = seed;
    ip.step = d_step;
    const int faces = g.sy * g.sz;
    k_inject<T><<<(faces + 127) / 128, 128, 0, st>>>(g, P, ip);
    return 1;
}

template <typename T>
int launch_place(const Geom& g, const PopSet<T>& S, cudaStream_t st) {
    if (S.n <= 0) return 0;
    // the flagged cells onto the dirty lists (a thread per cell)
    int64_t cb = ((int64_t)g.ncells + 255) / 256;
    if (cb > 152 * 8) cb = 152 * 8;
    k_dirty_compact<T><<<dim3((unsigned)cb, S.n), 256, 0, st>>>(g.ncells, S);
    // a group of kPlaceLanes lanes per dirty cell
    int64_t blocks = ((int64_t)g.ncells + 7) / 8;
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_place<T><<<dim3((unsigned)blocks, S.n), 256, 0, st>>>(g, S);
    return 2;
}

template <typename T>
int launch_pending_rotate(const PopSet<T>& S, uint64_t* step, cudaStream_t st) {
    if (S.n <= 0) return 0;
    k_pending_rotate<T><<<dim3(152, S.n), 256, 0, st>>>(S, step);
    return 1;
}

template <typename T>
int launch_relayout(const Pop<T>& from, const Pop<T>& to, int ncells, int32_t* pend_per_cell_scratch,
                    cudaStream_t st) {
    (void)pend_per_cell_scratch;
    const int64_t threads = (int64_t)ncells * 32;
    k_relayout_copy<T><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(from, to, ncells);
    k_pending_place<T><<<152, 256, 0, st>>>(from.pending_in, from.pending_in_count, to);
    return 2;
}

template <typename T>
int launch_pending_count(const Pop<T>& P, int32_t* per_cell, cudaStream_t st) {
    k_pending_count<T><<<152, 256, 0, st>>>(P.pending_in, P.pending_in_count, per_cell);
    return 1;
}

// ---- batched ensemble ------------------------------------------------------
// cta_job[b] = (job, CTA of the job) for the push, blk_job[b] = (job, first
// cell) for the placement (8 cells of one job per 256-thread block).
template <typename T>
__global__ void __launch_bounds__(kPushThreads) k_push_batch(const PopJob<T>* __restrict__ jobs,
                                                             const int2* __restrict__ cta_job, int mode) {
    __shared__ PopJob<T> job;
    const int2 cj = __ldg(cta_job + blockIdx.x);
    load_job(job, jobs + cj.x);
    push_body<T>(job.g, job.P, cj.y, mode);
}

template <typename T>
__global__ void k_push_pending_batch(const PopJob<T>* __restrict__ jobs) {
    const PopJob<T>& J = jobs[blockIdx.y];
    push_pending_body<T>(J.g, J.P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Placement of a batch: blockIdx.y = job, the job's warps stride over its
// dirty-cell list (cells with holes or arrivals only).
// Batched dirty lists: block b lists the flagged cells of the 512-cell
// range tab[b].y of job tab[b].x.
template <typename T>
__global__ void k_dirty_compact_batch(const PopJob<T>* __restrict__ jobs, const int2* __restrict__ tab) {
    const int2 e = tab[blockIdx.x];
    const PopJob<T>& J = jobs[e.x];
    const int c0 = e.y * 512, c1 = c0 + 512 < J.g.ncells ? c0 + 512 : J.g.ncells;
    dirty_compact_body<T>(J.P, c0, c1, threadIdx.x, blockDim.x);
}

// Batched placement: block b is block tab[b].y of the place_blocks(ncells)
// blocks of job tab[b].x (its share grows with the universe), groups of
// kPlaceLanes lanes striding over the job's dirty list.
template <typename T>
__global__ void k_place_batch(const PopJob<T>* __restrict__ jobs, const int2* __restrict__ tab) {
    const int2 e = tab[blockIdx.x];
    const PopJob<T>& J = jobs[e.x];
    const uint32_t n = J.P.ctr->dirty;
    const uint32_t g0 = ((uint32_t)e.y * blockDim.x + threadIdx.x) / kPlaceLanes,
                   ng = ((uint32_t)place_blocks(J.g.ncells) * blockDim.x) / kPlaceLanes;
    for (uint32_t i = g0; i < n; i += ng) place_body<T>(J.g, J.P, J.sort_tmp, J.P.dirty_list[i]);
}

template <typename T>
__global__ void k_pending_rotate_batch(const PopJob<T>* __restrict__ jobs) {
    const PopJob<T>& J = jobs[blockIdx.y];
    pending_rotate_body<T>(J.P, J.pend_count, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Start of a batched step: blockIdx.y < ninst clears universe y's J and rho
// (when depositing), blockIdx.y == ninst the step counters of every job and
// the re-layout flag.
template <typename T>
__global__ void k_batch_begin(const PopJob<T>* __restrict__ jobs, int njobs, const InstJob* __restrict__ inst,
                              int ninst, int deposit, uint32_t* flagged) {
    const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    if ((int)blockIdx.y == ninst) {
        for (int64_t j = t0; j < njobs; j += stride) {
            StepCounters* c = jobs[j].P.ctr;
            c->outbox = 0; c->pending_out = 0; c->deferred = 0;
            c->removed = 0; c->migrated = 0; c->injected = 0; c->dirty = 0;
        }
        if (t0 == 0) *flagged = 0;
        return;
    }
    if (!deposit) return;
    const Geom& g = inst[blockIdx.y].g;
    const int64_t nn = (int64_t)(g.sx + 1) * (g.sy + 1) * (g.sz + 1);
    for (int64_t t = t0; t < 4 * nn; t += stride) {
        if (t < 3 * nn) g.J[t] = 0.0;
        else g.rho[t - 3 * nn] = 0.0;
    }
}

// End of a batched step: every universe's step counter advances; universes
// whose waiting particles exceed their limit, or that lost particles, are
// counted in *flagged.
template <typename T>
__global__ void k_batch_end(const PopJob<T>* __restrict__ jobs, const InstJob* __restrict__ inst, int ninst,
                            uint32_t* flagged) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    const InstJob& b = inst[i];
    *b.step += 1;
    uint32_t pend = 0, lost = 0;
    for (int j = b.job0; j < b.job0 + b.njobs; ++j) {
        pend += jobs[j].P.ctr->pending_out;
        lost += jobs[j].P.ctr->lost;
    }
    if (pend > b.pend_limit || lost) atomicAdd(flagged, 1u);
}

template <typename T>
__global__ void k_batch_status(const PopJob<T>* __restrict__ jobs, int njobs, JobStatus* out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs) return;
    JobStatus s;
    s.c = *jobs[j].P.ctr;
    s.pending_in = *jobs[j].pend_count;
    s.pad = 0;
    out[j] = s;
}

template <typename T>
int launch_push_batch_generic(const PopJob<T>* jobs, const int2* cta_job, int64_t nctas, int mode, cudaStream_t st) {
    if (nctas <= 0) return 0;
    k_push_batch<T><<<(unsigned)nctas, kPushThreads, 0, st>>>(jobs, cta_job, mode);
    return 1;
}

template <typename T>
int launch_push_pending_batch(const PopJob<T>* jobs, int njobs, cudaStream_t st);

template <typename T>
int launch_push_pending_batch_generic(const PopJob<T>* jobs, int njobs, cudaStream_t st) {
    k_push_pending_batch<T><<<dim3(2, njobs), 128, 0, st>>>(jobs);
    return 1;
}

template <typename T>
int launch_place_batch(const PopJob<T>* jobs, const int2* tab, int64_t nblocks, cudaStream_t st) {
    if (nblocks <= 0) return 0;
    k_dirty_compact_batch<T><<<(unsigned)nblocks, 256, 0, st>>>(jobs, tab);
    k_place_batch<T><<<(unsigned)nblocks, 256, 0, st>>>(jobs, tab);
    return 2;
}

template <typename T>
int launch_pending_rotate_batch(const PopJob<T>* jobs, int njobs, cudaStream_t st) {
    k_pending_rotate_batch<T><<<dim3(2, njobs), 256, 0, st>>>(jobs);
    return 1;
}

template <typename T>
int launch_batch_begin(const PopJob<T>* jobs, int njobs, const InstJob* inst, int ninst, int64_t max_nodes,
                       int deposit, uint32_t* flagged, cudaStream_t st) {
    int64_t gx = (4 * max_nodes + 255) / 256;
    if (gx < 1) gx = 1;
    if (gx > 64) gx = 64;
    k_batch_begin<T><<<dim3((unsigned)gx, ninst + 1), 256, 0, st>>>(jobs, njobs, inst, ninst, deposit, flagged);
    return 1;
}

template <typename T>
int launch_batch_end(const PopJob<T>* jobs, const InstJob* inst, int ninst, uint32_t* flagged, cudaStream_t st) {
    k_batch_end<T><<<(ninst + 127) / 128, 128, 0, st>>>(jobs, inst, ninst, flagged);
    return 1;
}

template <typename T>
int launch_batch_status(const PopJob<T>* jobs, int njobs, JobStatus* out, cudaStream_t st) {
    k_batch_status<T><<<(njobs + 127) / 128, 128, 0, st>>>(jobs, njobs, out);
    return 1;
}

}  // namespace ipg
