// Launchers of the particle kernels for one storage type; included once per
// type by particles_fp64.cu and particles_fp32.cu.
#pragma once

#include "launch.h"
#include "particle_kernels.cuh"

namespace ipg {

template <typename T>
int launch_push(const Geom& g, const Pop<T>& P, int mode, cudaStream_t st);
template <typename T>
int launch_push_pending(const Geom& g, const Pop<T>& P, cudaStream_t st);

// generic versions (the FP64 path); particles_fp32.cu specialises both
template <typename T>
int launch_push_generic(const Geom& g, const Pop<T>& P, int mode, cudaStream_t st) {
    if (P.capacity <= 0) return 0;
    const int64_t blocks = (P.capacity + kSlotsPerCta - 1) / kSlotsPerCta;
    k_push<T><<<(unsigned)blocks, kPushThreads, 0, st>>>(g, P, mode);
    return 1;
}

template <typename T>
int launch_push_pending_generic(const Geom& g, const Pop<T>& P, cudaStream_t st) {
    k_push_pending<T><<<152, 128, 0, st>>>(g, P);
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
int launch_place(const Geom& g, const Pop<T>& P, int32_t* sort_tmp, cudaStream_t st) {
    const int64_t threads = (int64_t)g.ncells * 32;
    k_place<T><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(g, P, sort_tmp);
    return 1;
}

template <typename T>
int launch_pending_rotate(const Pop<T>& P, uint32_t* pending_in_count, cudaStream_t st) {
    k_pending_rotate<T><<<152, 256, 0, st>>>(P, pending_in_count);
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

}  // namespace ipg
