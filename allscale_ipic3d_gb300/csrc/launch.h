// Host-side launchers of the GB300 particle path's kernels. Each returns the
// number of kernels it enqueued (the context counts its launches).
#pragma once

#include <cuda_runtime.h>

#include "device.cuh"

namespace ipg {

// particles (particles_fp64.cu / particles_fp32.cu)
template <typename T>
int launch_push(const Geom& g, const Pop<T>& P, int mode, cudaStream_t st);
template <typename T>
int launch_push_pending(const Geom& g, const Pop<T>& P, cudaStream_t st);
template <typename T>
int launch_inject(const Geom& g, const Pop<T>& P, double per_cell, const double drift[3], const double vth[3],
                  uint64_t seed, const uint64_t* d_step, cudaStream_t st);
template <typename T>
int launch_place(const Geom& g, const Pop<T>& P, int32_t* sort_tmp, cudaStream_t st);
template <typename T>
int launch_pending_rotate(const Pop<T>& P, uint32_t* pending_in_count, cudaStream_t st);
template <typename T>
int launch_relayout(const Pop<T>& from, const Pop<T>& to, int ncells, int32_t* pend_per_cell_scratch,
                    cudaStream_t st);
template <typename T>
int launch_pending_count(const Pop<T>& P, int32_t* per_cell, cudaStream_t st);

// fields (fields.cu)
int launch_ghost(const Geom& g, cudaStream_t st);
int launch_leapfrog(const Geom& g, bool refresh_node_b, cudaStream_t st);
int launch_forward(const Geom& g, cudaStream_t st);
int launch_j_finalize(const Geom& g, bool div8, cudaStream_t st);
int launch_node32(const Geom& g, float4* node32, cudaStream_t st);
int launch_cell_coef(const Geom& g, float* coef, cudaStream_t st);  // particles_fp32.cu
int reduce_blocks();
template <typename T>
int launch_reduce_particles(const Pop<T>& P, int ncells, double* partial, cudaStream_t st);
int launch_reduce_fields(const Geom& g, double* partial, cudaStream_t st);
int launch_reduce_final(const double* partial, int blocks, int kq, double* out, cudaStream_t st);

// misc (ipic3d_gpu.cu)
// records a status and message for ipic3d_gpu_last_error (this thread)
int set_last_error(int status, const char* msg);
int launch_boris(const void* parts, uint64_t n, const double E[3], const double B[3], double dt, uint64_t nsteps,
                 int push_position, void* out, cudaStream_t st);

}  // namespace ipg
