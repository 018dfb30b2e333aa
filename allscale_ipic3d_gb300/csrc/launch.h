// Host-side launchers of the GB300 particle path's kernels. Each returns the
// number of kernels it enqueued (the context counts its launches).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/ipic3d_types.h"
#include "device.cuh"

namespace ipg {

// particles (particles_fp64.cu / particles_fp32.cu); the PopSet launchers
// advance all populations of a set with one launch
// `shp`: launch shape of the FP32 push (the FP64 push has one shape)
template <typename T>
int launch_push(const Geom& g, const PopSet<T>& S, int mode, const PushShape& shp, cudaStream_t st);
template <typename T>
int launch_push_pending(const Geom& g, const PopSet<T>& S, cudaStream_t st);
template <typename T>
int launch_inject(const Geom& g, const Pop<T>& P, double per_cell, const double drift[3], const double vth[3],
                  uint64_t seed, const uint64_t* d_step, cudaStream_t st);
template <typename T>
int launch_place(const Geom& g, const PopSet<T>& S, cudaStream_t st);
// `step` (may be null): the device step counter, advanced by the launch
template <typename T>
int launch_pending_rotate(const PopSet<T>& S, uint64_t* step, cudaStream_t st);
template <typename T>
int launch_relayout(const Pop<T>& from, const Pop<T>& to, int ncells, int32_t* pend_per_cell_scratch,
                    cudaStream_t st);
template <typename T>
int launch_pending_count(const Pop<T>& P, int32_t* per_cell, cudaStream_t st);

// batched ensemble: job tables built by the host (particles_fp64/32.cu)
template <typename T>
int launch_push_batch(const PopJob<T>* jobs, const int2* cta_job, int64_t nctas, int mode, const Geom& g0,
                      const PushShape& shp, cudaStream_t st);  // g0: the policy fields (mover, flags, deposit) shared by the jobs
template <typename T>
int launch_push_pending_batch(const PopJob<T>* jobs, int njobs, cudaStream_t st);
// tab: nblocks entries (job, block of the job), place_blocks(ncells) blocks
// per job (device.cuh)
template <typename T>
int launch_place_batch(const PopJob<T>* jobs, const int2* tab, int64_t nblocks, cudaStream_t st);
template <typename T>
int launch_pending_rotate_batch(const PopJob<T>* jobs, int njobs, cudaStream_t st);
template <typename T>
int launch_batch_begin(const PopJob<T>* jobs, int njobs, const InstJob* inst, int ninst, int64_t max_nodes,
                       int deposit, uint32_t* flagged, cudaStream_t st);
template <typename T>
int launch_batch_end(const PopJob<T>* jobs, const InstJob* inst, int ninst, uint32_t* flagged, cudaStream_t st);
template <typename T>
int launch_batch_status(const PopJob<T>* jobs, int njobs, JobStatus* out, cudaStream_t st);
int launch_cell_coef_batch(const InstJob* inst, int ninst, int64_t max_cells, cudaStream_t st);  // particles_fp32.cu
Push32Const push32_const(const Geom& g, const Pop<float>& P);                                    // particles_fp32.cu
cudaError_t init_push32(int dev);  // once per device, before any capture (particles_fp32.cu)
int push32_blocks_per_sm(int dev);  // resident pipelined-push blocks per SM (after init_push32)
int launch_ghost_batch(const InstJob* jobs, int ninst, int max_s, cudaStream_t st);              // fields.cu
int launch_leapfrog_batch(const InstJob* jobs, int ninst, int max_s, bool refresh_node_b, cudaStream_t st);
int launch_forward_batch(const InstJob* jobs, int ninst, int max_s, cudaStream_t st);
int launch_j_finalize_batch(const InstJob* jobs, int ninst, int64_t max_cells, cudaStream_t st);

// fields (fields.cu)
int launch_ghost(const Geom& g, cudaStream_t st);
// raw_j: g.J holds the deposit's raw node sums (no J finalisation yet); the E
// update folds and normalises them on the read as launch_j_finalize(g, div8,
// exact) would. after_e (may be null) is recorded once the E update is done.
int launch_leapfrog(const Geom& g, bool refresh_node_b, bool exact, cudaStream_t st, bool raw_j = false,
                    bool div8 = false, cudaEvent_t after_e = nullptr);
int launch_forward(const Geom& g, cudaStream_t st, bool raw_j = false, bool div8 = false, bool exact = true,
                   cudaEvent_t after_e = nullptr);
// exact: the reference's divisions (FP64 parity); else one multiplication
int launch_j_finalize(const Geom& g, bool div8, bool exact, cudaStream_t st);
int launch_node32(const Geom& g, float4* node32, cudaStream_t st);
int launch_cell_coef(const Geom& g, float* coef, cudaStream_t st);  // particles_fp32.cu
int reduce_blocks();
template <typename T>
int launch_reduce_particles(const Pop<T>& P, int ncells, double* partial, cudaStream_t st);
int launch_reduce_fields(const Geom& g, double* partial, cudaStream_t st);
int launch_reduce_final(const double* partial, int blocks, int kq, double* out, cudaStream_t st);

// initCells(uniform) of the reference's :U:N mode into `out` (AoS records,
// grouped by cell), its random streams replayed on the device (init.cu)
int launch_init_uniform(int sx, int sy, int sz, const double origin[3], const double w[3], uint64_t num_particles,
                        void* out, cudaStream_t st);
// initCells<uniform_pos_normal_speed> (cell.h:492-636): phase 1 (per-cell
// counts) on the host, phase 2 (every particle) on the device into `out`
// (grouped by cell, cell c from record d_off[c]) (init.cu)
void init_normal_counts(const ipic3d_props& pr, uint64_t num_particles, const double low[3], const double hig[3],
                        std::vector<uint64_t>& counts);
int launch_init_normal(const ipic3d_props& pr, const double mean[3], const double stddev[3], double q, double qom,
                       const uint64_t* d_count, const int64_t* d_off, void* out, cudaStream_t st);

// misc (ipic3d_gpu.cu)
// records a status and message for ipic3d_gpu_last_error (this thread)
int set_last_error(int status, const char* msg);
int launch_boris(const void* parts, uint64_t n, const double E[3], const double B[3], double dt, uint64_t nsteps,
                 int push_position, void* out, cudaStream_t st);

}  // namespace ipg
