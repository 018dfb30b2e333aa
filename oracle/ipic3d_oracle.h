/*
 * CPU oracle of the GB300 particle path: a plain C++/OpenMP restatement of
 * the AllScale iPIC3D reference's timestep (mover, export, import, current
 * projection, boundary copy, field solvers, conserved quantities).
 *
 * TEST INFRASTRUCTURE ONLY. The tests, the smoke check and bench.py's CPU
 * baseline call it as the checker / as the timed reference implementation;
 * nothing in the shipped library links or calls it.
 *
 * The API mirrors include/ipic3d_gpu.h so that one scenario can run through
 * both. Everything is FP64 with absolute positions (the reference's
 * representation, particle.h:9-60) whatever the config's precision is.
 */
#ifndef IPIC3D_ORACLE_H
#define IPIC3D_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/ipic3d_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_sim oracle_sim;

int oracle_create(const ipic3d_props* props, const ipic3d_config* cfg, oracle_sim** out);
void oracle_destroy(oracle_sim* s);
void oracle_set_threads(int n);
int oracle_upload_particles(oracle_sim* s, const ipic3d_particle* p, const uint64_t* counts, const uint32_t* ids);
int oracle_upload_fields(oracle_sim* s, const double* field, const double* bcfield, const double* density);
int oracle_download_fields(oracle_sim* s, double* field, double* bcfield, double* density, double* rho);
uint64_t oracle_particle_count(oracle_sim* s);
int oracle_download_particles(oracle_sim* s, ipic3d_particle* p, uint64_t cap, uint64_t* counts, uint32_t* ids);
int oracle_step(oracle_sim* s, uint64_t n);
int oracle_project(oracle_sim* s);
int oracle_update_boundaries(oracle_sim* s);
int oracle_solve_fields(oracle_sim* s);
int oracle_move(oracle_sim* s);
int oracle_conserved(oracle_sim* s, ipic3d_conserved* out);
/* stats of the last move: particles that changed cell, removed, injected */
int oracle_last_counts(oracle_sim* s, uint64_t* migrated, uint64_t* removed, uint64_t* injected);

/* the reference's particle initialisations (ipic3d_oracle_init.cpp) */
int oracle_init_uniform_pos_normal_speed(const ipic3d_props* props, uint64_t numParticles, const double low[3],
                                         const double hig[3], const double mean[3], const double stddev[3],
                                         ipic3d_particle* out, uint64_t* counts, uint64_t* n_out);
int oracle_init_uniform_bench(const ipic3d_props* props, uint64_t numParticles, ipic3d_particle* out,
                              uint64_t* counts);
void oracle_generate_uniform_pos_normal_speed(const double low[3], const double hig[3], const double mean[3],
                                              const double stddev[3], uint32_t seed, uint64_t n,
                                              ipic3d_particle* out);

/* the standalone tracer (ipic3d_oracle_tracer.cpp, pic_tracer.cxx) */
int oracle_tracer_config(int32_t R, ipic3d_props* out);
int oracle_tracer_particles(const ipic3d_props* props, uint64_t n, uint32_t seed, ipic3d_particle* out);
int oracle_trace(const ipic3d_props* props, const ipic3d_particle* particles, uint64_t n, int32_t steps,
                 int32_t frame_interval, int32_t num_frames, uint32_t* counts);

int oracle_boris(ipic3d_particle* p, uint64_t n, const double E[3], const double B[3], double dt, uint64_t nsteps,
                 int push_position);
double oracle_trilinear(const double corners[8], const double pos[3], double vol);
int oracle_aggregate_contributions(const ipic3d_props* props, const double* contrib, double* J);

#ifdef __cplusplus
}
#endif

#endif
