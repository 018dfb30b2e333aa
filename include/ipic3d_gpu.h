/*
 * ipic3d_gpu.h -- C ABI of the GB300 (sm_103a) particle hot path.
 *
 * Replaces the per-timestep loop of the AllScale iPIC3D reference,
 *   template<P,F,M> simulateSteps(numSteps, Universe&)
 *     code/app/include/ipic3d/app/simulator.h:42-47,127-242
 * with its policy functors (simulator.h:244-276):
 *   default_particle_mover      -> mover IPIC3D_MOVER_DIPOLE   (cell.h:896-964 + 975-1159)
 *   default_field_solver        -> solver IPIC3D_SOLVER_STATIC (field.h:272-289)
 *   leapfrog_field_solver       -> solver IPIC3D_SOLVER_LEAPFROG (field.h:342-402)
 *   forward_field_solver        -> solver IPIC3D_SOLVER_FORWARD (field.h:294-337)
 *   default_particle_to_field_projector -> projector IPIC3D_PROJECT_CIC (cell.h:787-824)
 * and the migration mailboxes TransferBuffers (transfer_buffer.h:48-95) with
 * importParticles (cell.h:1195-1310).
 *
 * One context = one Universe (universe.h:12-51) resident on one GPU:
 * particles structure-of-arrays, grouped by cell, FP64 absolute or FP32
 * cell-relative positions; fields FP64. All entry points are
 * single-host-thread and ordered on the context's CUDA stream. Every call
 * returns IPIC3D_OK (0) or a negative IPIC3D_E* status;
 * ipic3d_gpu_last_error() describes the last failure. (The reference aborts
 * through assert_* instead, e.g. cell.h:1309.)
 */
#ifndef IPIC3D_GPU_H
#define IPIC3D_GPU_H

#include <stddef.h>
#include <stdint.h>

#include "ipic3d_types.h"

#ifdef __cplusplus
extern "C" {
#endif

#define IPIC3D_GPU_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------- */
#define IPIC3D_OK 0
#define IPIC3D_E_INVALID -1     /* bad argument / configuration            */
#define IPIC3D_E_NOMEM -2       /* device or host allocation failed        */
#define IPIC3D_E_CUDA -3        /* a CUDA runtime call failed              */
#define IPIC3D_E_CAPACITY -4    /* particle storage full (grow and retry)  */
#define IPIC3D_E_NODEVICE -5    /* no usable sm_103 device                 */
#define IPIC3D_E_STATE -6       /* call out of order (e.g. no particles)   */
#define IPIC3D_E_TIMEOUT -7     /* a kernel gave up a bounded device wait  */

/* ---- step configuration (the simulateSteps template arguments) ---------- */
enum ipic3d_precision {
    IPIC3D_FP64 = 0, /* absolute FP64 positions, reference arithmetic order   */
    IPIC3D_FP32 = 1  /* FP32 cell-relative positions and velocities; FP64
                        node accumulation, field update and reductions        */
};

enum ipic3d_mover {
    /* moveParticles (cell.h:896-964): analytic Earth dipole at the origin,
       E = 0, adaptive sub-cycling (<= 100). The field grid is not read.      */
    IPIC3D_MOVER_DIPOLE = 0,
    /* field-gather mover of the commented code at cell.h:905-937: trilinear
       interpolation of node E and B (trilinearInterpolationF2P, cell.h:867),
       same sub-cycling rule; IPIC3D_F_DIPOLE_IN_GATHER adds the analytic
       dipole B.                                                              */
    IPIC3D_MOVER_FIELD = 1
};

enum ipic3d_solver {
    IPIC3D_SOLVER_STATIC = 0,   /* solveFieldStatically: no-op (field.h:272)  */
    IPIC3D_SOLVER_LEAPFROG = 1, /* solveFieldLeapfrog, E then Bc (field.h:342) */
    IPIC3D_SOLVER_FORWARD = 2   /* solveFieldForward, E, Bc, node B (field.h:294) */
};

enum ipic3d_projector {
    IPIC3D_PROJECT_NONE = 0, /* the reference's active loop (simulator.h:189) */
    IPIC3D_PROJECT_CIC = 1   /* cloud-in-cell J (cell.h:787-824) and rho     */
};

/* particle boundary of one domain face */
enum ipic3d_boundary {
    IPIC3D_BC_REFLECT = 0,  /* exportParticles' wall rule (cell.h:1102-1121):
                               shift by half a cell width, negate velocity   */
    IPIC3D_BC_PERIODIC = 1, /* wrap around (both faces of the axis)          */
    IPIC3D_BC_OPEN = 2      /* outflow: the particle is removed             */
};

/* flags */
#define IPIC3D_F_J_DIV8 (1u << 0)          /* J = Js/vol/8 as cell.h:823 (else Js/vol) */
#define IPIC3D_F_GATHER_DIV_VOL (1u << 1)  /* trilinear result / vol as cell.h:884     */
#define IPIC3D_F_DIPOLE_IN_GATHER (1u << 2)/* FIELD mover adds the analytic dipole B   */
#define IPIC3D_F_REFRESH_NODE_B (1u << 3)  /* after LEAPFROG, node B = interpC2N(Bc)   */
#define IPIC3D_F_TRACK_IDS (1u << 4)       /* keep a 32-bit id per particle            */
#define IPIC3D_F_INJECT_LOW_X (1u << 5)    /* inject a drifting Maxwellian at -x face  */
#define IPIC3D_F_USE_GRAPH (1u << 6)       /* run multi-step calls as a CUDA graph     */

typedef struct ipic3d_config {
    int32_t precision;      /* enum ipic3d_precision */
    int32_t mover;          /* enum ipic3d_mover     */
    int32_t solver;         /* enum ipic3d_solver    */
    int32_t projector;      /* enum ipic3d_projector */
    int32_t bc_low[3];      /* enum ipic3d_boundary, faces x=0, y=0, z=0   */
    int32_t bc_high[3];     /* enum ipic3d_boundary, faces x=L, y=L, z=L   */
    uint32_t flags;         /* IPIC3D_F_*                                  */
    /* storage: per-cell slack (fraction of the particles uploaded into the
       cell, plus `slack_min` slots) reserved for arrivals; 0 = defaults.     */
    double slack;
    int32_t slack_min;
    int32_t block_size;     /* 0 = autotuned FP32 push shape, else the
                               default shape (ipic3d_push_shape)           */
    /* injection at the x=0 face (IPIC3D_F_INJECT_LOW_X, bc_low[0] OPEN):
       expected particles per face cell per step, their q, qom, drift and
       thermal velocities, and the seed of the counter-based generator.      */
    double inject_per_cell;
    double inject_q, inject_qom;
    double inject_drift[3];
    double inject_vth[3];
    uint64_t seed;
    uint64_t reserved[8];
} ipic3d_config;

/* Fills a config with the reference's defaults: FP64, dipole mover, static
 * solver, no projection, reflecting walls, no flags (simulator.h:42-47). */
void ipic3d_gpu_config_default(ipic3d_config* cfg);

typedef struct ipic3d_ctx ipic3d_ctx;

/* ---- lifetime ------------------------------------------------------------ */
/* Creates a context on the current CUDA device with the Universe's properties
 * (Universe(properties), universe.h:36). Fields start at zero. */
int ipic3d_gpu_create(const ipic3d_props* props, const ipic3d_config* cfg, ipic3d_ctx** out);
int ipic3d_gpu_destroy(ipic3d_ctx* ctx);

/* ---- state transfer (host memory) --------------------------------------- */
/* Uploads the particles of Universe::cells (cell.h:31-38): n particles
 * grouped by cell in row-major cell order, cell_counts[ncells] of them per
 * cell. ids may be NULL (then ids are the input indices when tracking).
 * Replaces all particles. Capacity = n plus the configured slack. */
int ipic3d_gpu_upload_particles(ipic3d_ctx* ctx, const ipic3d_particle* particles, const uint64_t* cell_counts,
                                const uint32_t* ids);
/* Reserves room for at least `n` particles (allocation happens here, not in
 * ipic3d_gpu_step). */
int ipic3d_gpu_reserve(ipic3d_ctx* ctx, uint64_t n);
/* initCells(properties, num_particles, uniform<>) (cell.h:638-697), the
 * universe of the reference's ":U:N" benchmark mode, made on the device:
 * floor(N / cells) particles per cell (+1 for the first N mod cells cells),
 * positions uniform in the cell and velocities U(-0.2, 0.2) per component
 * from the reference's per-cell std::minstd_rand streams (bit-identical
 * values), electrons (q = -1, q/m = -25). Replaces the context's particles
 * as an upload does (ids = index in cell order). */
int ipic3d_gpu_init_uniform(ipic3d_ctx* ctx, uint64_t num_particles);
/* initCells(properties, num_particles, uniform_pos_normal_speed<>(low, hig,
 * mean, stddev)) (cell.h:492-636), the .inp driver's universe
 * (src/ipic3d.cxx:69-82, createUniverseFromDistribution universe.h:84-103):
 * the per-cell counts from 100 pseudo-particles per cell of the position
 * stream (phase 1, cell.h:505-590, on the host), then every cell's particles
 * from its reseeded streams (phase 2, cell.h:596-632, on the device):
 * positions uniform in the cell, velocities mean + stddev * a ziggurat
 * normal variate per component, q = e, q/m = e / m_p. Bit-identical to the
 * reference's particles. Replaces the context's particles as an upload does
 * (ids = index in cell order). low / hig: the distribution's position box,
 * which must meet the universe; mean / stddev: the velocity distribution. */
int ipic3d_gpu_init_uniform_pos_normal_speed(ipic3d_ctx* ctx, uint64_t num_particles, const double low[3],
                                             const double hig[3], const double mean[3], const double stddev[3]);
/* Number of particles currently stored. */
int ipic3d_gpu_particle_count(ipic3d_ctx* ctx, uint64_t* n);
/* Downloads particles grouped by cell (row-major) with per-cell counts; the
 * order inside a cell is unspecified. `capacity` = entries in particles/ids;
 * cell_counts and ids may be NULL. */
int ipic3d_gpu_download_particles(ipic3d_ctx* ctx, ipic3d_particle* particles, uint64_t capacity,
                                  uint64_t* cell_counts, uint32_t* ids);
/* No counterpart in the reference. ipic3d_gpu_download_particles in two
 * halves, so that a caller that moves the whole state every step can
 * overlap this step's device-to-host copies with the next upload's
 * host-to-device copies (the host link is full duplex): this call fills
 * cell_counts, packs the records on the device and enqueues their copies,
 * then returns; the particles / ids buffers are complete only after
 * ipic3d_gpu_download_wait. Until then they must stay allocated and unread.
 * Other calls may run meanwhile (an upload, a step); the next download (of
 * either kind) and ipic3d_gpu_destroy wait for this one first. */
int ipic3d_gpu_download_particles_async(ipic3d_ctx* ctx, ipic3d_particle* particles, uint64_t capacity,
                                        uint64_t* cell_counts, uint32_t* ids);
/* Waits for the copies of an asynchronous download and completes its
 * buffers (returns at once when none is in flight). */
int ipic3d_gpu_download_wait(ipic3d_ctx* ctx);
/* The positions of every particle (3 doubles each, x y z), in the order of
 * ipic3d_gpu_download_particles (grouped by cell): what
 * outputParticlePositions (cell.h:1400-1429) writes. Packed on the device,
 * so only these 24 bytes per particle cross the host link. capacity is in
 * particles; cell_counts (may be NULL) receives the per-cell counts.
 * xyz == NULL returns the counts only. */
int ipic3d_gpu_download_positions(ipic3d_ctx* ctx, double* xyz, uint64_t capacity, uint64_t* cell_counts);
/* Per-cell particle counts (outputNumberOfParticlesPerCell, cell.h:1360). */
int ipic3d_gpu_cell_counts(ipic3d_ctx* ctx, uint64_t* cell_counts);

/* Field grids in the reference layout (ipic3d_types.h); any pointer may be
 * NULL to skip that grid. rho is (size+1)^3 doubles (download only).
 * With the CIC projector the deposit is fused into the push, so after
 * ipic3d_gpu_step J and rho hold the projection of the current particles --
 * what the reference's projector computes at the start of the next step
 * (simulator.h:189-194) -- rather than the projection made at the start of
 * the last step. */
int ipic3d_gpu_upload_fields(ipic3d_ctx* ctx, const double* field, const double* bcfield, const double* density);
int ipic3d_gpu_download_fields(ipic3d_ctx* ctx, double* field, double* bcfield, double* density, double* rho);

/* ---- the timestep ------------------------------------------------------- */
/* simulateSteps(numSteps, universe) (simulator.h:127-242) with the policies
 * of the context's config: per step
 *   projector (J, rho) -> updateFieldsOnBoundaries -> field solver
 *   -> mover + export -> import (-> injection)
 * Asynchronous: returns once the work is enqueued. */
int ipic3d_gpu_step(ipic3d_ctx* ctx, uint64_t num_steps);
/* Single phases, for the reference's per-function tests:
 * projectToDensityField over all nodes (cell.h:787-824) into J (and rho). */
int ipic3d_gpu_project(ipic3d_ctx* ctx);
/* updateFieldsOnBoundaries (field.h:407-440). */
int ipic3d_gpu_update_boundaries(ipic3d_ctx* ctx);
/* the configured field solver over [1, size+2)^3 (simulator.h:207-209). */
int ipic3d_gpu_solve_fields(ipic3d_ctx* ctx);
/* mover + export + import for every cell (simulator.h:214-223). */
int ipic3d_gpu_move(ipic3d_ctx* ctx);

/* Conserved quantities (simulator.h:76-83) computed on the device with
 * compensated FP64 sums. Synchronous. */
int ipic3d_gpu_conserved(ipic3d_ctx* ctx, ipic3d_conserved* out);
/* Waits for all work on the context's stream. */
int ipic3d_gpu_synchronize(ipic3d_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t) for callers that order their
 * own work after the step. */
void* ipic3d_gpu_stream(ipic3d_ctx* ctx);

/* ---- counters ------------------------------------------------------------ */
typedef struct ipic3d_stats {
    uint64_t steps;             /* steps executed                          */
    uint64_t particles;         /* particles stored                        */
    uint64_t capacity;          /* particle slots allocated                */
    uint64_t migrated_last;     /* particles that changed cell, last step  */
    uint64_t removed_last;      /* particles removed (planet/outflow)      */
    uint64_t injected_last;     /* particles injected, last step           */
    uint64_t rebuilds;          /* storage re-layouts (overflow of a cell) */
    uint64_t kernel_launches;   /* kernels launched by this context        */
    uint64_t pending_last;      /* particles waiting for a slot, last step */
    uint64_t relayout_steps;    /* steps after which a re-layout ran       */
} ipic3d_stats;
int ipic3d_gpu_stats(ipic3d_ctx* ctx, ipic3d_stats* out);

/* ---- per-phase timing (CUDA events on the context's stream) ------------- */
enum ipic3d_phase {
    IPIC3D_PHASE_PUSH = 0,     /* fused mover + export + deposit kernel      */
    IPIC3D_PHASE_PENDING = 1,  /* push of particles that waited for a slot   */
    IPIC3D_PHASE_INJECT = 2,   /* x = 0 injection                            */
    IPIC3D_PHASE_PLACE = 3,    /* import: holes / arrivals / compaction      */
    IPIC3D_PHASE_FIELDS = 4,   /* ghost faces + field solver (+ FP32 copy)   */
    IPIC3D_PHASE_MOMENTS = 5,  /* J, rho clear + periodic fold + normalise   */
    IPIC3D_PHASE_COUNT = 8
};
typedef struct ipic3d_profile {
    double ms[IPIC3D_PHASE_COUNT];         /* summed device time per phase     */
    uint64_t launches[IPIC3D_PHASE_COUNT]; /* timed intervals per phase        */
    uint64_t particles[IPIC3D_PHASE_COUNT];/* particles processed (push phase) */
} ipic3d_profile;
/* enable != 0: later steps run without a CUDA graph and every phase is
 * bracketed by CUDA events (adds a synchronisation per step). */
int ipic3d_gpu_profile(ipic3d_ctx* ctx, int enable);
/* Copies the accumulated times; reset != 0 clears them afterwards. */
int ipic3d_gpu_profile_read(ipic3d_ctx* ctx, ipic3d_profile* out, int reset);

/* ---- launch shape of the FP32 push (autotuned) ---------------------------- */
/* No counterpart in the reference (its cell loop is a pfor over the grid,
 * simulator.h:127-242). The FP32 push walks 1024-slot tiles of the
 * cell-sorted particles: a tile of at most `item_cells` cells is cut into
 * work items of `item` particles that warps claim one at a time, a sparser
 * tile is pushed slot by slot, and `blocks_per_sm` persistent blocks run on
 * each SM. With block_size 0 in the config, the first steps of a workload
 * (after an upload with a particle count not seen before, within a factor
 * of two) are trials of candidate shapes, outside the step graph and each
 * an ordinary step; the fastest is kept and cached for later contexts of
 * the same workload. FP64 contexts have one shape and report it untuned. */
typedef struct ipic3d_push_shape {
    int32_t item;           /* particles per work item, power of two, 32..1024    */
    int32_t item_cells;     /* item mode for tiles of at most this many cells, 0..32 */
    int32_t blocks_per_sm;  /* persistent thread blocks per SM, >= 1              */
    int32_t tuned;          /* out: 1 = chosen by the autotuner (or its cache)    */
    int32_t tuning;         /* out: 1 = trial steps are still to run              */
    int32_t trials;         /* out: timed trial steps of the last tuning pass     */
    double push_ms;         /* out: push time per step under the shape (tuned)    */
} ipic3d_push_shape;
int ipic3d_gpu_get_push_shape(ipic3d_ctx* ctx, ipic3d_push_shape* out);
/* shape != NULL fixes the shape (no autotuning; out-of-range fields are
 * clamped at launch); shape == NULL restarts the autotuner: the next steps
 * are its trials. */
int ipic3d_gpu_set_push_shape(ipic3d_ctx* ctx, const ipic3d_push_shape* shape);
/* No counterpart in the reference (its runtime has no device waits). The
 * FP32 push's warps wait on their own thread block's shared-memory barriers
 * (bulk-copy completion, stage release); each wait gives up after a bounded
 * number of polls of about 20 us, the thread block then records a timeout,
 * lets its copies in flight land (always with the default bound) and
 * returns, and the step returns IPIC3D_E_TIMEOUT. polls < 0 restores the
 * default bound (about 1 s); polls >= 0 sets it (0: every wait gives up
 * before its first poll -- the way a test makes the bound run out). Takes
 * effect from the next step (captured step graphs are dropped). */
int ipic3d_gpu_set_wait_limit(ipic3d_ctx* ctx, int64_t polls);

/* ---- element kernels (the reference's unit-level functions) ------------- */
/* Particle::updateVelocity + updatePosition (particle.h:24-49) applied
 * nsteps times to n host particles with uniform E, B: the Boris KATs
 * (particle_test.cc:45-81, simulation_test.cc:237-246). push_position = 0
 * applies only updateVelocity. */
int ipic3d_gpu_boris(ipic3d_particle* particles, uint64_t n, const double E[3], const double B[3], double dt,
                     uint64_t nsteps, int push_position);

/* ---- batched ensemble ----------------------------------------------------- */
/* No counterpart in the reference, which runs one Universe per process
 * (ipic3d.cxx:94, simulator.h:127-242). A batch holds `count` independent
 * universes of possibly different sizes and advances all of them with one
 * launch per kernel of the timestep: every kernel reads a device table of
 * (universe, species) jobs, so a step costs the same dozen launches for 1
 * or 10,000 universes (count <= 65535, species per universe <= 16).
 *
 * props[i] describes universe i; `cfg` is shared by all of them (precision,
 * mover, solver, projector, boundaries, flags; IPIC3D_F_INJECT_LOW_X is not
 * supported in a batch). IPIC3D_F_USE_GRAPH captures one batched step as a
 * CUDA graph. Each universe is an ordinary context owned by the batch, on
 * the batch's stream: ipic3d_gpu_batch_universe() lends it out for uploads,
 * downloads, conserved quantities and counters (ipic3d_gpu_destroy refuses
 * a lent context with IPIC3D_E_STATE). */
typedef struct ipic3d_batch ipic3d_batch;
int ipic3d_gpu_batch_create(uint32_t count, const ipic3d_props* props, const ipic3d_config* cfg,
                            ipic3d_batch** out);
int ipic3d_gpu_batch_destroy(ipic3d_batch* batch);
int ipic3d_gpu_batch_size(ipic3d_batch* batch, uint32_t* count);
int ipic3d_gpu_batch_universe(ipic3d_batch* batch, uint32_t index, ipic3d_ctx** out);
/* num_steps timesteps of every universe; the same sequence as
 * ipic3d_gpu_step per universe, with its counters and re-layouts. */
int ipic3d_gpu_batch_step(ipic3d_batch* batch, uint64_t num_steps);
int ipic3d_gpu_batch_synchronize(ipic3d_batch* batch);
void* ipic3d_gpu_batch_stream(ipic3d_batch* batch);
/* Sums over the universes (steps = batched steps taken, kernel_launches =
 * the batch's own launches). */
int ipic3d_gpu_batch_stats(ipic3d_batch* batch, ipic3d_stats* out);
/* The batched push's shape: autotuned over the batch's first steps (config
 * block_size 0), as a context's. */
int ipic3d_gpu_batch_get_push_shape(ipic3d_batch* batch, ipic3d_push_shape* out);

/* ---- projection without allocation -------------------------------------- */
/* No counterpart in the reference. The same projection as
 * ipic3d_gpu_project, for callers that cannot allocate device memory: hosts
 * that hand out every byte of device memory from their own pool, or loops
 * where a cudaMalloc would synchronise the device. Nothing here allocates:
 * the caller passes device pointers to the particles (grouped by cell,
 * d_cell_offsets[c] .. d_cell_offsets[c+1] for cell c, ncells + 1 entries),
 * J ((size+1)^3 x 3 doubles) and rho ((size+1)^3 doubles, may be NULL); the
 * FP64 node sums in between live in one fixed device array of the library,
 * sized for grids of at most (32+1)^3 nodes (larger grids return
 * IPIC3D_E_CAPACITY before any work is enqueued). The first call in each
 * CUDA context (and the first after a cudaDeviceReset) looks up that array's
 * device address, so make it once before any stream capture. Every call
 * shares the array: calls that overlap on the GPU (other streams, other host
 * threads) race. flags: IPIC3D_F_J_DIV8. Work is enqueued on `stream` (a
 * cudaStream_t, NULL = default stream). */
int ipic3d_gpu_project_noalloc(const ipic3d_props* props, uint32_t flags, const ipic3d_particle* d_particles,
                               const uint64_t* d_cell_offsets, double* d_J, double* d_rho, void* stream);

/* ---- density contributions ---------------------------------------------- */
/* aggregateDensityContributions (cell.h:835-855) at every node of the
 * (size+1)^3 current-density grid: J(pos) += the contributions at 2 pos +
 * {-1, 0}^3 that lie inside the (2 size)^3 contribution grid (the buffer of
 * simulator.h:156, 3 doubles per entry, row-major), then J /= vol, J /= 8.
 * J is read and written in place (3 doubles per node), as the reference adds
 * into the node's current J. Device pointers; the work is enqueued on
 * `stream` (a cudaStream_t, NULL = default stream) without synchronising.
 * The reference allocates the contribution grid but no phase of its loop
 * fills it; this is the aggregation step for callers that do. */
int ipic3d_gpu_aggregate_contributions(const ipic3d_props* props, const double* d_contributions, double* d_J,
                                       void* stream);

/* ---- the standalone particle tracer (pic_tracer.cxx) -------------------- */
/* traceParticle (pic_tracer.cxx:77-148) for n independent particles, the
 * loop body of pic_tracer's map operator (pic_tracer.cxx:242-249). Each
 * particle is shifted by objectCenter, skipped if it starts inside the
 * planet (r^2 < planetRadius^2) or outside the universe box [origin,
 * origin + cellWidth * size], then moved `steps` times (pic_tracer's main
 * passes T + 1) through the analytic dipole B = -Bext.z R^3 / r^5 (3xz, 3yz,
 * 2z^2 - x^2 - y^2), E = 0, with the adaptive sub-cycling and Boris rotation
 * of the reference, wrapped periodically, and stopped once r^2 <=
 * planetRadius^2. On every step t with t % frame_interval == 0 that it
 * survives, the cell it was in before the move (getCellCoordinates,
 * cell.h:64-67) gains one count in frame t / frame_interval.
 *
 * counts is the ParticleCount vector (pic_tracer.cxx:26-71): num_frames x
 * size[0] x size[1] x size[2] uint32, row-major, frame slowest; the calls
 * ADD to it, as `res += ...` does (pic_tracer.cxx:282). A cell coordinate
 * on the upper face (a particle exactly at origin + cellWidth * size) lands
 * where the reference's flat index puts it; an index outside the vector,
 * undefined behaviour in the reference, is not counted. Arithmetic is FP64
 * in the reference's order: trajectories and counts equal those of its host
 * build. num_frames must exceed (steps - 1) / frame_interval (pic_tracer
 * uses T / S + 1); frame_interval > 0.
 *
 * ipic3d_gpu_trace takes host pointers (particles are copied in, counts in
 * and out; returns when done; calls are serialised, and the device buffers
 * and stream it uses are kept, grown on demand, until the process exits).
 * ipic3d_gpu_trace_device takes device pointers
 * (particles 16-byte aligned) and enqueues the work on `stream` (a
 * cudaStream_t, NULL = default stream) without synchronising. */
int ipic3d_gpu_trace(const ipic3d_props* props, const ipic3d_particle* particles, uint64_t n, int32_t steps,
                     int32_t frame_interval, int32_t num_frames, uint32_t* counts);
int ipic3d_gpu_trace_device(const ipic3d_props* props, const ipic3d_particle* d_particles, uint64_t n,
                            int32_t steps, int32_t frame_interval, int32_t num_frames, uint32_t* d_counts,
                            void* stream);

/* ---- errors -------------------------------------------------------------- */
/* Copies the message of the last failure on this thread into buf. Returns
 * the last status. */
int ipic3d_gpu_last_error(char* buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif /* IPIC3D_GPU_H */
