// Device-side data structures and helpers of the GB300 particle path.
//
// One "universe" (the reference's Universe, universe.h:12-51) lives in HBM as
//   * FP64 field grids in the reference layout (field.h:14-38):
//       field   (s+3)^3 x {E,B,Bext}     bcfield (s+2)^3 x Bc
//       J       (s+1)^3 x 3              rho     (s+1)^3
//   * one or more particle populations (one per distinct (q, qom) pair),
//     each a structure-of-arrays grouped by cell: cell c owns the slot range
//     [start[c], start[c+1]); its first count[c] slots hold particles, the
//     rest is slack for arrivals. start[] is a multiple of 8 so that a
//     thread's 4 or 8 consecutive slots always belong to one cell.
//   * FP64 populations store absolute positions (Particle::position,
//     particle.h:11); FP32 populations store the position relative to the
//     cell origin in units of the cell width, in [0, 1] when inside.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ipg {

constexpr int kVec = 4;                 // particles per thread (one float4 / 2x double2)
constexpr int kPushThreads = 256;       // threads per CTA of the push kernel
constexpr int kSlotsPerCta = kVec * kPushThreads;
constexpr int kSetPops = 4;             // populations per launch of the population-set kernels
constexpr int kSlotAlign = 8;          // start[] and every cell's capacity are multiples of 8
constexpr int kMaxCellsPerCta = kSlotsPerCta / kSlotAlign + 2;

// Geometry and physics of one universe (UniverseProperties plus the policy).
struct Geom {
    int sx, sy, sz;
    int ncells;
    double w[3], inv_w[3], half_w[3];
    double origin[3];
    double object_center[3];
    double L[3];            // domain length per axis
    double dt, c;
    double inv_pic;         // 1 / (pi c): the sub-cycle estimate
    double planet_r2;       // planetRadius * planetRadius (cell.h:1126)
    double mft;             // -Bext.z * pow(R, 3), host glibc pow (cell.h:923)
    double vol;             // w.x * w.y * w.z
    int bc_lo[3], bc_hi[3];
    uint32_t flags;
    int mover;              // 0 dipole, 1 field gather
    int deposit;            // 1 = deposit J/rho of the moved particles
    double* field;          // (s+3)^3 x 9
    double* bcfield;        // (s+2)^3 x 3
    double* J;              // (s+1)^3 x 3 raw sums during the deposit
    double* rho;            // (s+1)^3
    float4* node32;         // (s+3)^3 x 2 float4: {Ex,Ey,Ez,0},{Bx,By,Bz,0} (FP32 path, else null)
    const float* cellcoef;  // s^3 x 48: trilinear polynomial of E, B per cell (FP32 push)
};

// A particle that leaves its slot (migration) or waits for a slot (pending).
template <typename T>
struct Mover {
    int32_t cell;           // destination cell (for pending: the cell it is in)
    uint32_t id;
    T x, y, z, u, v, w;
};

// Step-global counters, reset at the start of every step.
struct StepCounters {
    uint32_t outbox;        // entries written to the outbox this step
    uint32_t pending_out;   // arrivals that found no slot -> pending next step
    uint32_t deferred;      // leavers kept in their slot (outbox full)
    uint32_t removed;       // particles removed (planet, open faces)
    uint32_t migrated;      // particles that changed cell
    uint32_t injected;
    uint32_t dirty;         // cells with holes or arrivals this step (entries of dirty_list)
    uint32_t lost;          // pending list overflow (must stay 0)
    uint32_t timeouts;      // CTAs that gave up a bounded wait (must stay 0)
};

template <typename T>
struct Pop {
    T *x, *y, *z, *u, *v, *w;
    uint32_t* id;           // nullable
    const int64_t* start;   // [ncells + 1]
    const int2* cta_cells;  // per push CTA: first cell and number of cells it touches
    int32_t* count;         // [ncells]
    int32_t* hole_cnt;      // [ncells]
    int32_t* hole_list;     // [capacity] holes of cell c at start[c] + k
    int32_t* arr_cnt;       // [ncells]
    int32_t* arr_list;      // [capacity] arrivals of cell c at start[c] + k (outbox index)
    int32_t* dirty_flag;    // [ncells] 1 while the cell is on this step's dirty list
    int32_t* dirty_list;    // [ncells] cells with holes or arrivals (the placement's work list)
    Mover<T>* outbox;
    uint32_t outbox_cap;
    Mover<T>* pending_in;   // pushed this step
    Mover<T>* pending_out;  // arrivals without a slot this step
    uint32_t pending_cap;
    const uint32_t* pending_in_count;
    StepCounters* ctr;
    int64_t capacity;       // total slots
    double q, qom;
    int32_t pad[2];
};

// Up to kSetPops populations of one universe advanced by one launch
// (blockIdx.y = population for the placement, pending and rotation kernels).
template <typename T>
struct PopSet {
    Pop<T> p[kSetPops];
    int32_t* sort_tmp[kSetPops];    // placement scratch of each population
    uint32_t* pend_count[kSetPops]; // = p[i].pending_in_count, writable (rotation)
    int n;
};

// Launch shape of the pipelined FP32 push, chosen per context (or batch) by
// the autotuner of ipic3d_gpu.cu: a tile of at most `item_cells` cells is
// split into work items of `item` particles (one warp each), a sparser tile
// is pushed slot by slot; `per_sm` persistent thread blocks run on each SM.
struct PushShape {
    int32_t item;        // a power of two, 32..1024
    int32_t item_cells;  // 0..32 (0: every tile slot by slot)
    int32_t per_sm;      // 1..the blocks that fit on an SM
    // polls (of ~20 us each) after which a wait on a shared-memory barrier
    // gives up; < 0: the default bound (about 1 s)
    int32_t wait_polls = -1;
};
constexpr PushShape kDefaultPushShape{256, 32, 2};

// Every constant of the step in FP32, computed on the host: the kernel runs
// no FP64 instruction per particle (GB300's FP64 rate is a small fraction of
// its FP32 rate).
struct Push32Const {
    float qom;        // charge over mass of the species
    float k_sub;      // dt * 4 |qom| / (pi c): dt / dt_sub = k_sub |B|^2
    float dt;
    float mft;        // -Bext.z R^3
    float planet_r2;
    float w[3], inv_w[3];
    float origin[3];  // domain origin relative to the dipole centre (0,0,0)
    float center[3];  // object centre (planet)
    float inv_sy, inv_sz;  // 1 / cells along y and z (cell index -> coordinates)
    float k1;         // qom * 0.5 * dt: the Boris factor of a single sub-cycle
    float a1[3];      // dt / w: the position step of a single sub-cycle (cell widths per velocity unit)
};

// The push constants of the populations of a PopSet.
struct Push32Set {
    Push32Const c[kSetPops];
};

// ---- batched ensemble ------------------------------------------------------
// One population of one universe of a batch: everything a batched particle
// kernel needs, read from a device table indexed by job.
template <typename T>
struct alignas(16) PopJob {  // 16-byte multiple: the FP32 push bulk-copies records
    Geom g;
    Pop<T> P;
    Push32Const pc;         // FP32 populations: the push constants
    int32_t* sort_tmp;      // placement scratch [capacity]
    uint32_t* pend_count;   // P.pending_in_count (written by the rotation)
};

// One universe of a batch (field-level kernels, counters).
struct InstJob {
    Geom g;
    uint64_t* step;         // device step counter
    int job0, njobs;        // its populations: PopJob entries [job0, job0 + njobs)
    uint32_t pend_limit;    // waiting particles above which it is re-laid out
    int div8;               // J = Js / vol / 8
    int refresh_b;          // leapfrog refreshes node B from Bc
    float* cellcoef;        // FP32 field-gather coefficients (writable view)
    double coef_scale;      // 1 / vol with the gather normalisation, else 1
};

// Copies a batch job record into shared memory (all threads of the block
// call it; followed by a barrier), so the kernel body reads its fields from
// shared memory instead of global memory.
template <typename Job>
__device__ __forceinline__ void load_job(Job& dst, const Job* src) {
    static_assert(sizeof(Job) % 4 == 0, "job records are word-sized");
    const int* s = reinterpret_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(Job) / 4); i += blockDim.x) d[i] = s[i];
    __syncthreads();
}

// Per-job counters as read back after a batched step.
struct JobStatus {
    StepCounters c;
    uint32_t pending_in;
    uint32_t pad;
};

// ---- small helpers --------------------------------------------------------

__device__ __forceinline__ int64_t field_index(const Geom& g, int x, int y, int z) {
    return ((int64_t)x * (g.sy + 3) + y) * (g.sz + 3) + z;
}
__device__ __forceinline__ int64_t bc_index(const Geom& g, int x, int y, int z) {
    return ((int64_t)x * (g.sy + 2) + y) * (g.sz + 2) + z;
}
__device__ __forceinline__ int64_t node_index(const Geom& g, int x, int y, int z) {
    return ((int64_t)x * (g.sy + 1) + y) * (g.sz + 1) + z;
}
__device__ __forceinline__ void cell_coords(const Geom& g, int c, int& x, int& y, int& z) {
    z = c % g.sz;
    int t = c / g.sz;
    y = t % g.sy;
    x = t / g.sy;
}
__device__ __forceinline__ int cell_id(const Geom& g, int x, int y, int z) { return (x * g.sy + y) * g.sz + z; }

// q = a / d, r = a % d for 0 <= a < 2^24 and 0 < d < 2^12 through a float
// reciprocal and one correction step (no integer division)
__device__ __forceinline__ int fast_div(int a, int d, float inv_d) {
    int q = __float2int_rz(__int2float_rn(a) * inv_d);
    const int r = a - q * d;
    q += (r >= d) - (r < 0);
    return q;
}

// Flags cell c as touched this step (holes or arrivals): a plain store, no
// round trip; k_dirty_compact lists the flagged cells for the placement,
// which clears the flag.
template <typename T>
__device__ __forceinline__ void mark_dirty(const Pop<T>& P, int c) {
    P.dirty_flag[c] = 1;
}

// Files slot `slot` as a hole of cell c (its slots start at cstart).
template <typename T>
__device__ __forceinline__ void file_hole(const Pop<T>& P, int c, int64_t cstart, int64_t slot) {
    const int k = atomicAdd(P.hole_cnt + c, 1);
    P.hole_list[cstart + k] = (int32_t)slot;
    mark_dirty(P, c);
}

// t = (a * n1 + b) * n2 + c for t in [0, n0 * n1 * n2): 32-bit divisions
// when t fits (64-bit division by a runtime divisor is a long software
// sequence on the GPU).
// Blocks of the batched placement for a universe of `ncells` cells: one per
// 512 cells (256 threads, a cell per 8 lanes: 32 cells at a time).
__host__ __device__ inline int place_blocks(int ncells) { return ncells > 0 ? (ncells + 511) / 512 : 1; }

__device__ __forceinline__ void split3(int64_t t, int n1, int n2, int& a, int& b, int& c) {
    if (t < 0x7fffffff) {
        const unsigned u = (unsigned)t, r = u / (unsigned)n2;
        c = (int)(u - r * (unsigned)n2);
        a = (int)(r / (unsigned)n1);
        b = (int)(r - (unsigned)a * (unsigned)n1);
    } else {
        c = (int)(t % n2);
        const int64_t r = t / n2;
        b = (int)(r % n1);
        a = (int)(r / n1);
    }
}

// Warp-aggregated atomic increment: one atomic per warp for all active
// lanes with pred set; returns this lane's slot (or undefined if !pred).
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    unsigned mask = __activemask();
    unsigned ballot = __ballot_sync(mask, pred);
    if (!ballot) return 0;
    int lane = threadIdx.x & 31;
    int leader = __ffs(ballot) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(ballot));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(ballot & ((1u << lane) - 1));
}

}  // namespace ipg
