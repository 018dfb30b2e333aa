// The FP32 push as a persistent, warp-specialised, TMA-pipelined kernel.
//
// Each CTA has one producer warp and eleven compute warps. The producer's
// elected lane streams 1024-slot tiles of a population through a ring of
// shared-memory stages with bulk copies (cp.async.bulk, completion counted
// on the stage's `full` mbarrier): x y z u v w of the tile's slots and the
// tile's slice of the cell tables start[] / count[]. The compute warps push
// the particles of a stage in shared memory and release it on its `empty`
// mbarrier; the producer then writes the stage back in place with bulk
// stores and refills it with the tile after next. No compute thread loads or
// stores particle state in global memory and no CTA-wide barrier separates
// the warps: a warp waits only for the data it works on.
//
// Work inside a tile. A tile whose cells are large (at most 32 cells) is cut
// into items: the occupied slots of one cell, PushShape::item at a time. Warps
// take items from a per-stage counter; lane l pushes the item's particles
// l, l + 32, ..., then a second pass over the stayers adds their cloud-in-
// cell moments to the lane's accumulators, so a warp sums one cell and
// flushes it once (transpose-reduction across the lanes). A tile of many small cells goes thread-per-4-slots instead:
// warp w pushes slots [128 w, 128 w + 128) and flushes its per-cell runs of
// lanes through a shared-memory tile.
//
// Per particle the physics is step32's (push32.cuh): field gather from the
// cell's trilinear polynomial and/or the analytic dipole, the reference's
// sub-cycled Boris mover (particle.h:31-49, cell.h:896-964) and the export
// classification (cell.h:1093-1146), with the wall logic skipped for cells
// that touch no reflecting or open face.
//
// Deposit of the stayers (cell.h:787-824 in scatter form): the monomial
// moments of the particles about the cell centre, Q m(r - 1/2) for Q in
// {u, v, w, 1} and m in {1, x, y, xy, z, xz, yz, xyz} (moment index = bits
// x|y<<1|z<<2), are summed per cell; lane v then owns value v = 8 Q + m and
// three butterflies (one per axis: (a, b) -> (a/2 - b, a/2 + b)) turn the
// moments into the sums of the cloud-in-cell weights (1 - r, r) per corner:
// one FP64 atomic per lane adds corner m's component Q to its node. Centred
// moments keep the FP32 sums small, so the butterflies' cancellation loses
// no more than the sums' own rounding.
//
// Every wait on an mbarrier is bounded (PushShape::wait_polls polls, by
// default kMaxPolls: about 1 s): on expiry the CTA records a timeout in the
// population's counters, drains its own copies in flight (with the default
// bound: those copies are real and complete) and returns; the host turns the
// count into IPIC3D_E_TIMEOUT.
#pragma once

#include <cstddef>

#include "push32.cuh"

namespace ipg {

// ---- bulk copy / mbarrier primitives (sm_90+ PTX) ---------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// One poll of the phase with parity `parity`; the thread sleeps in the
// barrier until the phase completes or about kPollNs nanoseconds pass.
constexpr uint32_t kPollNs = 20000;
__device__ __forceinline__ uint32_t mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "n"(kPollNs)
        : "memory");
    return ok;
}
// Polls until the phase completes: false after `polls` polls (the default
// kMaxPolls: about 1 s) or as soon as *abort is set.
constexpr uint32_t kMaxPolls = 1000000000u / kPollNs;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, const volatile int* abort,
                                          uint32_t polls = kMaxPolls) {
    for (uint32_t it = 0; it < polls; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort) break;
    }
    return false;
}
// global -> shared, `bytes` (multiple of 16, both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(smem_dst)),
                 "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// shared -> global, same rules
__device__ __forceinline__ void bulk_store(void* gdst, const void* smem_src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_u32(smem_src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the shared-memory sources of all committed bulk stores have been read
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// all committed bulk stores are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) accesses
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- shared-memory layout ------------------------------------------------------
constexpr int kTileSlots = kSlotsPerCta;  // 1024 slots per tile (the cta_cells table's unit)
// 11 compute warps + the producer: 2 CTAs = 24 warps per SM, 6 per
// scheduler, 80 registers per thread
constexpr int kComputeWarps = 11;
constexpr int kComputeThreads = kComputeWarps * 32;
constexpr int kPipeThreads = kComputeThreads + 32;  // + the producer warp
constexpr int kSlotWarps = kTileSlots / 128;        // slot mode: 128-slot slices of a tile
// item mode (tiles of at most PushShape::item_cells cells, work items of
// PushShape::item particles): the cells' field coefficients are staged
constexpr int kItemMaxCells = 32;

// Every member is a bulk-copy destination: 16-byte aligned offsets.
struct __align__(16) PipeStage {
    alignas(16) float s[6][kTileSlots];              // x y z u v w of the tile's slots
    alignas(16) float coef[kItemMaxCells * 48];      // item mode + field gather: cellcoef of the tile's cells
    alignas(16) int64_t start[kMaxCellsPerCta + 4];  // start[(c0 & ~1) ...]
    alignas(16) int32_t count[kMaxCellsPerCta + 8];  // count[(c0 & ~3) ...]
    alignas(16) PopJob<float> job;                   // batched launch: the tile's job record
};
static_assert(offsetof(PipeStage, coef) % 16 == 0 && offsetof(PipeStage, start) % 16 == 0 &&
                  offsetof(PipeStage, count) % 16 == 0 && offsetof(PipeStage, job) % 16 == 0 &&
                  sizeof(PipeStage) % 16 == 0 && sizeof(PopJob<float>) % 16 == 0,
              "bulk copies need 16-byte aligned shared-memory destinations");

// Item mode: what the compute warps need to know about a cell of the
// stage's tile -- its occupied slots [lo, hi) within the tile, the exclusive
// prefix of the tile's items before it, its first slot and its CellInfo --
// written once per tile by the first warp to reach it.
struct CellDesc {
    int lo, hi, excl, cst;
    CellInfo ci;
    int64_t node0;  // the node of the cell's corner (0,0,0)
    int64_t unused;
};
static_assert(sizeof(CellDesc) == 48, "three 16-byte loads per cell");

template <int kStages>
struct PipeSmem {
    PipeStage stage[kStages];
    CellDesc cells[kStages][kItemMaxCells];
    uint64_t full[kStages];               // the stage's copies landed
    uint64_t empty[kStages];              // the compute warps are done with the stage
    uint64_t ready[kStages];              // the tile's cell descriptors are written
    uint8_t item_cell[kStages][kTileSlots / 32 + kItemMaxCells];  // item j of the tile: its cell - c0
    int total[kStages];                   // items of the stage's tile
    int claim[kStages];                   // warps that reached the stage's tile (the first writes the descriptors)
    int2 desc[kStages];                   // (first cell, number of cells) of the stage's tile
    int pop[kStages];                     // population (batched launch: job) of the stage's tile
    int ltile[kStages];                   // the tile's index within its population
    int next_item[kStages];               // item counter of the stage's tile
    int abort;                            // a wait expired: every warp stops
};

static_assert(offsetof(PipeSmem<3>, stage) == 0, "stages first");

template <int kStages>
constexpr size_t pipe_smem_bytes() {
    return sizeof(PipeSmem<kStages>);
}

// Bulk-copy sizes of one tile (all multiples of 16 bytes; every source
// 16-byte aligned: slot bases are multiples of 1024, the cell tables are
// read from an even / multiple-of-4 index and allocated with padding).
struct TileCopy {
    int64_t base;
    uint32_t slot_bytes;   // per array
    int64_t s_first;       // first start[] entry copied
    uint32_t s_bytes;
    int64_t c_first;       // first count[] entry copied
    uint32_t c_bytes;
};

__device__ __forceinline__ TileCopy tile_copy(const Pop<float>& P, int tile, int2 desc) {
    TileCopy t;
    t.base = (int64_t)tile * kTileSlots;
    const int64_t n = P.capacity - t.base < kTileSlots ? P.capacity - t.base : kTileSlots;
    t.slot_bytes = (uint32_t)(n * 4);
    t.s_first = desc.x & ~1;
    const int64_t ns = ((int64_t)desc.x + desc.y + 1 - t.s_first + 1) & ~int64_t(1);
    t.s_bytes = (uint32_t)(ns * 8);
    t.c_first = desc.x & ~3;
    const int64_t ncnt = ((int64_t)desc.x + desc.y - t.c_first + 3) & ~int64_t(3);
    t.c_bytes = (uint32_t)(ncnt * 4);
    return t;
}

// Issued by the producer: the tile's copies into `st`, counted on `bar`
// (`extra` more bytes are expected from copies the caller issues);
// with `coef` (item mode, field gather) also the cells' field coefficients
// (48 floats = 192 bytes per cell, contiguous from cell c0). In two parts:
// the byte count and the cell tables first, the slot arrays second, so that
// a refill can start before the previous tile's bulk stores have read the
// slot arrays.
__device__ __forceinline__ void issue_tile_tables(const Pop<float>& P, const float* coef, int tile, int2 desc,
                                                  int item_cells, PipeStage& st, uint64_t* bar, uint32_t extra = 0) {
    const TileCopy t = tile_copy(P, tile, desc);
    const bool with_coef = coef != nullptr && desc.y <= item_cells;
    const uint32_t coef_bytes = with_coef ? (uint32_t)desc.y * 192u : 0u;
    mbar_arrive_expect_tx(bar, 6u * t.slot_bytes + t.s_bytes + t.c_bytes + coef_bytes + extra);
    bulk_load(st.start, P.start + t.s_first, t.s_bytes, bar);
    bulk_load(st.count, P.count + t.c_first, t.c_bytes, bar);
    if (coef_bytes) bulk_load(st.coef, coef + (size_t)desc.x * 48, coef_bytes, bar);
}
__device__ __forceinline__ void issue_tile_slots(const Pop<float>& P, int tile, int2 desc, PipeStage& st,
                                                 uint64_t* bar) {
    const TileCopy t = tile_copy(P, tile, desc);
    float* const arr[6] = {P.x, P.y, P.z, P.u, P.v, P.w};
#pragma unroll
    for (int a = 0; a < 6; ++a) bulk_load(st.s[a], arr[a] + t.base, t.slot_bytes, bar);
}

// ---- per-particle physics --------------------------------------------------------

// Compile-time policy of one pipelined push launch (template bit set).
enum : int {
    kPipeStep = 1,     // mover + export (else: deposit of the particles as they are)
    kPipeGather = 2,   // field-gather mover: E, B from the cell's polynomial
    kPipeDipole = 4,   // analytic dipole B added
    kPipeDeposit = 8,  // cloud-in-cell deposit of J and rho
};

__device__ __forceinline__ PState<float> load_slot(const PipeStage& st, int sl) {
    PState<float> p;
    p.x = st.s[0][sl]; p.y = st.s[1][sl]; p.z = st.s[2][sl];
    p.u = st.s[3][sl]; p.v = st.s[4][sl]; p.w = st.s[5][sl];
    return p;
}
__device__ __forceinline__ void store_slot(PipeStage& st, int sl, const PState<float>& p) {
    st.s[0][sl] = p.x; st.s[1][sl] = p.y; st.s[2][sl] = p.z;
    st.s[3][sl] = p.u; st.s[4][sl] = p.v; st.s[5][sl] = p.w;
}
// A slot whose particle left (a hole now, whose contents nothing reads):
// the cell centre at rest, so that the moment pass adds exactly zero for it
// (every centred monomial but 1 is 0, and so is the velocity; the rho count
// is taken apart).
__device__ __forceinline__ void clear_slot(PipeStage& st, int sl) {
    st.s[0][sl] = 0.5f; st.s[1][sl] = 0.5f; st.s[2][sl] = 0.5f;
    st.s[3][sl] = 0.f; st.s[4][sl] = 0.f; st.s[5][sl] = 0.f;
}

// FP64 atomic of corner m (bits x|y<<1|z<<2) and component q (0-2 J, 3 rho)
// of the cell at (cx, cy, cz).
__device__ __forceinline__ void corner_atomic_add(const Geom& g, int cx, int cy, int cz, int m, int q, double val) {
    const int64_t n = node_index(g, cx + (m & 1), cy + ((m >> 1) & 1), cz + (m >> 2));
    // one atomic instruction for the warp: the address is selected, not the branch
    double* p = q < 3 ? g.J + 3 * n + q : g.rho + n;
    atomicAdd(p, val);
}

// Cloud-in-cell deposit of the warp's leavers (ballot `lb`) into their
// destination cells, one leaver at a time: lane l adds component l >> 3 at
// corner l & 7 -- one 32-lane atomic per leaver.
__device__ __forceinline__ void deposit_leavers32(const Geom& g, unsigned lb, int nx, int ny, int nz,
                                                  const PState<float>& p, double q) {
    const int lane = threadIdx.x & 31, m = lane & 7, comp = lane >> 3;
    while (lb) {
        const int src = __ffs(lb) - 1;
        lb &= lb - 1;
        const int cx = __shfl_sync(0xffffffffu, nx, src), cy = __shfl_sync(0xffffffffu, ny, src),
                  cz = __shfl_sync(0xffffffffu, nz, src);
        const float x = __shfl_sync(0xffffffffu, p.x, src), y = __shfl_sync(0xffffffffu, p.y, src),
                    z = __shfl_sync(0xffffffffu, p.z, src);
        const float u = __shfl_sync(0xffffffffu, p.u, src), v = __shfl_sync(0xffffffffu, p.v, src),
                    w = __shfl_sync(0xffffffffu, p.w, src);
        const float wt = ((m & 1) ? x : 1.f - x) * ((m & 2) ? y : 1.f - y) * ((m & 4) ? z : 1.f - z);
        const float Q = comp == 0 ? u : (comp == 1 ? v : (comp == 2 ? w : 1.f));
        const double val = (double)(Q * wt) * q;
        if (val != 0.0) corner_atomic_add(g, cx, cy, cz, m, comp, val);
    }
}

// Adds the centred cloud-in-cell moments of a particle to acc (index 8 Q +
// m, Q in {u, v, w, 1}, m in {1, x, y, xy, z, xz, yz, xyz} of r - 1/2) in
// packed FP32 pairs (m, m + 1): four packed FMAs per velocity component and
// four packed adds for the rho moments. acc[24] counts every slot it is
// given, cleared or not; the callers replace that sum by the stayer count.
// A cleared slot (clear_slot) adds zero to every other moment.
__device__ __forceinline__ void add_moments(float (&acc)[32], const PState<float>& p) {
    const float x = p.x - 0.5f, y = p.y - 0.5f, z = p.z - 0.5f;
    // separate roundings (no fusion with the sums below in some kernels only)
    const float xy = __fmul_rn(x, y), xz = __fmul_rn(x, z), yz = __fmul_rn(y, z), xyz = __fmul_rn(xy, z);
    const float2 M[4] = {make_float2(1.f, x), make_float2(y, xy), make_float2(z, xz), make_float2(yz, xyz)};
    const float Q[3] = {p.u, p.v, p.w};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float2 Q2 = dup2(Q[q]);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            // Q * 1 + acc rounds as acc + Q
            const float2 r = fma2(Q2, M[k], make_float2(acc[q * 8 + 2 * k], acc[q * 8 + 2 * k + 1]));
            acc[q * 8 + 2 * k] = r.x;
            acc[q * 8 + 2 * k + 1] = r.y;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 r = add2(make_float2(acc[24 + 2 * k], acc[25 + 2 * k]), M[k]);
        acc[24 + 2 * k] = r.x;
        acc[25 + 2 * k] = r.y;
    }
}

// Lane v holds the summed moment v = 8 Q + m of one cell: the three axis
// butterflies give the cloud-in-cell corner sum of corner m, component Q;
// one FP64 atomic adds it (times the charge) to the node.
__device__ __forceinline__ void emit_corner_sums(const Geom& g, float s, int cx, int cy, int cz, double q) {
    const int lane = threadIdx.x & 31, m = lane & 7;
#pragma unroll
    for (int bit = 1; bit < 8; bit <<= 1) {
        const float o = __shfl_xor_sync(0xffffffffu, s, bit);
        s = (m & bit) ? fmaf(0.5f, o, s) : fmaf(0.5f, s, -o);
    }
    if (s != 0.f) corner_atomic_add(g, cx, cy, cz, m, lane >> 3, (double)s * q);
}

// emit_corner_sums for a cell given by the node of its corner (0,0,0).
__device__ __forceinline__ void emit_node_sums(const Geom& g, float s, int64_t node0, double q) {
    const int lane = threadIdx.x & 31, m = lane & 7, Q = lane >> 3;
#pragma unroll
    for (int bit = 1; bit < 8; bit <<= 1) {
        const float o = __shfl_xor_sync(0xffffffffu, s, bit);
        s = (m & bit) ? fmaf(0.5f, o, s) : fmaf(0.5f, s, -o);
    }
    const int64_t nz = g.sz + 1, nyz = (int64_t)(g.sy + 1) * nz;
    const int64_t n = node0 + ((m & 1) ? nyz : 0) + ((m & 2) ? nz : 0) + (m >> 2);
    double* p = Q < 3 ? g.J + 3 * n + Q : g.rho + n;
    if (s != 0.f) atomicAdd(p, (double)s * q);
}

// Leaver bookkeeping of one warp step: outbox (one warp-aggregated append),
// arrival list of the destination, cooperative deposit; the old slot is
// filed as a hole of its cell (leavers and drops). `dir` is the export's
// move. The round trips (the destination's arrival slot, the outbox slots,
// the hole slots) are issued together before any result is used, and cells
// are flagged with plain stores (k_dirty_compact lists them). kOneCell:
// every lane's slot is in `cell` (item mode), so the warp files its holes
// with one aggregated atomic.
template <bool kOneCell>
__device__ __forceinline__ void leave_and_hole(const Geom& g, const Pop<float>& P, const Push32Const& pc, int outcome,
                                               int dir, const PState<float>& p, int slot, int cell,
                                               int cstart, bool deposit, uint32_t& nmig, uint32_t& nrem) {
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const bool leave = outcome == kMove, hole = leave || outcome == kDrop;
    const unsigned lb = __ballot_sync(0xffffffffu, leave), hb = __ballot_sync(0xffffffffu, hole);
    if (!hb) return;  // (every leaver leaves a hole)
    // hole slots
    int hk = 0;
    if (kOneCell) {
        if (lane == __ffs(hb) - 1) hk = atomicAdd(P.hole_cnt + cell, __popc(hb));
    } else if (hole) {
        hk = atomicAdd(P.hole_cnt + cell, 1);
    }
    int nx = 0, ny = 0, nz = 0;
    if (lb) {
        // destination cell (periodic wrap of the index, as the outbox expects)
        const int3 c = cell_xyz(g, pc, cell);
        nx = c.x + (dir & 3) - 1;
        ny = c.y + ((dir >> 2) & 3) - 1;
        nz = c.z + ((dir >> 4) & 3) - 1;
        nx = nx < 0 ? nx + g.sx : (nx >= g.sx ? nx - g.sx : nx);
        ny = ny < 0 ? ny + g.sy : (ny >= g.sy ? ny - g.sy : ny);
        nz = nz < 0 ? nz + g.sz : (nz >= g.sz ? nz - g.sz : nz);
        const int dc = cell_id(g, nx, ny, nz);
        int ak = 0;
        int64_t ds = 0, de = 0;
        uint32_t id = 0u;
        if (leave) {
            ak = atomicAdd(P.arr_cnt + dc, 1);  // the arrival slot of the destination
            ds = P.start[dc];
            de = P.start[dc + 1];
            if (P.id) id = P.id[slot];
        }
        const int leader = __ffs(lb) - 1;
        uint32_t o = 0;
        if (lane == leader) o = atomicAdd(&P.ctr->outbox, (uint32_t)__popc(lb));
        o = __shfl_sync(0xffffffffu, o, leader) + __popc(lb & below);
        if (leave) {
            Mover<float> m;
            m.cell = dc;
            m.id = id;
            m.x = p.x; m.y = p.y; m.z = p.z;
            m.u = p.u; m.v = p.v; m.w = p.w;
            mark_dirty(P, dc);
            // the outbox holds every particle of the population plus the
            // pending and injected ones: o is always below its capacity
            const bool in_box = o < P.outbox_cap;
            if (in_box) P.outbox[o] = m;
            else atomicAdd(&P.ctr->lost, 1u);
            if (ak < (int)(de - ds)) {
                P.arr_list[ds + ak] = in_box ? (int32_t)o : 0;
            } else {  // the destination's slots are short: wait a step
                const uint32_t pi = atomicAdd(&P.ctr->pending_out, 1u);
                if (pi < P.pending_cap) P.pending_out[pi] = m;
                else atomicAdd(&P.ctr->lost, 1u);
            }
            ++nmig;
        }
        if (deposit) deposit_leavers32(g, lb, nx, ny, nz, p, P.q);
    }
    if (kOneCell) {
        hk = __shfl_sync(0xffffffffu, hk, __ffs(hb) - 1) + __popc(hb & below);
        if (lane == 0) mark_dirty(P, cell);
    } else if (hole) {
        mark_dirty(P, cell);
    }
    if (hole) P.hole_list[cstart + hk] = (int32_t)slot;
    if (outcome == kDrop) ++nrem;
}

// Item mode: the warp pushes particles [a, b) (tile-local slots, b - a <=
// PushShape::item) of cell `cell`, lane l taking a + l, a + l + 32, ... When
// no particle of a warp step needs more than one Boris sub-cycle (the common
// case) the step is straight-line code with the species' one-step
// constants. Stayers go back to the stage (the producer writes the whole
// tile back with bulk stores); the slots of leavers and drops are cleared
// (holes now). A second pass sums the stayers' cloud-in-cell moments and
// flushes the cell once, with the stayer count from the first pass's
// ballots. `coef` points at the cell's 48 field coefficients (shared memory).
template <int kF>
__device__ __forceinline__ void push_item(const Geom& g, const Pop<float>& P, const Push32Const& pc,
                                          const Push32Const& sp, PipeStage& st, const float* coef,
                                          const CellInfo& ci, int base, int cell, int64_t node0, int cstart, int a,
                                          int b, uint32_t& nmig, uint32_t& nrem) {
    constexpr bool kStep = (kF & kPipeStep) != 0, kDep = (kF & kPipeDeposit) != 0;
    constexpr bool kGather = (kF & kPipeGather) != 0, kDipole = (kF & kPipeDipole) != 0;
    const int lane = threadIdx.x & 31;
    int gone = 0;  // leavers and drops of the item (warp-uniform)
    if (kStep) {
        const float k1 = sp.k1, ksub = sp.k_sub;
        const bool plain = (ci.flags & (kCellEdge | kCellNear)) == 0;
#pragma unroll 1
        for (int s0 = a; s0 < b; s0 += 32) {
            const int sl = s0 + lane;
            // a lane past the item works on a copy of slot a and keeps nothing
            PState<float> p = load_slot(st, sl < b ? sl : a);
            float E[6];
            if (kGather) {
                fields_one<true>(coef, p, E);
            } else {
#pragma unroll
                for (int q = 0; q < 6; ++q) E[q] = 0.f;
            }
            if (kDipole) add_dipole(pc, ci, p, E);
            const float r = sub_ratio(ksub, E);
            if (__all_sync(0xffffffffu, r < 1.f))
                boris32<1>(k1, pc.a1[0], pc.a1[1], pc.a1[2], E, p);
            else if (r < 1.f)
                boris32<1>(k1, pc.a1[0], pc.a1[1], pc.a1[2], E, p);
            else
                boris_sub(pc, sp, r, E, p);
            // a cell away from the domain faces and the planet, whose
            // particles all stayed in it: export32 would return kStay for
            // each, so they go straight back to the stage
            const bool in = p.x >= 0.f && p.x <= 1.f && p.y >= 0.f && p.y <= 1.f && p.z >= 0.f && p.z <= 1.f;
            if (plain && __all_sync(0xffffffffu, in || sl >= b)) {
                if (sl < b) store_slot(st, sl, p);
                continue;
            }
            int dir = 0;
            int o = export32(g, pc, ci, p, dir);
            o = sl < b ? o : -1;
            if (o == kStay) store_slot(st, sl, p);
            else if (kDep && o > 0) clear_slot(st, sl);
            if (__any_sync(0xffffffffu, o > 0)) {
                gone += __popc(__ballot_sync(0xffffffffu, o > 0));
                leave_and_hole<true>(g, P, pc, o, dir, p, base + sl, cell, cstart, kDep, nmig, nrem);
            }
        }
        __syncwarp();
    }
    if (!kDep) return;
    float acc[32];
#pragma unroll
    for (int l = 0; l < 32; ++l) acc[l] = 0.f;
    int s0 = a;
#pragma unroll 1
    for (; s0 + 64 <= b; s0 += 64) {
        add_moments(acc, load_slot(st, s0 + lane));
        add_moments(acc, load_slot(st, s0 + 32 + lane));
    }
#pragma unroll 1
    for (; s0 < b; s0 += 32) {
        const int sl = s0 + lane;
        PState<float> p = load_slot(st, sl < b ? sl : a);
        if (sl >= b) {  // past the item: adds zero
            p.x = p.y = p.z = 0.5f;
            p.u = p.v = p.w = 0.f;
        }
        add_moments(acc, p);
    }
    float s = warp_transpose_sum<float>(acc);
    if (lane == 24) s = (float)(b - a - gone);  // the stayers: sum of the rho weights' 1 term
    emit_node_sums(g, s, node0, P.q);
}

// warp_transpose_sum of acc over the lanes with `mine` set (the others add
// zero), without a masked copy of acc: the first exchange applies the mask.
__device__ __forceinline__ float run_transpose_sum(const float (&acc)[32], bool mine) {
    const int lane = threadIdx.x & 31;
    const bool upper = (lane & 16) != 0;
    float v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const float send = mine ? (upper ? acc[i] : acc[i + 16]) : 0.f;
        const float keep = mine ? (upper ? acc[i + 16] : acc[i]) : 0.f;
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int off = 8; off >= 1; off >>= 1) {
        const bool up = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < off; ++i) {
            const float send = up ? v[i] : v[i + off];
            const float keep = up ? v[i + off] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    return v[0];
}

// Slot mode: slice w of the tile (slots [128 w, 128 w + 128)) is pushed by
// one warp, thread t of the slice the 4 slots from 4 t (one cell:
// capacities are multiples of 8), in two passes as in item mode (move, then
// moments of the stayers), and flushed per run of lanes of one cell.
template <int kF>
__device__ __forceinline__ void push_slots(const Geom& g, const Pop<float>& P, const Push32Const& pc,
                                           const Push32Const& sp, PipeStage& st, int base, int2 desc, int slice,
                                           uint32_t& nmig, uint32_t& nrem) {
    constexpr bool kStep = (kF & kPipeStep) != 0, kDep = (kF & kPipeDeposit) != 0;
    constexpr int kPer = 4;
    const int lane = threadIdx.x & 31, tid = slice * 32 + lane;
    const int c0 = desc.x, nc = desc.y;
    const int64_t* S = st.start + (c0 & 1);  // S[i] = start[c0 + i]
    const int32_t* N = st.count + (c0 & 3);  // N[i] = count[c0 + i]
    const int s0 = base + tid * kPer;
    int lc = 0;
    {
        int lo = 0, hi = nc - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (S[mid] <= s0) lo = mid; else hi = mid - 1;
        }
        lc = lo;
    }
    const int cell = c0 + lc;
    const int cstart = (int)S[lc];
    int nv = 0;
    if (s0 < P.capacity) {
        const int e = cstart + N[lc] - s0;
        nv = e <= 0 ? 0 : (e >= kPer ? kPer : e);
    }
    const CellInfo ci = cell_info(g, pc, cell);
    const int sl0 = tid * kPer;
    int nst = nv;  // this thread's stayers
    if (kStep) {
        const float* coef = g.cellcoef + (size_t)cell * 48;
        // lane groups start at different slots of their run of 4: the words a
        // warp reads in one step fall in 32 different banks
        const int rot = lane >> 3;
#pragma unroll 1
        for (int jj = 0; jj < kPer; ++jj) {
            const int j = (jj + rot) & (kPer - 1);
            const int sl = sl0 + j;
            PState<float> p;
            int outcome = -1, dir = 0;
            if (j < nv) {
                p = load_slot(st, sl);
                outcome = step32f<false, (kF & kPipeGather) != 0, (kF & kPipeDipole) != 0>(g, pc, sp, coef, ci, p,
                                                                                           dir);
                if (outcome == kStay) store_slot(st, sl, p);
                else if (kDep) clear_slot(st, sl);
            }
            if (outcome > 0) --nst;
            leave_and_hole<false>(g, P, pc, outcome, dir, p, base + sl, cell, cstart, kDep, nmig, nrem);
        }
        __syncwarp();
    }
    if (!kDep) return;
    float acc[32];
#pragma unroll
    for (int l = 0; l < 32; ++l) acc[l] = 0.f;
#pragma unroll 1
    for (int j = 0; j < nv; ++j) add_moments(acc, load_slot(st, sl0 + j));
    const unsigned todo = __ballot_sync(0xffffffffu, nst > 0);
    const int prev_cell = __shfl_up_sync(0xffffffffu, cell, 1);
    unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev_cell != cell);
    while (heads) {
        const int ra = __ffs(heads) - 1;
        heads &= heads - 1;
        const int rb = heads ? __ffs(heads) - 1 : 32;  // run [ra, rb)
        const unsigned run = (rb < 32 ? (1u << rb) : 0u) - (1u << ra);
        if (!(todo & run)) continue;
        const bool mine = ((run >> lane) & 1u) != 0;
        float s = run_transpose_sum(acc, mine);
        const int cnt = __reduce_add_sync(0xffffffffu, mine ? nst : 0);
        if (lane == 24) s = (float)cnt;
        const int3 c = cell_xyz(g, pc, __shfl_sync(0xffffffffu, cell, ra));
        emit_corner_sums(g, s, c.x, c.y, c.z, P.q);
    }
}

// Item mode: where the stage's tile descriptors live, and the phase of the
// stage's `ready` barrier that this use of the stage completes.
struct TileDescs {
    CellDesc* cells;
    uint8_t* item_cell;
    int* total;
    int* claim;
    uint64_t* ready;
    uint32_t parity;
    const volatile int* abort;
    uint32_t polls;
};

// The item-mode descriptors of the tile, by the warp with lane i describing
// cell c0 + i; the tile's items into *total.
__device__ __forceinline__ void write_cell_descs(const Geom& g, const Push32Const& pc, const PipeStage& st,
                                                 int base, int c0, int nc, int sh, CellDesc* cells,
                                                 uint8_t* item_cell, int* total) {
    const int lane = threadIdx.x & 31;
    const int64_t* S = st.start + (c0 & 1);
    const int32_t* N = st.count + (c0 & 3);
    int lo = 0, hi = 0, cst = 0;
    if (lane < nc) {
        cst = (int)S[lane];
        const int l = cst - base, h = cst + N[lane] - base;
        lo = l < 0 ? 0 : l;
        hi = h > kTileSlots ? kTileSlots : h;
    }
    const int items = hi > lo ? (hi - lo + (1 << sh) - 1) >> sh : 0;
    int incl = items;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    CellDesc d;
    d.lo = lo;
    d.hi = items > 0 ? hi : lo;  // cells with no slots here own no item
    d.excl = incl - items;
    d.cst = cst;
    const int cell = c0 + (lane < nc ? lane : 0);
    d.ci = cell_info(g, pc, cell);
    const int3 cx = cell_xyz(g, pc, cell);
    d.node0 = node_index(g, cx.x, cx.y, cx.z);
    d.unused = 0;
    cells[lane] = d;
    for (int k = 0; k < items; ++k) item_cell[d.excl + k] = (uint8_t)lane;
    if (lane == 31) *total = incl;
}

// One compute warp's share of the tile in `st`; false if a wait expired.
template <int kF>
__device__ __forceinline__ bool push_tile_warp(const Geom& g, const Pop<float>& P, const Push32Const& pc,
                                               const Push32Const& sp, int tile,
                                               int2 desc, const PushShape& shp, PipeStage& st, int* next_item,
                                               const TileDescs& td, uint32_t& nmig, uint32_t& nrem) {
    const int lane = threadIdx.x & 31;
    const int base = tile * kTileSlots;
    const int c0 = desc.x, nc = desc.y;
    // the first warp to reach the tile completes the phase of `ready` that
    // belongs to this use of the stage (in item mode after writing the cells'
    // descriptors, lane i: cell c0 + i); the others wait for it there
    int first = 0;
    if (lane == 0) first = atomicAdd(td.claim, 1) == 0;
    first = __shfl_sync(0xffffffffu, first, 0);
    if (nc > shp.item_cells) {
        if (first && lane == 0) mbar_arrive(td.ready);
        for (int w = threadIdx.x >> 5; w < kSlotWarps; w += kComputeWarps)
            push_slots<kF>(g, P, pc, sp, st, base, desc, w, nmig, nrem);
        return true;
    }
    const int sh = 31 - __clz(shp.item);  // items of 2^sh particles
    if (first) {
        write_cell_descs(g, pc, st, base, c0, nc, sh, td.cells, td.item_cell, td.total);
        __syncwarp();
        if (lane == 0) mbar_arrive(td.ready);
    } else if (!__all_sync(0xffffffffu, mbar_wait(td.ready, td.parity, td.abort, td.polls))) {
        return false;
    }
    const int total = *td.total;
    for (;;) {
        int j = 0;
        if (lane == 0) j = atomicAdd(next_item, 1);
        j = __shfl_sync(0xffffffffu, j, 0);
        if (j >= total) break;
        const int src = td.item_cell[j];
        const CellDesc d = td.cells[src];
        const int a = d.lo + ((j - d.excl) << sh);
        const int b = a + (1 << sh) < d.hi ? a + (1 << sh) : d.hi;
        push_item<kF>(g, P, pc, sp, st, st.coef + src * 48, d.ci, base, c0 + src, d.node0, d.cst, a, b, nmig, nrem);
    }
    return true;
}

// Tile t of a launch over several populations: population i holds tiles
// [first[i], first[i + 1]).
struct TileMap {
    int first[kSetPops + 1];
    int n;  // populations
};

__device__ __forceinline__ int tile_pop(const TileMap& tm, int t) {
    int i = 0;
    while (i + 1 < tm.n && t >= tm.first[i + 1]) ++i;
    return i;
}

// Adds a compute warp's migration / removal counts to population counters.
__device__ __forceinline__ void flush_counts(StepCounters* ctr, uint32_t& nmig, uint32_t& nrem) {
    const uint32_t m = __reduce_add_sync(0xffffffffu, nmig), r = __reduce_add_sync(0xffffffffu, nrem);
    if ((threadIdx.x & 31) == 0) {
        if (m) atomicAdd(&ctr->migrated, m);
        if (r) atomicAdd(&ctr->removed, r);
    }
    nmig = nrem = 0;
}

// The persistent kernel: CTA b pushes tiles b, b + G, b + 2G, ... (G =
// gridDim.x) of the populations of S, numbered through tm, with kStages
// shared-memory stages in flight; `shp` splits the tiles into work.
template <int kStages, int kMinBlocks, int kF>
__global__ void __launch_bounds__(kPipeThreads, kMinBlocks)
    k_push32_pipe(Geom g, const __grid_constant__ PopSet<float> S, const __grid_constant__ Push32Set pcs,
                  const __grid_constant__ TileMap tm, PushShape shp) {
    constexpr bool kStep = (kF & kPipeStep) != 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    PipeSmem<kStages>& sm = *reinterpret_cast<PipeSmem<kStages>*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int G = gridDim.x;
    const int ntiles = tm.first[tm.n];
    const uint32_t polls = shp.wait_polls < 0 ? kMaxPolls : (uint32_t)shp.wait_polls;
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&sm.full[s], 1);
            mbar_init(&sm.empty[s], kComputeWarps);
            mbar_init(&sm.ready[s], 1);
        }
        sm.abort = 0;
        fence_mbar_init();
    }
    __syncthreads();
    const volatile int* abort = &sm.abort;

    if (warp == kComputeWarps) {
        // ---- producer ----
        if (lane != 0) return;
        const float* coef = (kF & kPipeGather) ? g.cellcoef : nullptr;
        auto load_desc = [&](int t) {
            const int pi = tile_pop(tm, t);
            return __ldg(S.p[pi].cta_cells + (t - tm.first[pi]));
        };
        // wait_store: bulk stores of the stage's previous tile are in flight;
        // the slot arrays are loaded once they have read them
        auto issue = [&](int t, int s, int2 d, bool wait_store) {
            const int pi = tile_pop(tm, t);
            sm.desc[s] = d;
            sm.pop[s] = pi;
            sm.next_item[s] = 0;
            sm.claim[s] = 0;
            issue_tile_tables(S.p[pi], coef, t - tm.first[pi], d, shp.item_cells, sm.stage[s], &sm.full[s]);
            if (wait_store) bulk_wait_read_all();
            issue_tile_slots(S.p[pi], t - tm.first[pi], d, sm.stage[s], &sm.full[s]);
        };
        int issued = 0;  // tiles of this CTA whose copies were issued
        for (int s = 0; s < kStages; ++s) {
            const int t = blockIdx.x + s * G;
            if (t >= ntiles) break;
            issue(t, s, load_desc(t), false);
            ++issued;
        }
        int2 next_desc = make_int2(0, 0);
        if (blockIdx.x + kStages * G < ntiles) next_desc = load_desc(blockIdx.x + kStages * G);
        bool failed = false;
        int k = 0;
        for (int t = blockIdx.x; t < ntiles; t += G, ++k) {
            const int s = k % kStages;
            if (!mbar_wait(&sm.empty[s], (uint32_t)(k / kStages) & 1u, abort, polls)) {
                failed = true;
                break;
            }
            // the pushed tile goes back from the stage (stayers in place; the
            // slots of leavers and drops are holes)
            const bool store = kStep;
            if (store) {
                const Pop<float>& P = S.p[sm.pop[s]];
                const TileCopy c = tile_copy(P, t - tm.first[sm.pop[s]], sm.desc[s]);
                float* const arr[6] = {P.x, P.y, P.z, P.u, P.v, P.w};
#pragma unroll
                for (int a = 0; a < 6; ++a) bulk_store(arr[a] + c.base, sm.stage[s].s[a], c.slot_bytes);
                bulk_commit();
            }
            const int tn = t + kStages * G;
            if (tn < ntiles) {
                const int2 d = next_desc;
                if (tn + G < ntiles) next_desc = load_desc(tn + G);
                issue(tn, s, d, store);
                ++issued;
            }
        }
        if (failed) {
            if (atomicExch(&sm.abort, 1) == 0) atomicAdd(&S.p[0].ctr->timeouts, 1u);
            // copies still in flight land before the CTA leaves
            const int never = 0;
            for (int kk = k; kk < issued; ++kk)
                mbar_wait(&sm.full[kk % kStages], (uint32_t)(kk / kStages) & 1u, &never);
        }
        bulk_wait_all();
        return;
    }

    // ---- compute warps ----
    uint32_t nmig = 0, nrem = 0;
    int cur = -1;  // population of the counts held
    int k = 0;
    for (int t = blockIdx.x; t < ntiles; t += G, ++k) {
        const int s = k % kStages;
        // warp-uniform: every lane polls the same barrier
        if (!__all_sync(0xffffffffu, mbar_wait(&sm.full[s], (uint32_t)(k / kStages) & 1u, abort, polls))) {
            if (lane == 0 && atomicExch(&sm.abort, 1) == 0) atomicAdd(&S.p[0].ctr->timeouts, 1u);
            break;
        }
        const int pi = sm.pop[s];
        if (pi != cur) {
            if (cur >= 0) flush_counts(S.p[cur].ctr, nmig, nrem);
            cur = pi;
        }
        // constants other than the species' are the same for every
        // population of the launch: population 0's, at fixed offsets
        const TileDescs td{sm.cells[s], sm.item_cell[s], &sm.total[s], &sm.claim[s], &sm.ready[s],
                           (uint32_t)(k / kStages) & 1u, abort, polls};
        if (!push_tile_warp<kF>(g, S.p[pi], pcs.c[0], pcs.c[pi], t - tm.first[pi], sm.desc[s], shp, sm.stage[s],
                                &sm.next_item[s], td, nmig, nrem)) {
            if (lane == 0 && atomicExch(&sm.abort, 1) == 0) atomicAdd(&S.p[0].ctr->timeouts, 1u);
            break;
        }
        fence_proxy_async_smem();  // this warp's writes to the stage, before the bulk stores read it
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.empty[s]);
    }
    if (cur >= 0) flush_counts(S.p[cur].ctr, nmig, nrem);
}

// The batched form: tiles of many universes' populations in one launch.
// Global tile t is tile cta_job[t].y of job cta_job[t].x; the producer also
// bulk-copies the job record (geometry, population, push constants) into the
// stage, and the compute warps read everything about the tile from there.
template <int kStages, int kMinBlocks, int kF>
__global__ void __launch_bounds__(kPipeThreads, kMinBlocks)
    k_push32_pipe_jobs(const PopJob<float>* __restrict__ jobs, const int2* __restrict__ cta_job, int ntiles,
                       PushShape shp) {
    constexpr bool kStep = (kF & kPipeStep) != 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    PipeSmem<kStages>& sm = *reinterpret_cast<PipeSmem<kStages>*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int G = gridDim.x;
    const uint32_t polls = shp.wait_polls < 0 ? kMaxPolls : (uint32_t)shp.wait_polls;
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&sm.full[s], 1);
            mbar_init(&sm.empty[s], kComputeWarps);
            mbar_init(&sm.ready[s], 1);
        }
        sm.abort = 0;
        fence_mbar_init();
    }
    __syncthreads();
    const volatile int* abort = &sm.abort;

    if (warp == kComputeWarps) {
        // ---- producer ----
        if (lane != 0) return;
        auto issue = [&](int t, int s, bool wait_store) {
            const int2 cj = __ldg(cta_job + t);
            const PopJob<float>* J = jobs + cj.x;
            const Pop<float> P = J->P;
            const float* coef = (kF & kPipeGather) ? J->g.cellcoef : nullptr;
            const int2 d = __ldg(P.cta_cells + cj.y);
            sm.desc[s] = d;
            sm.pop[s] = cj.x;
            sm.ltile[s] = cj.y;
            sm.next_item[s] = 0;
            sm.claim[s] = 0;
            issue_tile_tables(P, coef, cj.y, d, shp.item_cells, sm.stage[s], &sm.full[s],
                              (uint32_t)sizeof(PopJob<float>));
            bulk_load(&sm.stage[s].job, J, (uint32_t)sizeof(PopJob<float>), &sm.full[s]);
            if (wait_store) bulk_wait_read_all();
            issue_tile_slots(P, cj.y, d, sm.stage[s], &sm.full[s]);
        };
        int issued = 0;
        for (int s = 0; s < kStages; ++s) {
            const int t = blockIdx.x + s * G;
            if (t >= ntiles) break;
            issue(t, s, false);
            ++issued;
        }
        bool failed = false;
        int k = 0;
        for (int t = blockIdx.x; t < ntiles; t += G, ++k) {
            const int s = k % kStages;
            if (!mbar_wait(&sm.empty[s], (uint32_t)(k / kStages) & 1u, abort, polls)) {
                failed = true;
                break;
            }
            const bool store = kStep;
            if (store) {
                const Pop<float>& P = sm.stage[s].job.P;
                const TileCopy c = tile_copy(P, sm.ltile[s], sm.desc[s]);
                float* const arr[6] = {P.x, P.y, P.z, P.u, P.v, P.w};
#pragma unroll
                for (int a = 0; a < 6; ++a) bulk_store(arr[a] + c.base, sm.stage[s].s[a], c.slot_bytes);
                bulk_commit();
            }
            const int tn = t + kStages * G;
            if (tn < ntiles) {
                issue(tn, s, store);
                ++issued;
            }
        }
        if (failed) {
            if (atomicExch(&sm.abort, 1) == 0) atomicAdd(&jobs[0].P.ctr->timeouts, 1u);
            const int never = 0;
            for (int kk = k; kk < issued; ++kk)
                mbar_wait(&sm.full[kk % kStages], (uint32_t)(kk / kStages) & 1u, &never);
        }
        bulk_wait_all();
        return;
    }

    // ---- compute warps ----
    uint32_t nmig = 0, nrem = 0;
    StepCounters* cur = nullptr;  // counters of the job whose counts are held
    int k = 0;
    for (int t = blockIdx.x; t < ntiles; t += G, ++k) {
        const int s = k % kStages;
        if (!__all_sync(0xffffffffu, mbar_wait(&sm.full[s], (uint32_t)(k / kStages) & 1u, abort, polls))) {
            if (lane == 0 && atomicExch(&sm.abort, 1) == 0) atomicAdd(&jobs[0].P.ctr->timeouts, 1u);
            break;
        }
        const PopJob<float>& J = sm.stage[s].job;
        if (J.P.ctr != cur) {
            if (cur) flush_counts(cur, nmig, nrem);
            cur = J.P.ctr;
        }
        const TileDescs td{sm.cells[s], sm.item_cell[s], &sm.total[s], &sm.claim[s], &sm.ready[s],
                           (uint32_t)(k / kStages) & 1u, abort, polls};
        if (!push_tile_warp<kF>(J.g, J.P, J.pc, J.pc, sm.ltile[s], sm.desc[s], shp, sm.stage[s], &sm.next_item[s],
                                td, nmig, nrem)) {
            if (lane == 0 && atomicExch(&sm.abort, 1) == 0) atomicAdd(&jobs[0].P.ctr->timeouts, 1u);
            break;
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.empty[s]);
    }
    if (cur) flush_counts(cur, nmig, nrem);
}

}  // namespace ipg
