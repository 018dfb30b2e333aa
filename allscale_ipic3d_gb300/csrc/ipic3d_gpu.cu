// Host side of the GB300 particle path: the C ABI of include/ipic3d_gpu.h.
//
// A context holds one Universe (universe.h:12-51) on the current GPU and runs
// simulateSteps (simulator.h:127-242) as a fixed sequence of kernels per step:
//   [project once if J is stale] -> ghost faces -> field solver -> push
//   (mover + export + deposit) -> pending push -> injection -> place (import)
//   -> J finalize.
// Particles are split into populations of equal (q, qom) -- the species of
// the reference's distributions (cell.h:104-133) -- so the hot kernel reads
// neither q nor qom per particle.
#include <algorithm>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/ipic3d_gpu.h"
#include "autotune.h"
#include "launch.h"
#include "upload.h"

namespace ipg {
namespace {

thread_local int g_last_status = IPIC3D_OK;
thread_local char g_last_msg[512] = "";

int fail(int status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_msg, sizeof(g_last_msg), fmt, ap);
    va_end(ap);
    g_last_status = status;
    return status;
}

}  // namespace

int set_last_error(int status, const char* msg) { return fail(status, "%s", msg); }

namespace {

#define CU(call)                                                                                              \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess)                                                                                \
            return fail(e_ == cudaErrorMemoryAllocation ? IPIC3D_E_NOMEM : IPIC3D_E_CUDA, "%s:%d %s: %s",      \
                        __FILE__, __LINE__, #call, cudaGetErrorString(e_));                                   \
    } while (0)

template <typename X>
void dfree(X*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

template <typename T>
struct PopStore {
    double q = 0, qom = 0;
    int64_t capacity = 0;
    uint32_t pending_cap = 0, outbox_cap = 0;
    T *x = nullptr, *y = nullptr, *z = nullptr, *u = nullptr, *v = nullptr, *w = nullptr;
    uint32_t* id = nullptr;
    int64_t* start = nullptr;
    int2* cta_cells = nullptr;
    int32_t *count = nullptr, *hole_cnt = nullptr, *arr_cnt = nullptr;
    int32_t *hole_list = nullptr, *arr_list = nullptr, *sort_tmp = nullptr;
    int32_t *dirty_flag = nullptr, *dirty_list = nullptr;
    Mover<T>*outbox = nullptr, *pending_in = nullptr, *pending_out = nullptr;
    uint32_t* pending_in_count = nullptr;
    StepCounters* ctr = nullptr;
    std::vector<int64_t> h_start;  // host copy of start[]

    void release() {
        dfree(x); dfree(y); dfree(z); dfree(u); dfree(v); dfree(w); dfree(id);
        dfree(start); dfree(cta_cells); dfree(count); dfree(hole_cnt); dfree(arr_cnt);
        dfree(hole_list); dfree(arr_list); dfree(sort_tmp); dfree(dirty_flag); dfree(dirty_list);
        dfree(outbox); dfree(pending_in); dfree(pending_out);
        dfree(pending_in_count); dfree(ctr);
        capacity = 0;
    }
    Pop<T> view() const {
        Pop<T> P;
        P.x = x; P.y = y; P.z = z; P.u = u; P.v = v; P.w = w;
        P.id = id;
        P.start = start;
        P.cta_cells = cta_cells;
        P.count = count;
        P.hole_cnt = hole_cnt;
        P.hole_list = hole_list;
        P.arr_cnt = arr_cnt;
        P.arr_list = arr_list;
        P.dirty_flag = dirty_flag;
        P.dirty_list = dirty_list;
        P.outbox = outbox;
        P.outbox_cap = outbox_cap;
        P.pending_in = pending_in;
        P.pending_out = pending_out;
        P.pending_cap = pending_cap;
        P.pending_in_count = pending_in_count;
        P.ctr = ctr;
        P.capacity = capacity;
        P.q = q;
        P.qom = qom;
        P.pad[0] = P.pad[1] = 0;
        return P;
    }
};

}  // namespace
}  // namespace ipg

namespace ipg {
constexpr int kMaxPops = 16;

// The populations in launch sets of up to kSetPops.
template <typename T>
std::vector<PopSet<T>> pop_sets(std::vector<PopStore<T>>& pops) {
    std::vector<PopSet<T>> out;
    for (size_t i = 0; i < pops.size(); i += kSetPops) {
        PopSet<T> S{};
        S.n = (int)std::min<size_t>(kSetPops, pops.size() - i);
        for (int k = 0; k < S.n; ++k) {
            S.p[k] = pops[i + k].view();
            S.sort_tmp[k] = pops[i + k].sort_tmp;
            S.pend_count[k] = pops[i + k].pending_in_count;
        }
        out.push_back(S);
    }
    return out;
}
// Advances the device step counter (keys the injection generator).
__global__ void k_step_end(uint64_t* step) { *step += 1; }
}  // namespace ipg

using namespace ipg;

struct ipic3d_ctx {
    ipic3d_props props;
    ipic3d_config cfg;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = true;  // false: the stream of the batch that owns this context
    bool lent = false;       // a universe of a batch (destroyed with the batch)
    bool fp32 = false;
    Geom g{};
    double *field = nullptr, *bcfield = nullptr, *J = nullptr, *rho = nullptr;
    float4* node32 = nullptr;
    float* cellcoef = nullptr;  // FP32 field-gather mover: per-cell polynomial
    uint64_t* d_step = nullptr;
    double *d_partial = nullptr, *d_result = nullptr;
    std::vector<PopStore<float>> p32;
    std::vector<PopStore<double>> p64;
    bool j_valid = false;
    uint64_t steps = 0, launches = 0, rebuilds = 0;
    uint64_t pending_last = 0, relayout_steps = 0;
    StepCounters last{};
    // step graphs (StepKind): the whole step, or, in a run of steps with a
    // field solver, the first solve alone, then the moves with the next
    // step's solve beside the placement, the last move without it
    cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
    uint64_t graph_kernels[4] = {0, 0, 0, 0};  // kernels one replay runs
    // pending-list watch: per step an async copy of the pending counts into
    // pinned memory, read one step later (ring of two)
    uint32_t* h_pending = nullptr;  // [2][kMaxPops]
    // after a run of steps: every population's counters and pending count,
    // copied in one go (pinned)
    StepCounters* h_ctr = nullptr;  // [kMaxPops]
    uint32_t* h_pin = nullptr;      // [kMaxPops]
    cudaEvent_t pend_ev[2] = {nullptr, nullptr};
    uint64_t particles_hint = 0;
    // species table of the populations (index = population) and the device
    // staging buffers of the upload path
    std::vector<std::pair<double, double>> species;
    void* st_parts = nullptr;
    size_t st_parts_cap = 0;
    uint32_t* st_ids = nullptr;
    size_t st_ids_cap = 0;
    uint8_t* st_sid = nullptr;
    size_t st_sid_cap = 0;
    int64_t* st_off = nullptr;
    size_t st_off_cap = 0;
    int32_t* st_cnt = nullptr;
    size_t st_cnt_cap = 0;
    int* st_unknown = nullptr;
    int* st_flags = nullptr;            // fused upload: unknown species, cell overflow
    int64_t* st_dst = nullptr;          // download: output index of each (population, cell)
    size_t st_dst_cap = 0;
    // the download's own staging buffers, copy stream and completion state
    // (an asynchronous download's copies may run while the next upload's do)
    void* st_dl = nullptr;
    size_t st_dl_cap = 0;
    uint32_t* st_dl_ids = nullptr;
    size_t st_dl_ids_cap = 0;
    cudaStream_t dl_stream = nullptr;
    cudaEvent_t dl_ev = nullptr;
    struct DlFill {                     // a waiting particle, written after the copies
        int64_t at;
        ipic3d_particle rec;
        uint32_t id;
    };
    std::vector<DlFill> dl_fill;
    ipic3d_particle* dl_parts = nullptr;
    uint32_t* dl_ids = nullptr;
    double* dl_xyz = nullptr;
    bool dl_busy = false;
    cudaStream_t copy_stream = nullptr; // copies of the chunked upload and download
    cudaEvent_t copy_ev = nullptr;
    // second stream of a step: kernels that run beside the push / placement
    cudaStream_t aux_stream = nullptr;
    // fork, join (push), fork, join (placement), the next step's E update done
    cudaEvent_t aux_ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // per-phase event timing
    bool profiling = false;
    cudaEvent_t ph_ev[IPIC3D_PHASE_COUNT][2] = {};
    bool ph_open[IPIC3D_PHASE_COUNT] = {};
    ipic3d_profile prof{};
    uint64_t push_particles = 0;
    // launch shape of the FP32 push: autotuned (config block_size 0) unless
    // fixed by ipic3d_gpu_set_push_shape
    PushTuner tuner;
    bool shape_fixed = false;
    int32_t wait_polls = -1;       // bounded-wait polls of the FP32 push (< 0: default)
    uint64_t tuned_particles = 0;  // particle count the shape was tuned for
    bool tune_timing = false;      // this step is a trial: time the push
    cudaEvent_t tune_ev[2] = {nullptr, nullptr};

    int npops() const { return fp32 ? (int)p32.size() : (int)p64.size(); }
    int64_t nfield() const { return (props.size[0] + 3) * (props.size[1] + 3) * (props.size[2] + 3); }
    int64_t nbc() const { return (props.size[0] + 2) * (props.size[1] + 2) * (props.size[2] + 2); }
    int64_t nnode() const { return (props.size[0] + 1) * (props.size[1] + 1) * (props.size[2] + 1); }
    int64_t ncells() const { return props.size[0] * props.size[1] * props.size[2]; }
};

namespace {

void drop_graph(ipic3d_ctx* ctx) {
    for (auto& gr : ctx->graph) {
        if (gr) cudaGraphExecDestroy(gr);
        gr = nullptr;
    }
}

// What one replay of a step graph does.
enum StepKind : int {
    kStepFull = 0,       // field solve, then the move
    kStepSolve = 1,      // the field solve alone (first step of a run)
    kStepMoveSolve = 2,  // the move, the next step's solve beside its placement
    kStepMove = 3,       // the move alone (last step of a run)
};

void release_pops(ipic3d_ctx* ctx) {
    for (auto& p : ctx->p32) p.release();
    for (auto& p : ctx->p64) p.release();
    ctx->p32.clear();
    ctx->p64.clear();
}

// Slots reserved for a cell holding n particles: n plus the slack, rounded up
// to a multiple of kSlotAlign (a push thread's slots), at least kSlotAlign. The slack is the largest
// of slack_min, slack * n and 2 sqrt(n): a thermal plasma that starts with
// equal counts per cell relaxes to Poisson counts (standard deviation
// sqrt(n)), and two deviations keep all but a few percent of the cells
// inside their slots, so few arrivals wait in the pending list.
int64_t cell_capacity(const ipic3d_config& cfg, uint64_t n) {
    double slack = cfg.slack > 0 ? cfg.slack : 0.125;
    int64_t smin = cfg.slack_min > 0 ? cfg.slack_min : 8;
    int64_t extra = std::max<int64_t>(smin, (int64_t)std::ceil(slack * (double)n));
    extra = std::max<int64_t>(extra, (int64_t)std::ceil(2.0 * std::sqrt((double)n)));
    int64_t cap = (int64_t)n + extra;
    cap = (cap + kSlotAlign - 1) & ~int64_t(kSlotAlign - 1);
    return std::max<int64_t>(cap, kSlotAlign);
}

template <typename T>
int alloc_pop(ipic3d_ctx* ctx, PopStore<T>& P, const std::vector<uint64_t>& counts, int64_t extra_pending) {
    const int64_t nc = ctx->ncells();
    P.h_start.assign(nc + 1, 0);
    for (int64_t c = 0; c < nc; ++c) P.h_start[c + 1] = P.h_start[c] + cell_capacity(ctx->cfg, counts[c]);
    P.capacity = P.h_start[nc];
    // every particle can wait at most once per step: capacity entries suffice
    P.pending_cap = (uint32_t)std::min<int64_t>(std::max<int64_t>(1 << 12, P.capacity), 0x7fffffff);
    int64_t inject_cap = 0;
    if (ctx->cfg.flags & IPIC3D_F_INJECT_LOW_X)
        inject_cap = (int64_t)(ctx->props.size[1] * ctx->props.size[2]) * ((int64_t)ctx->cfg.inject_per_cell + 1);
    const int64_t ob = P.capacity + P.pending_cap + inject_cap + extra_pending;
    if (ob > 0x7fffffff) return fail(IPIC3D_E_CAPACITY, "population too large for 32-bit outbox indices");
    P.outbox_cap = (uint32_t)ob;
    const size_t cap = (size_t)P.capacity;
    CU(cudaMalloc(&P.x, cap * sizeof(T)));
    CU(cudaMalloc(&P.y, cap * sizeof(T)));
    CU(cudaMalloc(&P.z, cap * sizeof(T)));
    CU(cudaMalloc(&P.u, cap * sizeof(T)));
    CU(cudaMalloc(&P.v, cap * sizeof(T)));
    CU(cudaMalloc(&P.w, cap * sizeof(T)));
    if (ctx->cfg.flags & IPIC3D_F_TRACK_IDS) CU(cudaMalloc(&P.id, cap * sizeof(uint32_t)));
    // padded: the FP32 push bulk-copies aligned slices of start[] / count[]
    // that may reach up to 3 entries past the last cell
    CU(cudaMalloc(&P.start, (nc + 4) * sizeof(int64_t)));
    CU(cudaMalloc(&P.count, (nc + 4) * sizeof(int32_t)));
    CU(cudaMemsetAsync(P.start, 0, (nc + 4) * sizeof(int64_t), ctx->stream));
    CU(cudaMemsetAsync(P.count, 0, (nc + 4) * sizeof(int32_t), ctx->stream));
    CU(cudaMalloc(&P.hole_cnt, nc * sizeof(int32_t)));
    CU(cudaMalloc(&P.arr_cnt, nc * sizeof(int32_t)));
    CU(cudaMalloc(&P.hole_list, cap * sizeof(int32_t)));
    CU(cudaMalloc(&P.arr_list, cap * sizeof(int32_t)));
    CU(cudaMalloc(&P.sort_tmp, cap * sizeof(int32_t)));
    CU(cudaMalloc(&P.dirty_flag, nc * sizeof(int32_t)));
    CU(cudaMalloc(&P.dirty_list, nc * sizeof(int32_t)));
    CU(cudaMemsetAsync(P.dirty_flag, 0, nc * sizeof(int32_t), ctx->stream));
    CU(cudaMalloc(&P.outbox, (size_t)P.outbox_cap * sizeof(Mover<T>)));
    CU(cudaMalloc(&P.pending_in, (size_t)P.pending_cap * sizeof(Mover<T>)));
    CU(cudaMalloc(&P.pending_out, (size_t)P.pending_cap * sizeof(Mover<T>)));
    CU(cudaMalloc(&P.pending_in_count, sizeof(uint32_t)));
    CU(cudaMalloc(&P.ctr, sizeof(StepCounters)));
    CU(cudaMemsetAsync(P.hole_cnt, 0, nc * sizeof(int32_t), ctx->stream));
    CU(cudaMemsetAsync(P.arr_cnt, 0, nc * sizeof(int32_t), ctx->stream));
    CU(cudaMemsetAsync(P.pending_in_count, 0, sizeof(uint32_t), ctx->stream));
    CU(cudaMemsetAsync(P.ctr, 0, sizeof(StepCounters), ctx->stream));
    CU(cudaMemcpyAsync(P.start, P.h_start.data(), (nc + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    // push CTA b covers slots [b*kSlotsPerCta, (b+1)*kSlotsPerCta): its cells
    const int64_t nb = (P.capacity + kSlotsPerCta - 1) / kSlotsPerCta;
    std::vector<int2> cc((size_t)std::max<int64_t>(nb, 1));
    int64_t c = 0;
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t first = b * kSlotsPerCta, last = std::min(first + kSlotsPerCta, P.capacity) - 1;
        while (P.h_start[c + 1] <= first) ++c;
        int64_t e = c;
        while (P.h_start[e + 1] <= last) ++e;
        cc[b] = make_int2((int)c, (int)(e - c + 1));
        if (e - c + 1 > kMaxCellsPerCta) return fail(IPIC3D_E_INVALID, "layout: a push CTA spans too many cells");
    }
    CU(cudaMalloc(&P.cta_cells, cc.size() * sizeof(int2)));
    CU(cudaMemcpyAsync(P.cta_cells, cc.data(), cc.size() * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));  // cc and h_start copies complete
    return IPIC3D_OK;
}

// Copies one population's particles (input indices `order`, grouped by cell
// with per-cell `counts`) into the slot layout. FP32 stores the position
// relative to the cell origin in cell widths.
template <typename T>
int fill_pop(ipic3d_ctx* ctx, PopStore<T>& P, const ipic3d_particle* parts, const uint32_t* ids,
             const std::vector<int64_t>& order, const std::vector<uint64_t>& counts,
             const std::vector<int64_t>& cell_of) {
    const int64_t nc = ctx->ncells();
    const size_t cap = (size_t)P.capacity;
    std::vector<T> hx(cap, T(0)), hy(cap, T(0)), hz(cap, T(0)), hu(cap, T(0)), hv(cap, T(0)), hw(cap, T(0));
    std::vector<uint32_t> hid(P.id ? cap : 0, 0);
    std::vector<int32_t> hcount(nc);
    const ipic3d_props& pr = ctx->props;
    int64_t k = 0;
    for (int64_t c = 0; c < nc; ++c) {
        hcount[c] = (int32_t)counts[c];
        int64_t cx = c / (pr.size[1] * pr.size[2]), cy = (c / pr.size[2]) % pr.size[1], cz = c % pr.size[2];
        for (uint64_t i = 0; i < counts[c]; ++i, ++k) {
            const int64_t src = order[k];
            const ipic3d_particle& p = parts[src];
            const size_t s = (size_t)(P.h_start[c] + (int64_t)i);
            (void)cell_of;
            if (std::is_same<T, float>::value) {
                double ox = pr.origin[0] + (double)cx * pr.cell_width[0];
                double oy = pr.origin[1] + (double)cy * pr.cell_width[1];
                double oz = pr.origin[2] + (double)cz * pr.cell_width[2];
                hx[s] = (T)((p.position[0] - ox) / pr.cell_width[0]);
                hy[s] = (T)((p.position[1] - oy) / pr.cell_width[1]);
                hz[s] = (T)((p.position[2] - oz) / pr.cell_width[2]);
            } else {
                hx[s] = (T)p.position[0];
                hy[s] = (T)p.position[1];
                hz[s] = (T)p.position[2];
            }
            hu[s] = (T)p.velocity[0];
            hv[s] = (T)p.velocity[1];
            hw[s] = (T)p.velocity[2];
            if (P.id) hid[s] = ids ? ids[src] : (uint32_t)src;
        }
    }
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(P.x, hx.data(), cap * sizeof(T), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P.y, hy.data(), cap * sizeof(T), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P.z, hz.data(), cap * sizeof(T), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P.u, hu.data(), cap * sizeof(T), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P.v, hv.data(), cap * sizeof(T), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P.w, hw.data(), cap * sizeof(T), cudaMemcpyHostToDevice, st));
    if (P.id) CU(cudaMemcpyAsync(P.id, hid.data(), cap * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P.count, hcount.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    CU(cudaStreamSynchronize(st));  // host staging buffers die here
    return IPIC3D_OK;
}

struct Species {
    double q, qom;
};

// Splits the input into species (exact (q, qom) equality) and uploads.
int upload_impl(ipic3d_ctx* ctx, const ipic3d_particle* parts, const uint64_t* cell_counts, const uint32_t* ids) {
    const int64_t nc = ctx->ncells();
    uint64_t n = 0;
    for (int64_t c = 0; c < nc; ++c) n += cell_counts[c];
    if (n > 0 && !parts) return fail(IPIC3D_E_INVALID, "particles == NULL with %llu particles", (unsigned long long)n);
    std::vector<Species> sp;
    std::vector<uint8_t> sid(n);
    if (ctx->cfg.flags & IPIC3D_F_INJECT_LOW_X) sp.push_back({ctx->cfg.inject_q, ctx->cfg.inject_qom});
    for (uint64_t i = 0; i < n; ++i) {
        size_t k = 0;
        for (; k < sp.size(); ++k)
            if (sp[k].q == parts[i].q && sp[k].qom == parts[i].qom) break;
        if (k == sp.size()) {
            if (sp.size() >= 16) return fail(IPIC3D_E_INVALID, "more than 16 distinct (q, qom) species");
            sp.push_back({parts[i].q, parts[i].qom});
        }
        sid[i] = (uint8_t)k;
    }
    if (sp.empty()) sp.push_back({0.0, 1.0});
    // per species: order grouped by cell, counts
    std::vector<std::vector<int64_t>> order(sp.size());
    std::vector<std::vector<uint64_t>> counts(sp.size(), std::vector<uint64_t>(nc, 0));
    std::vector<int64_t> cell_of;
    {
        uint64_t k = 0;
        for (int64_t c = 0; c < nc; ++c)
            for (uint64_t i = 0; i < cell_counts[c]; ++i, ++k) {
                order[sid[k]].push_back((int64_t)k);
                counts[sid[k]][c]++;
            }
    }
    drop_graph(ctx);
    release_pops(ctx);
    ctx->species.clear();
    for (auto& x : sp) ctx->species.push_back({x.q, x.qom});
    for (size_t s = 0; s < sp.size(); ++s) {
        int rc;
        if (ctx->fp32) {
            ctx->p32.emplace_back();
            auto& P = ctx->p32.back();
            P.q = sp[s].q;
            P.qom = sp[s].qom;
            if ((rc = alloc_pop(ctx, P, counts[s], 0))) return rc;
            if ((rc = fill_pop(ctx, P, parts, ids, order[s], counts[s], cell_of))) return rc;
        } else {
            ctx->p64.emplace_back();
            auto& P = ctx->p64.back();
            P.q = sp[s].q;
            P.qom = sp[s].qom;
            if ((rc = alloc_pop(ctx, P, counts[s], 0))) return rc;
            if ((rc = fill_pop(ctx, P, parts, ids, order[s], counts[s], cell_of))) return rc;
        }
    }
    ctx->j_valid = false;
    ctx->particles_hint = n;
    return IPIC3D_OK;
}

int check_launch(ipic3d_ctx* ctx, int n);

template <typename X>
int grow(X*& p, size_t& cap, size_t need) {
    if (need <= cap && p) return IPIC3D_OK;
    dfree(p);
    size_t n = std::max<size_t>(need, 1);
    CU(cudaMalloc(&p, n * sizeof(X)));
    cap = n;
    return IPIC3D_OK;
}

template <typename T>
int scatter_pops(ipic3d_ctx* ctx, std::vector<PopStore<T>>& pops, const std::vector<std::vector<uint64_t>>& cnt,
                 int64_t n, bool have_ids, bool& relaid) {
    const int64_t nc = ctx->ncells();
    int rc;
    relaid = false;
    for (size_t k = 0; k < pops.size(); ++k) {
        auto& P = pops[k];
        bool fits = (int64_t)P.h_start.size() == nc + 1;
        for (int64_t c = 0; fits && c < nc; ++c) fits = (int64_t)cnt[k][c] <= P.h_start[c + 1] - P.h_start[c];
        if (!fits) {
            double q = P.q, qom = P.qom;
            P.release();
            P.q = q;
            P.qom = qom;
            if ((rc = alloc_pop(ctx, P, cnt[k], 0))) return rc;
            relaid = true;
        }
    }
    UploadPops<T> U{};
    U.npop = (int)pops.size();
    U.relative = std::is_same<T, float>::value ? 1 : 0;
    for (size_t k = 0; k < pops.size(); ++k) {
        auto& P = pops[k];
        U.x[k] = P.x; U.y[k] = P.y; U.z[k] = P.z; U.u[k] = P.u; U.v[k] = P.v; U.w[k] = P.w;
        U.id[k] = P.id;
        U.start[k] = P.start;
        U.count[k] = P.count;
        cudaStream_t st = ctx->stream;
        CU(cudaMemsetAsync(P.hole_cnt, 0, nc * sizeof(int32_t), st));
        CU(cudaMemsetAsync(P.arr_cnt, 0, nc * sizeof(int32_t), st));
        CU(cudaMemsetAsync(P.dirty_flag, 0, nc * sizeof(int32_t), st));
        CU(cudaMemsetAsync(P.pending_in_count, 0, sizeof(uint32_t), st));
        CU(cudaMemsetAsync(P.ctr, 0, sizeof(StepCounters), st));
    }
    UploadGeom g;
    g.ncells = (int)nc;
    g.sx = (int)ctx->props.size[0];
    g.sy = (int)ctx->props.size[1];
    g.sz = (int)ctx->props.size[2];
    for (int a = 0; a < 3; ++a) {
        g.origin[a] = ctx->props.origin[a];
        g.w[a] = ctx->props.cell_width[a];
    }
    int nl = launch_scatter<T>(ctx->st_parts, have_ids ? ctx->st_ids : nullptr, ctx->st_sid, ctx->st_off, U, g,
                               ctx->stream);
    (void)n;
    return check_launch(ctx, nl);
}

// Fast path of the device upload, for populations whose slot layout exists:
// the AoS records go to the device in chunks of whole cells on the copy
// stream, and each chunk's fused classify + scatter (+ deposit) kernel runs
// on the context stream as soon as its bytes have landed, so the kernels
// hide behind the copies. Returns 0 when done, 1 when a species is unknown
// (the host path creates it), 2 when a cell's slots were too few (the
// slower path re-lays out), < 0 on error. on_device: the records are in the
// staging buffer already (made on the device), one kernel over all cells.
template <typename T>
int upload_fast(ipic3d_ctx* ctx, std::vector<PopStore<T>>& pops, const ipic3d_particle* parts,
                const std::vector<int64_t>& off, const uint32_t* ids, bool on_device = false) {
    const int64_t nc = ctx->ncells(), n = off[nc];
    const int npop = (int)pops.size();
    for (auto& P : pops)
        if ((int64_t)P.h_start.size() != nc + 1) return 2;
    int rc;
    size_t cap_f = 0;
    // staging buffers keep their capacity: a cudaFree here would wait for
    // every stream of the device, an asynchronous download's copies included
    if ((rc = grow(reinterpret_cast<char*&>(ctx->st_parts), ctx->st_parts_cap, (size_t)n * sizeof(ipic3d_particle))))
        return rc;
    if (ids && (rc = grow(ctx->st_ids, ctx->st_ids_cap, (size_t)n))) return rc;
    if ((rc = grow(ctx->st_off, ctx->st_off_cap, (size_t)nc + 1))) return rc;
    if (!ctx->st_flags && (rc = grow(ctx->st_flags, cap_f, 2))) return rc;
    if (!ctx->copy_stream) CU(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    if (!ctx->copy_ev) CU(cudaEventCreateWithFlags(&ctx->copy_ev, cudaEventDisableTiming));
    cudaStream_t st = ctx->stream, cs = ctx->copy_stream;
    const bool deposit = ctx->fp32 && ctx->cfg.projector == IPIC3D_PROJECT_CIC;
    // the staging buffers are free once the context stream's earlier work is done
    CU(cudaEventRecord(ctx->copy_ev, st));
    CU(cudaStreamWaitEvent(cs, ctx->copy_ev, 0));
    CU(cudaMemcpyAsync(ctx->st_off, off.data(), (nc + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, cs));
    UploadPops<T> U{};
    U.npop = npop;
    U.relative = std::is_same<T, float>::value ? 1 : 0;
    for (int k = 0; k < npop; ++k) {
        auto& P = pops[k];
        U.x[k] = P.x; U.y[k] = P.y; U.z[k] = P.z; U.u[k] = P.u; U.v[k] = P.v; U.w[k] = P.w;
        U.id[k] = P.id;
        U.start[k] = P.start;
        U.count[k] = P.count;
        CU(cudaMemsetAsync(P.hole_cnt, 0, nc * sizeof(int32_t), st));
        CU(cudaMemsetAsync(P.arr_cnt, 0, nc * sizeof(int32_t), st));
        CU(cudaMemsetAsync(P.dirty_flag, 0, nc * sizeof(int32_t), st));
        CU(cudaMemsetAsync(P.pending_in_count, 0, sizeof(uint32_t), st));
        CU(cudaMemsetAsync(P.ctr, 0, sizeof(StepCounters), st));
    }
    CU(cudaMemsetAsync(ctx->st_flags, 0, 2 * sizeof(int), st));
    UploadDeposit dep{};
    dep.on = deposit ? 1 : 0;
    dep.sx = (int)ctx->props.size[0];
    dep.sy = (int)ctx->props.size[1];
    dep.sz = (int)ctx->props.size[2];
    dep.J = ctx->J;
    dep.rho = ctx->rho;
    if (deposit) {
        CU(cudaMemsetAsync(ctx->J, 0, ctx->nnode() * 3 * sizeof(double), st));
        CU(cudaMemsetAsync(ctx->rho, 0, ctx->nnode() * sizeof(double), st));
    }
    SpeciesTable sp{};
    sp.n = npop;
    for (int k = 0; k < npop; ++k) {
        sp.q[k] = pops[k].q;
        sp.qom[k] = pops[k].qom;
    }
    UploadGeom g;
    g.ncells = (int)nc;
    g.sx = (int)ctx->props.size[0];
    g.sy = (int)ctx->props.size[1];
    g.sz = (int)ctx->props.size[2];
    for (int a = 0; a < 3; ++a) {
        g.origin[a] = ctx->props.origin[a];
        g.w[a] = ctx->props.cell_width[a];
    }
    // chunks of about 16 MB of records, cut at cell boundaries (the last
    // chunk's kernel runs after the last copy: small chunks keep that short)
    const int64_t chunk = on_device ? std::max<int64_t>(1, n)
                                    : std::max<int64_t>(1, (int64_t)(16u << 20) / (int64_t)sizeof(ipic3d_particle));
    int nl = 0;
    for (int64_t c0 = 0; c0 < nc;) {
        int64_t c1 = c0 + 1;
        while (c1 < nc && off[c1] - off[c0] < chunk) ++c1;
        const int64_t p0 = off[c0], pn = off[c1] - off[c0];
        if (pn > 0 && !on_device) {
            CU(cudaMemcpyAsync(reinterpret_cast<char*>(ctx->st_parts) + p0 * sizeof(ipic3d_particle), parts + p0,
                               (size_t)pn * sizeof(ipic3d_particle), cudaMemcpyHostToDevice, cs));
            if (ids) CU(cudaMemcpyAsync(ctx->st_ids + p0, ids + p0, (size_t)pn * sizeof(uint32_t),
                                        cudaMemcpyHostToDevice, cs));
        }
        CU(cudaEventRecord(ctx->copy_ev, cs));
        CU(cudaStreamWaitEvent(st, ctx->copy_ev, 0));
        nl += launch_upload_cells<T>(ctx->st_parts, ids ? ctx->st_ids : nullptr, ctx->st_off, (int)c0, (int)c1, sp, U,
                                     g, dep, ctx->st_flags, st);
        c0 = c1;
    }
    if (deposit) nl += launch_j_finalize(ctx->g, (ctx->cfg.flags & IPIC3D_F_J_DIV8) != 0, !ctx->fp32, st);
    if ((rc = check_launch(ctx, nl))) return rc;
    int flags[2] = {0, 0};
    CU(cudaMemcpyAsync(flags, ctx->st_flags, sizeof(flags), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (flags[0]) return 1;
    if (flags[1]) return 2;
    ctx->j_valid = deposit;
    ctx->particles_hint = (uint64_t)n;
    return IPIC3D_OK;
}

// Upload through the device: one copy of the AoS records, then the species
// classification and the scatter run on the GPU. Returns 1 when the host
// path must be taken instead (a species the context does not know yet).
int upload_device(ipic3d_ctx* ctx, const ipic3d_particle* parts, const uint64_t* cell_counts, const uint32_t* ids) {
    const int64_t nc = ctx->ncells();
    const int npop = ctx->npops();
    if (ctx->species.empty() || npop != (int)ctx->species.size() || npop > kUploadMaxPops) return 1;
    std::vector<int64_t> off(nc + 1, 0);
    for (int64_t c = 0; c < nc; ++c) off[c + 1] = off[c] + (int64_t)cell_counts[c];
    const int64_t n = off[nc];
    if (n == 0) return 1;
    int rc = ctx->fp32 ? upload_fast(ctx, ctx->p32, parts, off, ids) : upload_fast(ctx, ctx->p64, parts, off, ids);
    if (rc <= 1) return rc;  // done, error, or the host path (unknown species)
    size_t cap_u = 0;
    if ((rc = grow(reinterpret_cast<char*&>(ctx->st_parts), ctx->st_parts_cap, (size_t)n * sizeof(ipic3d_particle))))
        return rc;
    if (ids && (rc = grow(ctx->st_ids, ctx->st_ids_cap, (size_t)n))) return rc;
    if ((rc = grow(ctx->st_sid, ctx->st_sid_cap, (size_t)n))) return rc;
    if ((rc = grow(ctx->st_off, ctx->st_off_cap, (size_t)nc + 1))) return rc;
    if ((rc = grow(ctx->st_cnt, ctx->st_cnt_cap, (size_t)nc * npop))) return rc;
    if (!ctx->st_unknown && (rc = grow(ctx->st_unknown, cap_u, 1))) return rc;
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(ctx->st_parts, parts, (size_t)n * sizeof(ipic3d_particle), cudaMemcpyHostToDevice, st));
    if (ids) CU(cudaMemcpyAsync(ctx->st_ids, ids, (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->st_off, off.data(), (nc + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(ctx->st_unknown, 0, sizeof(int), st));
    SpeciesTable sp{};
    sp.n = npop;
    for (int k = 0; k < npop; ++k) {
        sp.q[k] = ctx->species[k].first;
        sp.qom[k] = ctx->species[k].second;
    }
    int nl = launch_classify(ctx->st_parts, n, sp, ctx->st_sid, ctx->st_unknown, st);
    std::vector<std::vector<uint64_t>> cnt(npop, std::vector<uint64_t>(nc, 0));
    if (npop == 1) {
        for (int64_t c = 0; c < nc; ++c) cnt[0][c] = cell_counts[c];
    } else {
        nl += launch_count(ctx->st_sid, ctx->st_off, (int)nc, npop, ctx->st_cnt, st);
    }
    if ((rc = check_launch(ctx, nl))) return rc;
    int unknown = 0;
    CU(cudaMemcpyAsync(&unknown, ctx->st_unknown, sizeof(int), cudaMemcpyDeviceToHost, st));
    std::vector<int32_t> hc(npop > 1 ? (size_t)nc * npop : 0);
    if (npop > 1) CU(cudaMemcpyAsync(hc.data(), ctx->st_cnt, hc.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (unknown) return 1;
    if (npop > 1)
        for (int k = 0; k < npop; ++k)
            for (int64_t c = 0; c < nc; ++c) cnt[k][c] = (uint64_t)hc[(size_t)k * nc + c];
    bool relaid = false;
    if (ctx->fp32)
        rc = scatter_pops(ctx, ctx->p32, cnt, n, ids != nullptr, relaid);
    else
        rc = scatter_pops(ctx, ctx->p64, cnt, n, ids != nullptr, relaid);
    if (rc) return rc;
    if (relaid) drop_graph(ctx);
    ctx->j_valid = false;
    ctx->particles_hint = (uint64_t)n;
    return IPIC3D_OK;
}

// initCells(uniform) of the reference's :U:N benchmark mode (cell.h:638-697)
// made on the device (init.cu) and stored like an upload: the populations
// (the injection species first, as an upload orders them, then the
// electrons) are laid out for the known per-cell counts.
int init_uniform_impl(ipic3d_ctx* ctx, uint64_t n) {
    const int64_t nc = ctx->ncells();
    if (n > 0x7fffffffull) return fail(IPIC3D_E_INVALID, "%llu particles: at most 2^31 - 1", (unsigned long long)n);
    std::vector<uint64_t> counts(nc), zeros(nc, 0);
    std::vector<int64_t> off(nc + 1, 0);
    const uint64_t per = n / (uint64_t)nc, rem = n % (uint64_t)nc;
    for (int64_t c = 0; c < nc; ++c) {
        counts[c] = per + ((uint64_t)c < rem ? 1 : 0);
        off[c + 1] = off[c] + (int64_t)counts[c];
    }
    const std::pair<double, double> electron{-1.0, -25.0};  // species::electron (cell.h:107-118)
    std::vector<std::pair<double, double>> sp;
    if (ctx->cfg.flags & IPIC3D_F_INJECT_LOW_X) sp.push_back({ctx->cfg.inject_q, ctx->cfg.inject_qom});
    if (sp.empty() || sp[0] != electron) sp.push_back(electron);
    drop_graph(ctx);
    release_pops(ctx);
    ctx->species = sp;
    int rc;
    for (auto& x : sp) {
        const std::vector<uint64_t>& cnt = x == electron ? counts : zeros;
        if (ctx->fp32) {
            ctx->p32.emplace_back();
            ctx->p32.back().q = x.first;
            ctx->p32.back().qom = x.second;
            if ((rc = alloc_pop(ctx, ctx->p32.back(), cnt, 0))) return rc;
        } else {
            ctx->p64.emplace_back();
            ctx->p64.back().q = x.first;
            ctx->p64.back().qom = x.second;
            if ((rc = alloc_pop(ctx, ctx->p64.back(), cnt, 0))) return rc;
        }
    }
    if (n == 0) {
        ctx->j_valid = false;
        ctx->particles_hint = 0;
        return IPIC3D_OK;
    }
    if ((rc = grow(reinterpret_cast<char*&>(ctx->st_parts), ctx->st_parts_cap, (size_t)n * sizeof(ipic3d_particle))))
        return rc;
    int nl = launch_init_uniform((int)ctx->props.size[0], (int)ctx->props.size[1], (int)ctx->props.size[2],
                                 ctx->props.origin, ctx->props.cell_width, n, ctx->st_parts, ctx->stream);
    if ((rc = check_launch(ctx, nl))) return rc;
    rc = ctx->fp32 ? upload_fast(ctx, ctx->p32, nullptr, off, nullptr, true)
                   : upload_fast(ctx, ctx->p64, nullptr, off, nullptr, true);
    if (rc < 0) return rc;
    if (rc > 0) return fail(IPIC3D_E_CUDA, "device initialisation: the scatter found an unexpected layout");
    return IPIC3D_OK;
}

// initCells<uniform_pos_normal_speed> of the .inp driver (cell.h:492-636):
// the per-cell counts on the host (phase 1: one sequential stream), every
// particle on the device (phase 2: per-cell streams), stored like an
// upload. One species: q = e, q/m = e / m_p (cell.h:502-503, 624-625); with
// injection on, the injection species comes first, as an upload orders it.
int init_normal_impl(ipic3d_ctx* ctx, uint64_t n, const double low[3], const double hig[3], const double mean[3],
                     const double stddev[3]) {
    const int64_t nc = ctx->ncells();
    if (n > 0x7fffffffull) return fail(IPIC3D_E_INVALID, "%llu particles: at most 2^31 - 1", (unsigned long long)n);
    for (int a = 0; a < 3; ++a)
        if (!(low[a] < hig[a])) return fail(IPIC3D_E_INVALID, "position box: low must be below hig on every axis");
    if (n > 0) {  // phase 1 must find positions inside the universe
        const ipic3d_props& pr = ctx->props;
        for (int a = 0; a < 3; ++a) {
            const double top = pr.origin[a] + pr.size[a] * pr.cell_width[a];
            if (!(hig[a] > pr.origin[a] && low[a] < top))
                return fail(IPIC3D_E_INVALID, "position box does not meet the universe on axis %d", a);
        }
    }
    std::vector<uint64_t> counts, zeros(nc, 0);
    init_normal_counts(ctx->props, n, low, hig, counts);
    std::vector<int64_t> off(nc + 1, 0);
    for (int64_t c = 0; c < nc; ++c) off[c + 1] = off[c] + (int64_t)counts[c];
    const double e = 1.602176565e-19, m = 1.672621777e-27;
    const std::pair<double, double> proton{e, e / m};
    std::vector<std::pair<double, double>> sp;
    if (ctx->cfg.flags & IPIC3D_F_INJECT_LOW_X) sp.push_back({ctx->cfg.inject_q, ctx->cfg.inject_qom});
    if (sp.empty() || sp[0] != proton) sp.push_back(proton);
    drop_graph(ctx);
    release_pops(ctx);
    ctx->species = sp;
    int rc;
    for (auto& x : sp) {
        const std::vector<uint64_t>& cnt = x == proton ? counts : zeros;
        if (ctx->fp32) {
            ctx->p32.emplace_back();
            ctx->p32.back().q = x.first;
            ctx->p32.back().qom = x.second;
            if ((rc = alloc_pop(ctx, ctx->p32.back(), cnt, 0))) return rc;
        } else {
            ctx->p64.emplace_back();
            ctx->p64.back().q = x.first;
            ctx->p64.back().qom = x.second;
            if ((rc = alloc_pop(ctx, ctx->p64.back(), cnt, 0))) return rc;
        }
    }
    const uint64_t total = (uint64_t)off[nc];
    if (total == 0) {
        ctx->j_valid = false;
        ctx->particles_hint = 0;
        return IPIC3D_OK;
    }
    if ((rc = grow(reinterpret_cast<char*&>(ctx->st_parts), ctx->st_parts_cap, (size_t)total * sizeof(ipic3d_particle))))
        return rc;
    // per-cell counts (a temporary buffer) and offsets (the upload path's
    // staging array) for the generator
    uint64_t* d_count = nullptr;
    CU(cudaMalloc(&d_count, (size_t)nc * sizeof(uint64_t)));
    if ((rc = grow(ctx->st_off, ctx->st_off_cap, (size_t)nc + 1))) {
        cudaFree(d_count);
        return rc;
    }
    cudaStream_t st = ctx->stream;
    cudaError_t e1 = cudaMemcpyAsync(d_count, counts.data(), (size_t)nc * sizeof(uint64_t), cudaMemcpyHostToDevice, st);
    if (e1 == cudaSuccess)
        e1 = cudaMemcpyAsync(ctx->st_off, off.data(), (size_t)(nc + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
    int nl = 0;
    if (e1 == cudaSuccess)
        nl = launch_init_normal(ctx->props, mean, stddev, proton.first, proton.second, d_count, ctx->st_off,
                                ctx->st_parts, st);
    if (e1 == cudaSuccess) e1 = cudaStreamSynchronize(st);
    cudaFree(d_count);
    if (e1 != cudaSuccess) return fail(IPIC3D_E_CUDA, "device initialisation: %s", cudaGetErrorString(e1));
    if ((rc = check_launch(ctx, nl))) return rc;
    rc = ctx->fp32 ? upload_fast(ctx, ctx->p32, nullptr, off, nullptr, true)
                   : upload_fast(ctx, ctx->p64, nullptr, off, nullptr, true);
    if (rc < 0) return rc;
    if (rc > 0) return fail(IPIC3D_E_CUDA, "device initialisation: the scatter found an unexpected layout");
    return IPIC3D_OK;
}

// Downloads every population, adding the pending particles to their cells.
// The reference's record of a particle of population P in cell c from its
// GPU state (cell-relative FP32 positions made absolute in FP64 with the
// pack kernel's formula).
template <typename T>
ipic3d_particle host_record(const ipic3d_ctx* ctx, const PopStore<T>& P, int64_t c, const Mover<T>& m) {
    const ipic3d_props& pr = ctx->props;
    ipic3d_particle p;
    if (std::is_same<T, float>::value) {
        const int64_t cx = c / (pr.size[1] * pr.size[2]), cy = (c / pr.size[2]) % pr.size[1], cz = c % pr.size[2];
        p.position[0] = (pr.origin[0] + (double)cx * pr.cell_width[0]) + (double)m.x * pr.cell_width[0];
        p.position[1] = (pr.origin[1] + (double)cy * pr.cell_width[1]) + (double)m.y * pr.cell_width[1];
        p.position[2] = (pr.origin[2] + (double)cz * pr.cell_width[2]) + (double)m.z * pr.cell_width[2];
    } else {
        p.position[0] = (double)m.x;
        p.position[1] = (double)m.y;
        p.position[2] = (double)m.z;
    }
    p.velocity[0] = (double)m.u;
    p.velocity[1] = (double)m.v;
    p.velocity[2] = (double)m.w;
    p.q = P.q;
    p.qom = P.qom;
    return p;
}

// Download through the device. The per-cell output offsets come from the
// counts and the cells of the particles waiting for a slot (host, small);
// the AoS records are packed on the device in chunks of cells and each
// chunk is copied to the host on the copy stream while the next is packed
// (one cudaMemcpyAsync per chunk and array); the waiting particles (few)
// are filled in on the host. Order per cell: population 0's particles in
// slot order, then its waiting particles in list order, then population
// 1's, and so on. `particles` / `ids` may be NULL (counts only).
// Completes a download: waits for its copies, then writes the waiting
// particles into their places.
int download_finish(ipic3d_ctx* ctx) {
    if (!ctx->dl_busy) return IPIC3D_OK;
    ctx->dl_busy = false;
    CU(cudaStreamSynchronize(ctx->dl_stream));
    for (const auto& f : ctx->dl_fill) {
        if (ctx->dl_xyz)
            for (int a = 0; a < 3; ++a) ctx->dl_xyz[3 * f.at + a] = f.rec.position[a];
        else if (ctx->dl_parts)
            ctx->dl_parts[f.at] = f.rec;
        if (ctx->dl_ids) ctx->dl_ids[f.at] = f.id;
    }
    ctx->dl_fill.clear();
    return IPIC3D_OK;
}

template <typename T>
int download_device(ipic3d_ctx* ctx, std::vector<PopStore<T>>& pops, ipic3d_particle* particles, uint64_t capacity,
                    uint64_t* cell_counts, uint32_t* ids, double* xyz = nullptr, bool async = false) {
    int rc = download_finish(ctx);  // one download at a time
    if (rc) return rc;
    const int64_t nc = ctx->ncells();
    const int npop = (int)pops.size();
    if (npop > kUploadMaxPops) return fail(IPIC3D_E_CAPACITY, "%d populations: at most %d", npop, kUploadMaxPops);
    cudaStream_t st = ctx->stream;
    std::vector<int32_t> cnt((size_t)npop * nc);
    std::vector<uint32_t> npend(npop, 0);
    for (int k = 0; k < npop; ++k) {
        CU(cudaMemcpyAsync(cnt.data() + (size_t)k * nc, pops[k].count, nc * sizeof(int32_t), cudaMemcpyDeviceToHost,
                           st));
        CU(cudaMemcpyAsync(&npend[k], pops[k].pending_in_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    }
    CU(cudaStreamSynchronize(st));
    std::vector<std::vector<Mover<T>>> pend(npop);
    std::vector<int32_t> pcell;  // waiting particles per (population, cell), if any
    bool waiting = false;
    for (int k = 0; k < npop; ++k) {
        if (!npend[k]) continue;
        pend[k].resize(npend[k]);
        CU(cudaMemcpyAsync(pend[k].data(), pops[k].pending_in, npend[k] * sizeof(Mover<T>), cudaMemcpyDeviceToHost,
                           st));
        waiting = true;
    }
    if (waiting) CU(cudaStreamSynchronize(st));
    for (int k = 0; k < npop; ++k)
        for (const auto& m : pend[k]) {
            if (m.cell < 0 || m.cell >= nc) return fail(IPIC3D_E_STATE, "waiting particle in cell %d", m.cell);
            if (pcell.empty()) pcell.assign((size_t)npop * nc, 0);
            ++pcell[(size_t)k * nc + m.cell];
        }
    std::vector<int64_t> dst((size_t)npop * nc);
    int64_t n = 0;
    for (int64_t c = 0; c < nc; ++c) {
        const int64_t first = n;
        for (int k = 0; k < npop; ++k) {
            const size_t i = (size_t)k * nc + c;
            dst[i] = n;
            n += cnt[i] + (pcell.empty() ? 0 : pcell[i]);
        }
        if (cell_counts) cell_counts[c] = (uint64_t)(n - first);
    }
    if ((!particles && !ids && !xyz) || n == 0) return IPIC3D_OK;
    if ((uint64_t)n > capacity)
        return fail(IPIC3D_E_CAPACITY, "output capacity %llu too small", (unsigned long long)capacity);
    if ((rc = grow(reinterpret_cast<char*&>(ctx->st_dl), ctx->st_dl_cap, (size_t)n * sizeof(ipic3d_particle))))
        return rc;
    if (ids && (rc = grow(ctx->st_dl_ids, ctx->st_dl_ids_cap, (size_t)n))) return rc;
    if ((rc = grow(ctx->st_dst, ctx->st_dst_cap, dst.size()))) return rc;
    if (!ctx->dl_stream) CU(cudaStreamCreateWithFlags(&ctx->dl_stream, cudaStreamNonBlocking));
    if (!ctx->dl_ev) CU(cudaEventCreateWithFlags(&ctx->dl_ev, cudaEventDisableTiming));
    CU(cudaMemcpyAsync(ctx->st_dst, dst.data(), dst.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    PackPops<T> P{};
    P.npop = npop;
    P.relative = std::is_same<T, float>::value ? 1 : 0;
    for (int k = 0; k < npop; ++k) {
        const auto& S = pops[k];
        P.x[k] = S.x; P.y[k] = S.y; P.z[k] = S.z; P.u[k] = S.u; P.v[k] = S.v; P.w[k] = S.w;
        P.id[k] = S.id;
        P.start[k] = S.start;
        P.count[k] = S.count;
        P.q[k] = S.q;
        P.qom[k] = S.qom;
    }
    P.dst = ctx->st_dst;
    P.positions_only = xyz ? 1 : 0;
    UploadGeom g;
    g.ncells = (int)nc;
    g.sx = (int)ctx->props.size[0];
    g.sy = (int)ctx->props.size[1];
    g.sz = (int)ctx->props.size[2];
    for (int a = 0; a < 3; ++a) {
        g.origin[a] = ctx->props.origin[a];
        g.w[a] = ctx->props.cell_width[a];
    }
    // chunks of about 64 MB of records, cut at cell boundaries: few enough
    // that enqueueing them (a pack kernel, an event and a copy each) costs
    // little host time, which otherwise delays the caller's next upload
    const int64_t chunk = std::max<int64_t>(1, (int64_t)(64u << 20) / (int64_t)sizeof(ipic3d_particle));
    cudaStream_t cs = ctx->dl_stream;
    auto* stage = static_cast<ipic3d_particle*>(ctx->st_dl);
    auto* stage_xyz = static_cast<double*>(ctx->st_dl);  // positions only: 3 doubles per particle
    int nl = 0;
    for (int64_t c0 = 0; c0 < nc;) {
        const int64_t o0 = dst[(size_t)c0];
        int64_t c1 = c0 + 1;
        while (c1 < nc && dst[(size_t)c1] - o0 < chunk) ++c1;
        const int64_t o1 = c1 < nc ? dst[(size_t)c1] : n;
        nl += launch_pack_cells<T>(P, g, (int)c0, (int)c1, stage, ids ? ctx->st_dl_ids : nullptr, st);
        if (o1 > o0) {
            CU(cudaEventRecord(ctx->dl_ev, st));
            CU(cudaStreamWaitEvent(cs, ctx->dl_ev, 0));
            if (xyz)
                CU(cudaMemcpyAsync(xyz + 3 * o0, stage_xyz + 3 * o0, (size_t)(o1 - o0) * 3 * sizeof(double),
                                   cudaMemcpyDeviceToHost, cs));
            else if (particles)
                CU(cudaMemcpyAsync(particles + o0, stage + o0, (size_t)(o1 - o0) * sizeof(ipic3d_particle),
                                   cudaMemcpyDeviceToHost, cs));
            if (ids)
                CU(cudaMemcpyAsync(ids + o0, ctx->st_dl_ids + o0, (size_t)(o1 - o0) * sizeof(uint32_t),
                                   cudaMemcpyDeviceToHost, cs));
        }
        c0 = c1;
    }
    if ((rc = check_launch(ctx, nl))) return rc;
    // the waiting particles go into the gaps after each cell's slots once
    // the copies have landed
    ctx->dl_fill.clear();
    for (int k = 0; k < npop; ++k) {
        if (pend[k].empty()) continue;
        std::vector<int32_t> rank(nc, 0);
        for (const auto& m : pend[k]) {
            const size_t i = (size_t)k * nc + m.cell;
            ctx->dl_fill.push_back({dst[i] + cnt[i] + rank[m.cell]++, host_record(ctx, pops[k], m.cell, m), m.id});
        }
    }
    ctx->dl_parts = particles;
    ctx->dl_ids = ids;
    ctx->dl_xyz = xyz;
    ctx->dl_busy = true;
    if (async) return IPIC3D_OK;
    return download_finish(ctx);
}

// Device re-layout of one population: new per-cell capacities from the
// stored counts plus the particles waiting for a slot, then a copy of every
// cell and the placement of the waiting particles.
template <typename T>
int relayout_pop(ipic3d_ctx* ctx, PopStore<T>& P) {
    const int64_t nc = ctx->ncells();
    cudaStream_t st = ctx->stream;
    int32_t* d_pend = nullptr;
    CU(cudaMalloc(&d_pend, nc * sizeof(int32_t)));
    CU(cudaMemsetAsync(d_pend, 0, nc * sizeof(int32_t), st));
    int nl = launch_pending_count<T>(P.view(), d_pend, st);
    std::vector<int32_t> hcnt(nc), hpend(nc);
    CU(cudaMemcpyAsync(hcnt.data(), P.count, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(hpend.data(), d_pend, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    cudaFree(d_pend);
    std::vector<uint64_t> counts(nc);
    for (int64_t c = 0; c < nc; ++c) counts[c] = (uint64_t)hcnt[c] + (uint64_t)hpend[c];
    PopStore<T> N;
    N.q = P.q;
    N.qom = P.qom;
    int rc = alloc_pop(ctx, N, counts, 0);
    if (rc) {
        N.release();
        return rc;
    }
    nl += launch_relayout<T>(P.view(), N.view(), (int)nc, nullptr, st);
    if ((rc = check_launch(ctx, nl))) {
        N.release();
        return rc;
    }
    CU(cudaStreamSynchronize(st));
    P.release();
    P = std::move(N);
    N.x = N.y = N.z = N.u = N.v = N.w = nullptr;  // moved-from: nothing to free
    return IPIC3D_OK;
}

// Re-lays out every population on the device (cells ran out of slack).
int relayout(ipic3d_ctx* ctx) {
    drop_graph(ctx);
    int rc;
    for (auto& P : ctx->p32)
        if ((rc = relayout_pop(ctx, P))) return rc;
    for (auto& P : ctx->p64)
        if ((rc = relayout_pop(ctx, P))) return rc;
    ctx->rebuilds++;
    return IPIC3D_OK;
}

void refresh_geom(ipic3d_ctx* ctx) {
    Geom& g = ctx->g;
    const ipic3d_props& p = ctx->props;
    g.sx = (int)p.size[0];
    g.sy = (int)p.size[1];
    g.sz = (int)p.size[2];
    g.ncells = (int)ctx->ncells();
    for (int a = 0; a < 3; ++a) {
        g.w[a] = p.cell_width[a];
        g.inv_w[a] = 1.0 / p.cell_width[a];
        g.half_w[a] = p.cell_width[a] / 2.0;
        g.origin[a] = p.origin[a];
        g.object_center[a] = p.object_center[a];
        g.L[a] = (double)p.size[a] * p.cell_width[a];
        g.bc_lo[a] = ctx->cfg.bc_low[a];
        g.bc_hi[a] = ctx->cfg.bc_high[a];
    }
    g.dt = p.dt;
    g.c = p.speed_of_light;
    g.inv_pic = 1.0 / (3.14159265358979323846 * p.speed_of_light);
    g.planet_r2 = p.planet_radius * p.planet_radius;
    g.mft = -p.external_b[2] * std::pow(p.planet_radius, 3);  // host libm, as cell.h:923
    g.vol = p.cell_width[0] * p.cell_width[1] * p.cell_width[2];
    g.flags = ctx->cfg.flags;
    g.mover = ctx->cfg.mover;
    g.deposit = ctx->cfg.projector == IPIC3D_PROJECT_CIC ? 1 : 0;
    g.field = ctx->field;
    g.bcfield = ctx->bcfield;
    g.J = ctx->J;
    g.rho = ctx->rho;
    g.node32 = ctx->fp32 ? ctx->node32 : nullptr;  // the FP32 gather's node copy
    g.cellcoef = ctx->cellcoef;
}

int check_launch(ipic3d_ctx* ctx, int n) {
    ctx->launches += (uint64_t)n;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "kernel launch: %s", cudaGetErrorString(e));
    return IPIC3D_OK;
}

// Phase brackets: events recorded only while profiling.
void ph_begin(ipic3d_ctx* ctx, int ph) {
    if (!ctx->profiling) return;
    cudaEventRecord(ctx->ph_ev[ph][0], ctx->stream);
    ctx->ph_open[ph] = true;
}
void ph_end(ipic3d_ctx* ctx, int ph) {
    if (!ctx->profiling || !ctx->ph_open[ph]) return;
    cudaEventRecord(ctx->ph_ev[ph][1], ctx->stream);
}
// After a profiled step: add the closed intervals to the totals.
int ph_collect(ipic3d_ctx* ctx) {
    if (!ctx->profiling) return IPIC3D_OK;
    CU(cudaStreamSynchronize(ctx->stream));
    for (int ph = 0; ph < IPIC3D_PHASE_COUNT; ++ph) {
        if (!ctx->ph_open[ph]) continue;
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, ctx->ph_ev[ph][0], ctx->ph_ev[ph][1]));
        ctx->prof.ms[ph] += ms;
        ctx->prof.launches[ph] += 1;
        ctx->ph_open[ph] = false;
    }
    ctx->prof.particles[IPIC3D_PHASE_PUSH] += ctx->push_particles;
    return IPIC3D_OK;
}

// projectToDensityField over the stored particles (deposit-only pass).
int project_impl(ipic3d_ctx* ctx) {
    cudaStream_t st = ctx->stream;
    CU(cudaMemsetAsync(ctx->J, 0, ctx->nnode() * 3 * sizeof(double), st));
    CU(cudaMemsetAsync(ctx->rho, 0, ctx->nnode() * sizeof(double), st));
    Geom g = ctx->g;
    g.deposit = 1;
    int n = 0;
    for (auto& S : pop_sets(ctx->p32)) n += launch_push<float>(g, S, 1, ctx->tuner.shape(), st);
    for (auto& S : pop_sets(ctx->p64)) n += launch_push<double>(g, S, 1, ctx->tuner.shape(), st);
    n += launch_j_finalize(g, (ctx->cfg.flags & IPIC3D_F_J_DIV8) != 0, !ctx->fp32, st);
    ctx->j_valid = true;
    return check_launch(ctx, n);
}

// The solver's kernels (no ghost copy) on stream `st`; returns the launches.
// raw_j: J holds the deposit's raw node sums, which the E update folds and
// normalises as the J finalisation would; after_e: recorded after the E
// update (the last read of J).
int enqueue_solver(ipic3d_ctx* ctx, cudaStream_t st, bool raw_j = false, cudaEvent_t after_e = nullptr) {
    const bool div8 = (ctx->cfg.flags & IPIC3D_F_J_DIV8) != 0;
    int n = 0;
    if (ctx->cfg.solver == IPIC3D_SOLVER_LEAPFROG)
        n += launch_leapfrog(ctx->g, (ctx->cfg.flags & IPIC3D_F_REFRESH_NODE_B) != 0, !ctx->fp32, st, raw_j, div8,
                             after_e);
    else if (ctx->cfg.solver == IPIC3D_SOLVER_FORWARD)
        n += launch_forward(ctx->g, st, raw_j, div8, !ctx->fp32, after_e);
    if (ctx->fp32 && ctx->cfg.mover == IPIC3D_MOVER_FIELD && ctx->cfg.solver != IPIC3D_SOLVER_STATIC)
        n += launch_cell_coef(ctx->g, ctx->cellcoef, st);
    return n;
}

int solve_impl(ipic3d_ctx* ctx) {
    ph_begin(ctx, IPIC3D_PHASE_FIELDS);
    const int n = enqueue_solver(ctx, ctx->stream);
    ph_end(ctx, IPIC3D_PHASE_FIELDS);
    return check_launch(ctx, n);
}

// mover + export + import of all populations (+ injection), with the fused
// deposit when the projector is on. The pending push and the injection only
// append to the outbox and the arrival lists and deposit with atomics, as the
// push does: they run on a second stream beside the push (in its tail, as its
// persistent blocks finish) and join before the placement; the J
// finalisation, which needs every deposit but nothing of the placement, runs
// beside the placement, and so does the next step's field solve
// (`next_solve`: the ghost faces beside the push, the solver once every
// deposit is in; they read and write fields and J only, the move and the
// placement touch particles, J and interior nodes' reads only). Then the
// E update reads the raw deposit sums and folds and normalises them itself:
// no J finalisation, and J and rho are cleared for the next step's deposit
// once it has read them (`cleared`: a step that starts so skips its own
// clear). With phase timing on, everything runs on one stream.
int move_impl(ipic3d_ctx* ctx, bool deposit, bool next_solve = false, bool cleared = false) {
    cudaStream_t st = ctx->stream;
    Geom g = ctx->g;
    g.deposit = deposit ? 1 : 0;
    int n = 0;
    for (auto& P : ctx->p32) CU(cudaMemsetAsync(P.ctr, 0, offsetof(StepCounters, lost), st));
    for (auto& P : ctx->p64) CU(cudaMemsetAsync(P.ctr, 0, offsetof(StepCounters, lost), st));
    if (deposit) {
        ph_begin(ctx, IPIC3D_PHASE_MOMENTS);
        if (!cleared) {
            CU(cudaMemsetAsync(ctx->J, 0, ctx->nnode() * 3 * sizeof(double), st));
            CU(cudaMemsetAsync(ctx->rho, 0, ctx->nnode() * sizeof(double), st));
        }
    }
    const bool fork = !ctx->profiling;
    if (fork && !ctx->aux_stream) {
        // the higher priority: the solver chain on it is the longer branch
        int least = 0, greatest = 0;
        CU(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CU(cudaStreamCreateWithPriority(&ctx->aux_stream, cudaStreamNonBlocking, greatest));
        for (auto& e : ctx->aux_ev) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    cudaStream_t aux = fork ? ctx->aux_stream : st;
    if (fork) {
        CU(cudaEventRecord(ctx->aux_ev[0], st));
        CU(cudaStreamWaitEvent(aux, ctx->aux_ev[0], 0));
        // the next step's ghost faces: they copy this step's solved fields
        // into ghost nodes and ghost cells, which the move does not read
        if (next_solve) n += launch_ghost(ctx->g, aux);
    }
    const auto s32 = pop_sets(ctx->p32);
    const auto s64 = pop_sets(ctx->p64);
    PushShape shp = ctx->tuner.next();
    shp.wait_polls = ctx->wait_polls;
    ph_begin(ctx, IPIC3D_PHASE_PUSH);
    if (ctx->tune_timing) CU(cudaEventRecord(ctx->tune_ev[0], st));
    for (auto& S : s32) n += launch_push<float>(g, S, 0, shp, st);
    for (auto& S : s64) n += launch_push<double>(g, S, 0, shp, st);
    if (ctx->tune_timing) CU(cudaEventRecord(ctx->tune_ev[1], st));
    ph_end(ctx, IPIC3D_PHASE_PUSH);
    ctx->push_particles = ctx->particles_hint;
    ph_begin(ctx, IPIC3D_PHASE_PENDING);
    for (auto& S : s32) n += launch_push_pending<float>(g, S, aux);
    for (auto& S : s64) n += launch_push_pending<double>(g, S, aux);
    ph_end(ctx, IPIC3D_PHASE_PENDING);
    const bool inject = (ctx->cfg.flags & IPIC3D_F_INJECT_LOW_X) && ctx->cfg.bc_low[0] == IPIC3D_BC_OPEN &&
                        ctx->cfg.inject_per_cell > 0;
    if (inject) {
        ph_begin(ctx, IPIC3D_PHASE_INJECT);
        if (ctx->fp32)
            n += launch_inject<float>(g, ctx->p32[0].view(), ctx->cfg.inject_per_cell, ctx->cfg.inject_drift,
                                      ctx->cfg.inject_vth, ctx->cfg.seed, ctx->d_step, aux);
        else
            n += launch_inject<double>(g, ctx->p64[0].view(), ctx->cfg.inject_per_cell, ctx->cfg.inject_drift,
                                       ctx->cfg.inject_vth, ctx->cfg.seed, ctx->d_step, aux);
        ph_end(ctx, IPIC3D_PHASE_INJECT);
    }
    if (fork) {  // every append and deposit is done
        CU(cudaEventRecord(ctx->aux_ev[1], aux));
        CU(cudaStreamWaitEvent(st, ctx->aux_ev[1], 0));
    }
    const bool jfork = fork && (deposit || next_solve);
    const bool raw_j = jfork && deposit && next_solve;
    if (jfork) {
        CU(cudaEventRecord(ctx->aux_ev[2], st));
        CU(cudaStreamWaitEvent(aux, ctx->aux_ev[2], 0));
        if (raw_j) {
            n += enqueue_solver(ctx, aux, true, ctx->aux_ev[4]);
        } else {
            if (deposit) n += launch_j_finalize(g, (ctx->cfg.flags & IPIC3D_F_J_DIV8) != 0, !ctx->fp32, aux);
            if (next_solve) n += enqueue_solver(ctx, aux);
        }
    }
    ph_begin(ctx, IPIC3D_PHASE_PLACE);
    for (auto& S : s32) n += launch_place<float>(g, S, st);
    for (auto& S : s64) n += launch_place<double>(g, S, st);
    // the last rotation also advances the device step counter
    for (size_t i = 0; i < s32.size(); ++i)
        n += launch_pending_rotate<float>(s32[i], s64.empty() && i + 1 == s32.size() ? ctx->d_step : nullptr, st);
    for (size_t i = 0; i < s64.size(); ++i)
        n += launch_pending_rotate<double>(s64[i], i + 1 == s64.size() ? ctx->d_step : nullptr, st);
    if (s32.empty() && s64.empty()) {
        k_step_end<<<1, 1, 0, st>>>(ctx->d_step);
        ++n;
    }
    ph_end(ctx, IPIC3D_PHASE_PLACE);
    if (raw_j) {  // the E update has read J: clear J and rho for the next step
        CU(cudaStreamWaitEvent(st, ctx->aux_ev[4], 0));
        CU(cudaMemsetAsync(ctx->J, 0, ctx->nnode() * 3 * sizeof(double), st));
        CU(cudaMemsetAsync(ctx->rho, 0, ctx->nnode() * sizeof(double), st));
    }
    if (jfork) {
        CU(cudaEventRecord(ctx->aux_ev[3], aux));
        CU(cudaStreamWaitEvent(st, ctx->aux_ev[3], 0));
    } else {
        if (deposit) {
            n += launch_j_finalize(g, (ctx->cfg.flags & IPIC3D_F_J_DIV8) != 0, !ctx->fp32, st);
            ph_end(ctx, IPIC3D_PHASE_MOMENTS);
        }
        if (next_solve) {
            n += launch_ghost(ctx->g, st);
            ph_begin(ctx, IPIC3D_PHASE_FIELDS);
            n += enqueue_solver(ctx, st);
            ph_end(ctx, IPIC3D_PHASE_FIELDS);
        }
    }
    return check_launch(ctx, n);
}

// ---- push-shape autotuning ---------------------------------------------------
// Shapes the autotuner chose, per device and workload: a later context or
// batch with the same workload starts from the cached shape without trials.
using TuneKey = std::vector<int64_t>;
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<PushShape, float>> g_tune_cache;

int ilog2(uint64_t n) {
    int k = 0;
    while (n >>= 1) ++k;
    return k;
}

// what a shape's speed depends on: the grid, the populations, the particle
// count (to a factor of two), the mover, the deposit, the boundaries
TuneKey tune_key(int dev, int kind, int64_t a, int64_t b, int64_t c, int pops, uint64_t particles,
                 const ipic3d_config& cfg) {
    TuneKey k{dev, kind, a, b, c, pops, ilog2(particles), cfg.mover, cfg.projector, cfg.solver, (int64_t)cfg.flags};
    for (int ax = 0; ax < 3; ++ax) {
        k.push_back(cfg.bc_low[ax]);
        k.push_back(cfg.bc_high[ax]);
    }
    return k;
}

bool tune_lookup(const TuneKey& k, PushTuner& t) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(k);
    if (it == g_tune_cache.end()) return false;
    t.adopt(it->second.first, it->second.second);
    return true;
}

void tune_store(const TuneKey& k, const PushTuner& t) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[k] = {t.shape(), t.best_ms()};
}

TuneKey ctx_tune_key(const ipic3d_ctx* ctx) {
    return tune_key(ctx->device, 0, ctx->props.size[0], ctx->props.size[1], ctx->props.size[2], ctx->npops(),
                    ctx->particles_hint, ctx->cfg);
}

// Before a run of steps: a tuning pass starts (or a cached shape is taken)
// when the FP32 context tunes its shape and has particles it was not tuned
// for (none yet, or a count off by more than a factor of two).
void tune_prepare(ipic3d_ctx* ctx) {
    if (!ctx->fp32 || ctx->cfg.block_size != 0 || ctx->shape_fixed || ctx->tuner.running()) return;
    const uint64_t n = ctx->particles_hint, t = ctx->tuned_particles;
    if (n == 0 || (t && n <= 2 * t && 2 * n >= t)) return;
    ctx->tuned_particles = n;
    drop_graph(ctx);  // captured with the previous shape
    if (!tune_lookup(ctx_tune_key(ctx), ctx->tuner)) ctx->tuner.start(push32_blocks_per_sm(ctx->device));
}

// After a trial step: its push time to the tuner; a finished pass is cached.
int tune_record(ipic3d_ctx* ctx) {
    CU(cudaEventSynchronize(ctx->tune_ev[1]));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, ctx->tune_ev[0], ctx->tune_ev[1]));
    ctx->tuner.record(ms);
    if (!ctx->tuner.running()) {
        tune_store(ctx_tune_key(ctx), ctx->tuner);
        drop_graph(ctx);
    }
    return IPIC3D_OK;
}

// The kernel sequence of one step graph (kStepFull: one whole timestep).
int enqueue_step(ipic3d_ctx* ctx, int kind = kStepFull) {
    const bool project = ctx->cfg.projector == IPIC3D_PROJECT_CIC;
    int rc;
    if ((kind == kStepFull || kind == kStepSolve) && ctx->cfg.solver != IPIC3D_SOLVER_STATIC) {
        int n = launch_ghost(ctx->g, ctx->stream);
        if ((rc = check_launch(ctx, n))) return rc;
        if ((rc = solve_impl(ctx))) return rc;
    }
    if (kind == kStepSolve) {  // a move follows: J and rho cleared for its deposit
        if (project) {
            CU(cudaMemsetAsync(ctx->J, 0, ctx->nnode() * 3 * sizeof(double), ctx->stream));
            CU(cudaMemsetAsync(ctx->rho, 0, ctx->nnode() * sizeof(double), ctx->stream));
        }
        return IPIC3D_OK;
    }
    // advances the device step counter
    return move_impl(ctx, project, kind == kStepMoveSolve, kind == kStepMoveSolve || kind == kStepMove);
}

// Replays step graph `kind`, capturing it first if needed.
int run_graph(ipic3d_ctx* ctx, int kind) {
    if (!ctx->graph[kind]) {
        cudaGraph_t graph = nullptr;
        CU(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const uint64_t before = ctx->launches;
        const int rc = enqueue_step(ctx, kind);
        ctx->graph_kernels[kind] = ctx->launches - before;
        ctx->launches = before;  // capturing runs nothing
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&ctx->graph[kind], graph, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    CU(cudaGraphLaunch(ctx->graph[kind], ctx->stream));
    ctx->launches += ctx->graph_kernels[kind];
    return IPIC3D_OK;
}

// Reads the step counters back; rebuilds the layout when particles wait for
// a slot; reports lost particles.
int after_steps(ipic3d_ctx* ctx, bool force_relayout = false) {
    // the counters of every population: asynchronous copies, one wait
    const int np = std::min(ctx->npops(), kMaxPops);
    int k = 0;
    for (auto& P : ctx->p32)
        if (k < np) {
            CU(cudaMemcpyAsync(ctx->h_ctr + k, P.ctr, sizeof(StepCounters), cudaMemcpyDeviceToHost, ctx->stream));
            CU(cudaMemcpyAsync(ctx->h_pin + k++, P.pending_in_count, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               ctx->stream));
        }
    for (auto& P : ctx->p64)
        if (k < np) {
            CU(cudaMemcpyAsync(ctx->h_ctr + k, P.ctr, sizeof(StepCounters), cudaMemcpyDeviceToHost, ctx->stream));
            CU(cudaMemcpyAsync(ctx->h_pin + k++, P.pending_in_count, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               ctx->stream));
        }
    CU(cudaStreamSynchronize(ctx->stream));
    StepCounters total{};
    uint32_t pending = 0;
    auto acc = [&](const StepCounters& c, uint32_t pin) {
        total.removed += c.removed;
        total.migrated += c.migrated;
        total.injected += c.injected;
        total.lost += c.lost;
        total.timeouts += c.timeouts;
        total.pending_out += c.pending_out;
        pending += pin;
    };
    for (int i = 0; i < k; ++i) acc(ctx->h_ctr[i], ctx->h_pin[i]);
    ctx->last = total;
    ctx->pending_last = pending;
    if (total.lost) return fail(IPIC3D_E_CAPACITY, "%u particles lost: pending list full", total.lost);
    if (total.timeouts)
        return fail(IPIC3D_E_TIMEOUT, "%u thread blocks gave up waiting for a bulk copy", total.timeouts);
    // waiting particles are pushed and placed again every step (a cheap
    // path); re-lay out once they exceed 0.5% of the particles (or `force`)
    if (pending > std::max<uint64_t>(64, ctx->particles_hint / 200) || (pending && force_relayout))
        return relayout(ctx);
    return IPIC3D_OK;
}

int check_ctx(ipic3d_ctx* ctx) {
    if (!ctx) return fail(IPIC3D_E_INVALID, "context is NULL");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    return IPIC3D_OK;
}

int destroy_impl(ipic3d_ctx* ctx) {
    if (!ctx) return IPIC3D_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->dl_stream) cudaStreamSynchronize(ctx->dl_stream);
    drop_graph(ctx);
    release_pops(ctx);
    dfree(ctx->field);
    dfree(ctx->bcfield);
    dfree(ctx->J);
    dfree(ctx->rho);
    dfree(ctx->node32);
    dfree(ctx->cellcoef);
    dfree(ctx->d_step);
    dfree(ctx->d_partial);
    dfree(ctx->d_result);
    if (ctx->h_pending) cudaFreeHost(ctx->h_pending);
    if (ctx->h_ctr) cudaFreeHost(ctx->h_ctr);
    if (ctx->h_pin) cudaFreeHost(ctx->h_pin);
    dfree(ctx->st_parts);
    dfree(ctx->st_ids);
    dfree(ctx->st_sid);
    dfree(ctx->st_off);
    dfree(ctx->st_cnt);
    dfree(ctx->st_unknown);
    dfree(ctx->st_flags);
    dfree(ctx->st_dst);
    if (ctx->copy_ev) cudaEventDestroy(ctx->copy_ev);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    dfree(ctx->st_dl);
    dfree(ctx->st_dl_ids);
    if (ctx->dl_ev) cudaEventDestroy(ctx->dl_ev);
    if (ctx->dl_stream) cudaStreamDestroy(ctx->dl_stream);
    for (auto& e : ctx->aux_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
    for (auto& e : ctx->pend_ev)
        if (e) cudaEventDestroy(e);
    for (auto& pair : ctx->ph_ev)
        for (auto& e : pair)
            if (e) cudaEventDestroy(e);
    for (auto& e : ctx->tune_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream && ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return IPIC3D_OK;
}

// Creates a context; `shared` != NULL puts it on that stream (a universe of
// a batch), else it owns a new stream.
int create_impl(const ipic3d_props* props, const ipic3d_config* cfg, cudaStream_t shared, ipic3d_ctx** out) {
    if (!props || !cfg || !out) return fail(IPIC3D_E_INVALID, "NULL argument");
    *out = nullptr;
    for (int a = 0; a < 3; ++a) {
        if (props->size[a] <= 0) return fail(IPIC3D_E_INVALID, "size[%d] = %lld must be positive", a, (long long)props->size[a]);
        if (!(props->cell_width[a] > 0)) return fail(IPIC3D_E_INVALID, "cell_width[%d] must be positive", a);
        if ((cfg->bc_low[a] == IPIC3D_BC_PERIODIC) != (cfg->bc_high[a] == IPIC3D_BC_PERIODIC))
            return fail(IPIC3D_E_INVALID, "axis %d: periodic must apply to both faces", a);
        if (cfg->bc_low[a] < 0 || cfg->bc_low[a] > 2 || cfg->bc_high[a] < 0 || cfg->bc_high[a] > 2)
            return fail(IPIC3D_E_INVALID, "axis %d: unknown boundary", a);
    }
    if (!(props->dt > 0)) return fail(IPIC3D_E_INVALID, "dt must be positive");
    if (!(props->speed_of_light > 0)) return fail(IPIC3D_E_INVALID, "speed_of_light must be positive");
    if (props->planet_radius < 0) return fail(IPIC3D_E_INVALID, "planet_radius must be >= 0");
    if (cfg->precision != IPIC3D_FP64 && cfg->precision != IPIC3D_FP32) return fail(IPIC3D_E_INVALID, "precision");
    if (cfg->mover != IPIC3D_MOVER_DIPOLE && cfg->mover != IPIC3D_MOVER_FIELD) return fail(IPIC3D_E_INVALID, "mover");
    if (cfg->solver < 0 || cfg->solver > 2) return fail(IPIC3D_E_INVALID, "solver");
    if (cfg->projector < 0 || cfg->projector > 1) return fail(IPIC3D_E_INVALID, "projector");
    if (cfg->solver != IPIC3D_SOLVER_STATIC && !(props->size[0] == props->size[1] && props->size[1] == props->size[2]))
        return fail(IPIC3D_E_INVALID, "field solvers need a cubic grid (field.h:424)");
    const int64_t ncells = props->size[0] * props->size[1] * props->size[2];
    if (ncells > 0x7fffffff / 4) return fail(IPIC3D_E_INVALID, "grid too large");
    int dev = 0, ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(IPIC3D_E_NODEVICE, "no CUDA device");
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return fail(IPIC3D_E_NODEVICE, "cudaGetDeviceProperties");
    if (!(prop.major == 10 && prop.minor == 3))
        return fail(IPIC3D_E_NODEVICE, "device %d is sm_%d%d; this library is built for sm_103a only", dev,
                    prop.major, prop.minor);
    {
        const cudaError_t e = init_push32(dev);
        if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "push kernel set-up: %s", cudaGetErrorString(e));
    }
    auto* ctx = new (std::nothrow) ipic3d_ctx();
    if (!ctx) return fail(IPIC3D_E_NOMEM, "host allocation");
    ctx->props = *props;
    ctx->cfg = *cfg;
    ctx->device = dev;
    ctx->fp32 = cfg->precision == IPIC3D_FP32;
    auto bail = [&](int rc) {
        destroy_impl(ctx);
        return rc;
    };
#define CUB(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return bail(fail(e_ == cudaErrorMemoryAllocation ? IPIC3D_E_NOMEM : IPIC3D_E_CUDA, "%s: %s", #call, \
                             cudaGetErrorString(e_)));                                                    \
    } while (0)
    if (shared) {
        ctx->stream = shared;
        ctx->own_stream = false;
    } else {
        CUB(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    }
    CUB(cudaMalloc(&ctx->field, ctx->nfield() * 9 * sizeof(double)));
    CUB(cudaMalloc(&ctx->bcfield, ctx->nbc() * 3 * sizeof(double)));
    CUB(cudaMalloc(&ctx->J, ctx->nnode() * 3 * sizeof(double)));
    CUB(cudaMalloc(&ctx->rho, ctx->nnode() * sizeof(double)));
    CUB(cudaMalloc(&ctx->node32, ctx->nfield() * 2 * sizeof(float4)));
    CUB(cudaMalloc(&ctx->cellcoef, ncells * 48 * sizeof(float)));
    CUB(cudaMemsetAsync(ctx->cellcoef, 0, ncells * 48 * sizeof(float), ctx->stream));
    CUB(cudaMalloc(&ctx->d_step, sizeof(uint64_t)));
    CUB(cudaMalloc(&ctx->d_partial, (size_t)reduce_blocks() * 8 * sizeof(double)));
    CUB(cudaMalloc(&ctx->d_result, 8 * sizeof(double)));
    CUB(cudaMemsetAsync(ctx->field, 0, ctx->nfield() * 9 * sizeof(double), ctx->stream));
    CUB(cudaMemsetAsync(ctx->bcfield, 0, ctx->nbc() * 3 * sizeof(double), ctx->stream));
    CUB(cudaMemsetAsync(ctx->J, 0, ctx->nnode() * 3 * sizeof(double), ctx->stream));
    CUB(cudaMemsetAsync(ctx->rho, 0, ctx->nnode() * sizeof(double), ctx->stream));
    CUB(cudaMemsetAsync(ctx->node32, 0, ctx->nfield() * 2 * sizeof(float4), ctx->stream));
    CUB(cudaMemsetAsync(ctx->d_step, 0, sizeof(uint64_t), ctx->stream));
    CUB(cudaMallocHost(&ctx->h_pending, 2 * kMaxPops * sizeof(uint32_t)));
    CUB(cudaMallocHost(&ctx->h_ctr, kMaxPops * sizeof(StepCounters)));
    CUB(cudaMallocHost(&ctx->h_pin, kMaxPops * sizeof(uint32_t)));
    std::memset(ctx->h_pending, 0, 2 * kMaxPops * sizeof(uint32_t));
    for (auto& e : ctx->pend_ev) CUB(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto& e : ctx->tune_ev) CUB(cudaEventCreate(&e));
#undef CUB
    refresh_geom(ctx);
    // an empty particle set so that every call works before the first upload
    std::vector<uint64_t> zeros(ncells, 0);
    int rc = upload_impl(ctx, nullptr, zeros.data(), nullptr);
    if (rc) return bail(rc);
    *out = ctx;
    return IPIC3D_OK;
}

}  // namespace

// ============================================================================
extern "C" {

void ipic3d_gpu_config_default(ipic3d_config* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->precision = IPIC3D_FP64;
    cfg->mover = IPIC3D_MOVER_DIPOLE;
    cfg->solver = IPIC3D_SOLVER_STATIC;
    cfg->projector = IPIC3D_PROJECT_NONE;
    for (int a = 0; a < 3; ++a) cfg->bc_low[a] = cfg->bc_high[a] = IPIC3D_BC_REFLECT;
    cfg->seed = 12345;
}

int ipic3d_gpu_last_error(char* buf, size_t len) {
    if (buf && len) {
        std::strncpy(buf, g_last_msg, len - 1);
        buf[len - 1] = 0;
    }
    return g_last_status;
}

int ipic3d_gpu_create(const ipic3d_props* props, const ipic3d_config* cfg, ipic3d_ctx** out) {
    return create_impl(props, cfg, nullptr, out);
}

int ipic3d_gpu_destroy(ipic3d_ctx* ctx) {
    if (ctx && ctx->lent)
        return fail(IPIC3D_E_STATE, "this context is a universe of a batch: ipic3d_gpu_batch_destroy frees it");
    return destroy_impl(ctx);
}

int ipic3d_gpu_upload_particles(ipic3d_ctx* ctx, const ipic3d_particle* particles, const uint64_t* cell_counts,
                                const uint32_t* ids) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!cell_counts) return fail(IPIC3D_E_INVALID, "cell_counts == NULL");
    if (particles) {
        rc = upload_device(ctx, particles, cell_counts, ids);
        if (rc <= 0) return rc;  // done (0) or failed (< 0); 1 = take the host path
    }
    return upload_impl(ctx, particles, cell_counts, ids);
}

int ipic3d_gpu_init_uniform(ipic3d_ctx* ctx, uint64_t num_particles) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((rc = init_uniform_impl(ctx, num_particles))) return rc;
    CU(cudaStreamSynchronize(ctx->stream));
    return IPIC3D_OK;
}

int ipic3d_gpu_init_uniform_pos_normal_speed(ipic3d_ctx* ctx, uint64_t num_particles, const double low[3],
                                             const double hig[3], const double mean[3], const double stddev[3]) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!low || !hig || !mean || !stddev) return fail(IPIC3D_E_INVALID, "NULL argument");
    if ((rc = init_normal_impl(ctx, num_particles, low, hig, mean, stddev))) return rc;
    CU(cudaStreamSynchronize(ctx->stream));
    return IPIC3D_OK;
}

int ipic3d_gpu_reserve(ipic3d_ctx* ctx, uint64_t n) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    (void)n;  // capacity follows the per-cell slack; nothing to pre-size
    return IPIC3D_OK;
}

int ipic3d_gpu_particle_count(ipic3d_ctx* ctx, uint64_t* n) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!n) return fail(IPIC3D_E_INVALID, "n == NULL");
    std::vector<uint64_t> counts(ctx->ncells());
    if ((rc = ipic3d_gpu_cell_counts(ctx, counts.data()))) return rc;
    uint64_t t = 0;
    for (auto c : counts) t += c;
    *n = t;
    return IPIC3D_OK;
}

int ipic3d_gpu_cell_counts(ipic3d_ctx* ctx, uint64_t* cell_counts) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!cell_counts) return fail(IPIC3D_E_INVALID, "cell_counts == NULL");
    const int64_t nc = ctx->ncells();
    std::fill(cell_counts, cell_counts + nc, 0);
    std::vector<int32_t> h(nc);
    auto add = [&](const int32_t* dcount, const void* dpend, size_t msz, const uint32_t* dpin) -> int {
        CU(cudaMemcpyAsync(h.data(), dcount, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
        uint32_t np = 0;
        CU(cudaMemcpyAsync(&np, dpin, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
        for (int64_t c = 0; c < nc; ++c) cell_counts[c] += (uint64_t)h[c];
        if (np) {
            std::vector<char> buf((size_t)np * msz);
            CU(cudaMemcpy(buf.data(), dpend, buf.size(), cudaMemcpyDeviceToHost));
            for (uint32_t i = 0; i < np; ++i) cell_counts[*(const int32_t*)(buf.data() + (size_t)i * msz)] += 1;
        }
        return IPIC3D_OK;
    };
    for (auto& P : ctx->p32)
        if ((rc = add(P.count, P.pending_in, sizeof(Mover<float>), P.pending_in_count))) return rc;
    for (auto& P : ctx->p64)
        if ((rc = add(P.count, P.pending_in, sizeof(Mover<double>), P.pending_in_count))) return rc;
    return IPIC3D_OK;
}

int ipic3d_gpu_download_particles(ipic3d_ctx* ctx, ipic3d_particle* particles, uint64_t capacity,
                                  uint64_t* cell_counts, uint32_t* ids) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (ctx->fp32) return download_device(ctx, ctx->p32, particles, capacity, cell_counts, ids);
    return download_device(ctx, ctx->p64, particles, capacity, cell_counts, ids);
}

int ipic3d_gpu_download_particles_async(ipic3d_ctx* ctx, ipic3d_particle* particles, uint64_t capacity,
                                        uint64_t* cell_counts, uint32_t* ids) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (ctx->fp32) return download_device(ctx, ctx->p32, particles, capacity, cell_counts, ids, nullptr, true);
    return download_device(ctx, ctx->p64, particles, capacity, cell_counts, ids, nullptr, true);
}

int ipic3d_gpu_download_wait(ipic3d_ctx* ctx) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    return download_finish(ctx);
}

int ipic3d_gpu_download_positions(ipic3d_ctx* ctx, double* xyz, uint64_t capacity, uint64_t* cell_counts) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (ctx->fp32) return download_device(ctx, ctx->p32, nullptr, capacity, cell_counts, nullptr, xyz);
    return download_device(ctx, ctx->p64, nullptr, capacity, cell_counts, nullptr, xyz);
}

int ipic3d_gpu_upload_fields(ipic3d_ctx* ctx, const double* field, const double* bcfield, const double* density) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    if (field) CU(cudaMemcpyAsync(ctx->field, field, ctx->nfield() * 9 * sizeof(double), cudaMemcpyHostToDevice, st));
    if (bcfield) CU(cudaMemcpyAsync(ctx->bcfield, bcfield, ctx->nbc() * 3 * sizeof(double), cudaMemcpyHostToDevice, st));
    if (density) {
        CU(cudaMemcpyAsync(ctx->J, density, ctx->nnode() * 3 * sizeof(double), cudaMemcpyHostToDevice, st));
        // a supplied J is used as it is while the projector is off
    }
    if (field && ctx->fp32) {
        int n = launch_node32(ctx->g, ctx->node32, st);
        n += launch_cell_coef(ctx->g, ctx->cellcoef, st);
        if ((rc = check_launch(ctx, n))) return rc;
    }
    CU(cudaStreamSynchronize(st));
    return IPIC3D_OK;
}

int ipic3d_gpu_download_fields(ipic3d_ctx* ctx, double* field, double* bcfield, double* density, double* rho) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    if (field) CU(cudaMemcpyAsync(field, ctx->field, ctx->nfield() * 9 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (bcfield) CU(cudaMemcpyAsync(bcfield, ctx->bcfield, ctx->nbc() * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (density) CU(cudaMemcpyAsync(density, ctx->J, ctx->nnode() * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (rho) CU(cudaMemcpyAsync(rho, ctx->rho, ctx->nnode() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return IPIC3D_OK;
}

int ipic3d_gpu_step(ipic3d_ctx* ctx, uint64_t num_steps) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (num_steps == 0) return IPIC3D_OK;
    if (ctx->cfg.projector == IPIC3D_PROJECT_CIC && !ctx->j_valid)
        if ((rc = project_impl(ctx))) return rc;
    const bool use_graph = (ctx->cfg.flags & IPIC3D_F_USE_GRAPH) != 0 && !ctx->profiling;
    // re-lay out when more than 0.5% of the particles wait for a slot
    const uint64_t pend_limit = std::max<uint64_t>(64, ctx->particles_hint / 200);
    uint64_t watch_from = 0;  // first step whose pending count is still meaningful
    tune_prepare(ctx);
    // a run of graph steps with a field solver solves the next step's fields
    // beside the current step's placement: the first solve alone, the last
    // step without a solve after it
    const bool overlap = use_graph && ctx->cfg.solver != IPIC3D_SOLVER_STATIC;
    bool presolved = false;
    for (uint64_t done = 0; done < num_steps;) {
        if (ctx->tuner.running()) {  // a trial step of the autotuner: outside the graph, push timed
            ctx->tune_timing = true;
            rc = enqueue_step(ctx);
            ctx->tune_timing = false;
            if (rc) return rc;
            if ((rc = ph_collect(ctx))) return rc;
            if ((rc = tune_record(ctx))) return rc;
        } else if (overlap && (presolved || done + 1 < num_steps)) {
            if (!presolved && (rc = run_graph(ctx, kStepSolve))) return rc;
            const bool last = done + 1 == num_steps;
            if ((rc = run_graph(ctx, last ? kStepMove : kStepMoveSolve))) return rc;
            presolved = !last;
        } else if (use_graph) {  // a lone step (or no field solver): one graph
            if ((rc = run_graph(ctx, kStepFull))) return rc;
        } else {
            if ((rc = enqueue_step(ctx))) return rc;
            if ((rc = ph_collect(ctx))) return rc;
        }
        // this step's pending count -> pinned slot (done & 1)
        const int slot = (int)(done & 1);
        int k = 0;
        for (auto& P : ctx->p32)
            if (k < kMaxPops)
                CU(cudaMemcpyAsync(ctx->h_pending + slot * kMaxPops + k++, &P.ctr->pending_out, sizeof(uint32_t),
                                   cudaMemcpyDeviceToHost, ctx->stream));
        for (auto& P : ctx->p64)
            if (k < kMaxPops)
                CU(cudaMemcpyAsync(ctx->h_pending + slot * kMaxPops + k++, &P.ctr->pending_out, sizeof(uint32_t),
                                   cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaEventRecord(ctx->pend_ev[slot], ctx->stream));
        ++done;
        ++ctx->steps;
        // the previous step's count (the GPU works on this step meanwhile)
        if (done >= 2 && done - 2 >= watch_from && done < num_steps) {
            const int ps = (int)((done - 2) & 1);
            CU(cudaEventSynchronize(ctx->pend_ev[ps]));
            uint64_t pend = 0;
            for (int q = 0; q < k; ++q) pend += ctx->h_pending[ps * kMaxPops + q];
            if (pend > pend_limit) {
                ctx->relayout_steps += 1;
                if ((rc = after_steps(ctx))) return rc;  // waits, then re-lays out
                watch_from = done;  // counts recorded before the re-layout are stale
            }
        }
    }
    return after_steps(ctx);
}

int ipic3d_gpu_project(ipic3d_ctx* ctx) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((rc = project_impl(ctx))) return rc;
    CU(cudaStreamSynchronize(ctx->stream));
    return IPIC3D_OK;
}

int ipic3d_gpu_update_boundaries(ipic3d_ctx* ctx) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (ctx->props.size[0] != ctx->props.size[1] || ctx->props.size[1] != ctx->props.size[2])
        return fail(IPIC3D_E_INVALID, "updateFieldsOnBoundaries assumes a cubic grid (field.h:424)");
    int n = launch_ghost(ctx->g, ctx->stream);
    if ((rc = check_launch(ctx, n))) return rc;
    CU(cudaStreamSynchronize(ctx->stream));
    return IPIC3D_OK;
}

int ipic3d_gpu_solve_fields(ipic3d_ctx* ctx) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((rc = solve_impl(ctx))) return rc;
    CU(cudaStreamSynchronize(ctx->stream));
    return IPIC3D_OK;
}

int ipic3d_gpu_move(ipic3d_ctx* ctx) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if ((rc = move_impl(ctx, false))) return rc;
    ctx->j_valid = false;
    return after_steps(ctx);
}

int ipic3d_gpu_conserved(ipic3d_ctx* ctx, ipic3d_conserved* out) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out) return fail(IPIC3D_E_INVALID, "out == NULL");
    cudaStream_t st = ctx->stream;
    const int nb = reduce_blocks();
    double res[3] = {0, 0, 0}, fres[2] = {0, 0};
    double tot[3] = {0, 0, 0};
    int n = 0;
    auto one = [&](auto& P) -> int {
        n += launch_reduce_particles(P.view(), (int)ctx->ncells(), ctx->d_partial, st);
        n += launch_reduce_final(ctx->d_partial, nb, 3, ctx->d_result, st);
        CU(cudaMemcpyAsync(res, ctx->d_result, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        for (int k = 0; k < 3; ++k) tot[k] += res[k];
        return IPIC3D_OK;
    };
    for (auto& P : ctx->p32)
        if ((rc = one(P))) return rc;
    for (auto& P : ctx->p64)
        if ((rc = one(P))) return rc;
    n += launch_reduce_fields(ctx->g, ctx->d_partial, st);
    n += launch_reduce_final(ctx->d_partial, nb, 2, ctx->d_result, st);
    CU(cudaMemcpyAsync(fres, ctx->d_result, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if ((rc = check_launch(ctx, n))) return rc;
    out->total_momentum = tot[0];
    out->kinetic_energy = tot[1];
    out->total_charge = tot[2];
    out->e_energy = fres[0];
    out->b_energy = fres[1];
    uint64_t np = 0;
    if ((rc = ipic3d_gpu_particle_count(ctx, &np))) return rc;
    out->particles = np;
    return IPIC3D_OK;
}

int ipic3d_gpu_synchronize(ipic3d_ctx* ctx) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    CU(cudaStreamSynchronize(ctx->stream));
    return IPIC3D_OK;
}

void* ipic3d_gpu_stream(ipic3d_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int ipic3d_gpu_stats(ipic3d_ctx* ctx, ipic3d_stats* out) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out) return fail(IPIC3D_E_INVALID, "out == NULL");
    std::memset(out, 0, sizeof(*out));
    out->steps = ctx->steps;
    uint64_t np = 0;
    if ((rc = ipic3d_gpu_particle_count(ctx, &np))) return rc;
    out->particles = np;
    for (auto& P : ctx->p32) out->capacity += (uint64_t)P.capacity;
    for (auto& P : ctx->p64) out->capacity += (uint64_t)P.capacity;
    out->migrated_last = ctx->last.migrated;
    out->removed_last = ctx->last.removed;
    out->injected_last = ctx->last.injected;
    out->rebuilds = ctx->rebuilds;
    out->kernel_launches = ctx->launches;
    out->pending_last = ctx->pending_last;
    out->relayout_steps = ctx->relayout_steps;
    return IPIC3D_OK;
}

int ipic3d_gpu_profile(ipic3d_ctx* ctx, int enable) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (enable && !ctx->ph_ev[0][0])
        for (auto& pair : ctx->ph_ev)
            for (auto& e : pair) CU(cudaEventCreate(&e));
    ctx->profiling = enable != 0;
    return IPIC3D_OK;
}

int ipic3d_gpu_profile_read(ipic3d_ctx* ctx, ipic3d_profile* out, int reset) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out) return fail(IPIC3D_E_INVALID, "out == NULL");
    *out = ctx->prof;
    if (reset) std::memset(&ctx->prof, 0, sizeof(ctx->prof));
    return IPIC3D_OK;
}

int ipic3d_gpu_get_push_shape(ipic3d_ctx* ctx, ipic3d_push_shape* out) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out) return fail(IPIC3D_E_INVALID, "out == NULL");
    std::memset(out, 0, sizeof(*out));
    const PushShape& s = ctx->tuner.shape();
    out->item = s.item;
    out->item_cells = s.item_cells;
    out->blocks_per_sm = s.per_sm;
    out->tuned = ctx->tuner.tuned() ? 1 : 0;
    out->tuning = ctx->tuner.running() ? 1 : 0;
    out->trials = ctx->tuner.trials();
    out->push_ms = ctx->tuner.best_ms();
    return IPIC3D_OK;
}

int ipic3d_gpu_set_push_shape(ipic3d_ctx* ctx, const ipic3d_push_shape* shape) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    drop_graph(ctx);  // captured with the previous shape
    if (shape) {
        if (shape->item <= 0 || shape->item_cells < 0 || shape->blocks_per_sm <= 0)
            return fail(IPIC3D_E_INVALID, "push shape: item and blocks_per_sm must be positive, item_cells >= 0");
        ctx->tuner.fix(PushShape{shape->item, shape->item_cells, shape->blocks_per_sm});
        ctx->shape_fixed = true;
        return IPIC3D_OK;
    }
    ctx->shape_fixed = false;
    ctx->tuned_particles = 0;
    if (ctx->fp32 && ctx->particles_hint > 0) {
        ctx->tuned_particles = ctx->particles_hint;
        ctx->tuner.start(push32_blocks_per_sm(ctx->device));
    } else {
        ctx->tuner.fix(kDefaultPushShape);
    }
    return IPIC3D_OK;
}

int ipic3d_gpu_set_wait_limit(ipic3d_ctx* ctx, int64_t polls) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    drop_graph(ctx);  // captured with the previous bound
    ctx->wait_polls = polls < 0 ? -1 : (int32_t)std::min<int64_t>(polls, INT32_MAX);
    return IPIC3D_OK;
}

int ipic3d_gpu_boris(ipic3d_particle* particles, uint64_t n, const double E[3], const double B[3], double dt,
                     uint64_t nsteps, int push_position) {
    if (!particles || !E || !B) return fail(IPIC3D_E_INVALID, "NULL argument");
    if (n == 0) return IPIC3D_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(IPIC3D_E_NODEVICE, "no CUDA device");
    void* d = nullptr;
    CU(cudaMalloc(&d, n * sizeof(ipic3d_particle)));
    cudaError_t e = cudaMemcpy(d, particles, n * sizeof(ipic3d_particle), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_boris(d, n, E, B, dt, nsteps, push_position, d, nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(particles, d, n * sizeof(ipic3d_particle), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "boris: %s", cudaGetErrorString(e));
    return IPIC3D_OK;
}

}  // extern "C"

// ============================================================================
// Batched ensemble: independent universes advanced by one launch per kernel.
//
// Each universe is an ordinary context on the batch's stream. Before a
// batched step the host lists every (universe, species) population as a
// PopJob (its Geom, its Pop view and push constants) and every universe as
// an InstJob, plus two block maps: push CTA -> (job, CTA of the job) and
// placement block -> (job, block of the job). The tables are rebuilt only when a
// population's layout changed (upload, re-layout): the host compares the
// job records byte for byte.

struct ipic3d_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    ipic3d_config cfg{};
    bool fp32 = false;
    std::vector<ipic3d_ctx*> inst;
    // host copies of the device tables
    std::vector<PopJob<float>> j32;
    std::vector<PopJob<double>> j64;
    std::vector<InstJob> ij;
    char* d_jobs = nullptr;
    size_t d_jobs_cap = 0;
    InstJob* d_inst = nullptr;
    size_t d_inst_cap = 0;
    int2* d_cta = nullptr;
    size_t d_cta_cap = 0;
    int2* d_place = nullptr;
    size_t d_place_cap = 0;
    JobStatus* d_status = nullptr;
    size_t d_status_cap = 0;
    uint32_t* d_flag = nullptr;  // universes over their pending limit (this step)
    uint32_t* h_flag = nullptr;  // pinned ring of two
    cudaEvent_t flag_ev[2] = {nullptr, nullptr};
    int64_t nctas = 0, nplace = 0;
    int max_s = 0;
    int64_t max_cells = 0, max_nodes = 0;
    bool tables = false;
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    uint64_t graph_kernels = 0;
    uint64_t steps = 0, launches = 0;
    // second stream: the pending push beside the push, the J finalisation
    // beside the placement (as a context's step)
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t aux_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // launch shape of the FP32 batched push (autotuned as a context's)
    PushTuner tuner;
    bool tune_started = false;
    bool tune_timing = false;
    cudaEvent_t tune_ev[2] = {nullptr, nullptr};
};

namespace {

TuneKey batch_tune_key(const ipic3d_batch* b, uint64_t particles, int64_t cells) {
    return tune_key(b->device, 1, (int64_t)b->inst.size(), cells, 0, (int)(b->fp32 ? b->j32.size() : b->j64.size()),
                    particles, b->cfg);
}

void batch_drop_graph(ipic3d_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_valid = false;
}

template <typename T>
std::vector<PopStore<T>>& pops_of(ipic3d_ctx* c);
template <>
std::vector<PopStore<float>>& pops_of<float>(ipic3d_ctx* c) { return c->p32; }
template <>
std::vector<PopStore<double>>& pops_of<double>(ipic3d_ctx* c) { return c->p64; }

template <typename T>
std::vector<PopJob<T>>& jobs_of(ipic3d_batch* b);
template <>
std::vector<PopJob<float>>& jobs_of<float>(ipic3d_batch* b) { return b->j32; }
template <>
std::vector<PopJob<double>>& jobs_of<double>(ipic3d_batch* b) { return b->j64; }

template <typename T>
void fill_consts(PopJob<T>& J);
template <>
void fill_consts<float>(PopJob<float>& J) { J.pc = push32_const(J.g, J.P); }
template <>
void fill_consts<double>(PopJob<double>&) {}

// Builds the job records; uploads them (and the block maps) when they differ
// from the ones on the device.
template <typename T>
int batch_tables(ipic3d_batch* b) {
    std::vector<PopJob<T>> nj;
    std::vector<InstJob> ni(b->inst.size());
    const ipic3d_config& cfg = b->cfg;
    for (size_t i = 0; i < b->inst.size(); ++i) {
        ipic3d_ctx* c = b->inst[i];
        InstJob& I = ni[i];
        std::memset(&I, 0, sizeof(I));
        I.g = c->g;
        I.g.deposit = cfg.projector == IPIC3D_PROJECT_CIC ? 1 : 0;
        I.step = c->d_step;
        I.job0 = (int)nj.size();
        I.njobs = (int)pops_of<T>(c).size();
        I.pend_limit = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(64, c->particles_hint / 200), 0xffffffffu);
        I.div8 = (cfg.flags & IPIC3D_F_J_DIV8) ? 1 : 0;
        I.refresh_b = (cfg.flags & IPIC3D_F_REFRESH_NODE_B) ? 1 : 0;
        I.cellcoef = c->cellcoef;
        I.coef_scale = (cfg.flags & IPIC3D_F_GATHER_DIV_VOL) ? 1.0 / c->g.vol : 1.0;
        for (auto& P : pops_of<T>(c)) {
            PopJob<T> J;
            std::memset(&J, 0, sizeof(J));
            J.g = I.g;
            J.P = P.view();
            fill_consts<T>(J);
            J.sort_tmp = P.sort_tmp;
            J.pend_count = P.pending_in_count;
            nj.push_back(J);
        }
    }
    auto& cur = jobs_of<T>(b);
    if (b->tables && cur.size() == nj.size() && b->ij.size() == ni.size() &&
        std::memcmp(cur.data(), nj.data(), nj.size() * sizeof(PopJob<T>)) == 0 &&
        std::memcmp(b->ij.data(), ni.data(), ni.size() * sizeof(InstJob)) == 0)
        return IPIC3D_OK;
    if (nj.size() > 65535) return fail(IPIC3D_E_INVALID, "batch: more than 65535 populations");
    std::vector<int2> cta, place;
    int max_s = 1;
    int64_t max_cells = 1, max_nodes = 1;
    for (size_t j = 0; j < nj.size(); ++j) {
        const int64_t nb = (nj[j].P.capacity + kSlotsPerCta - 1) / kSlotsPerCta;
        for (int64_t k = 0; k < nb; ++k) cta.push_back(make_int2((int)j, (int)k));
        const int npb = place_blocks(nj[j].g.ncells);
        for (int k = 0; k < npb; ++k) place.push_back(make_int2((int)j, k));
    }
    for (auto& I : ni) {
        max_s = std::max(max_s, std::max(I.g.sx, std::max(I.g.sy, I.g.sz)));
        max_cells = std::max<int64_t>(max_cells, I.g.ncells);
        max_nodes = std::max<int64_t>(max_nodes, (int64_t)(I.g.sx + 1) * (I.g.sy + 1) * (I.g.sz + 1));
    }
    if (cta.size() > 0x7fffffffu || place.size() > 0x7fffffffu) return fail(IPIC3D_E_INVALID, "batch too large");
    int rc;
    size_t jb = b->d_jobs_cap;
    if ((rc = grow(b->d_jobs, jb, std::max<size_t>(1, nj.size()) * sizeof(PopJob<T>)))) return rc;
    b->d_jobs_cap = jb;
    if ((rc = grow(b->d_inst, b->d_inst_cap, ni.size()))) return rc;
    if ((rc = grow(b->d_cta, b->d_cta_cap, std::max<size_t>(1, cta.size())))) return rc;
    if ((rc = grow(b->d_place, b->d_place_cap, std::max<size_t>(1, place.size())))) return rc;
    if ((rc = grow(b->d_status, b->d_status_cap, std::max<size_t>(1, nj.size())))) return rc;
    cudaStream_t st = b->stream;
    CU(cudaMemcpyAsync(b->d_jobs, nj.data(), nj.size() * sizeof(PopJob<T>), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(b->d_inst, ni.data(), ni.size() * sizeof(InstJob), cudaMemcpyHostToDevice, st));
    if (!cta.empty()) CU(cudaMemcpyAsync(b->d_cta, cta.data(), cta.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
    if (!place.empty())
        CU(cudaMemcpyAsync(b->d_place, place.data(), place.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
    CU(cudaStreamSynchronize(st));  // the host vectors die here
    cur.swap(nj);
    b->ij.swap(ni);
    b->nctas = (int64_t)cta.size();
    b->nplace = (int64_t)place.size();
    b->max_s = max_s;
    b->max_cells = max_cells;
    b->max_nodes = max_nodes;
    b->tables = true;
    batch_drop_graph(b);
    return IPIC3D_OK;
}

// One batched timestep (the body the graph captures); the kernel order of
// enqueue_step per universe.
template <typename T>
int batch_enqueue_step(ipic3d_batch* b) {
    cudaStream_t st = b->stream;
    const ipic3d_config& cfg = b->cfg;
    const PopJob<T>* jobs = reinterpret_cast<const PopJob<T>*>(b->d_jobs);
    const int ni = (int)b->inst.size(), nj = (int)jobs_of<T>(b).size();
    const int deposit = cfg.projector == IPIC3D_PROJECT_CIC ? 1 : 0;
    int n = 0;
    if (cfg.solver != IPIC3D_SOLVER_STATIC) {
        n += launch_ghost_batch(b->d_inst, ni, b->max_s, st);
        if (cfg.solver == IPIC3D_SOLVER_LEAPFROG)
            n += launch_leapfrog_batch(b->d_inst, ni, b->max_s, (cfg.flags & IPIC3D_F_REFRESH_NODE_B) != 0, st);
        else
            n += launch_forward_batch(b->d_inst, ni, b->max_s, st);
        if (b->fp32 && cfg.mover == IPIC3D_MOVER_FIELD) n += launch_cell_coef_batch(b->d_inst, ni, b->max_cells, st);
    }
    n += launch_batch_begin<T>(jobs, nj, b->d_inst, ni, b->max_nodes, deposit, b->d_flag, st);
    cudaStream_t aux = b->aux_stream;
    auto fork = [&](int e, cudaStream_t from, cudaStream_t to) -> int {
        CU(cudaEventRecord(b->aux_ev[e], from));
        CU(cudaStreamWaitEvent(to, b->aux_ev[e], 0));
        return IPIC3D_OK;
    };
    int rc;
    if (nj > 0) {
        if ((rc = fork(0, st, aux))) return rc;
        if (b->tune_timing) CU(cudaEventRecord(b->tune_ev[0], st));
        n += launch_push_batch<T>(jobs, b->d_cta, b->nctas, 0, jobs_of<T>(b)[0].g, b->tuner.next(), st);
        if (b->tune_timing) CU(cudaEventRecord(b->tune_ev[1], st));
        n += launch_push_pending_batch<T>(jobs, nj, aux);
        if ((rc = fork(1, aux, st))) return rc;
    }
    if (deposit) {
        if ((rc = fork(2, st, aux))) return rc;
        n += launch_j_finalize_batch(b->d_inst, ni, b->max_cells, aux);
    }
    if (nj > 0) {
        n += launch_place_batch<T>(jobs, b->d_place, b->nplace, st);
        n += launch_pending_rotate_batch<T>(jobs, nj, st);
    }
    if (deposit && (rc = fork(3, aux, st))) return rc;
    n += launch_batch_end<T>(jobs, b->d_inst, ni, b->d_flag, st);
    b->launches += (uint64_t)n;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "batched kernel launch: %s", cudaGetErrorString(e));
    return IPIC3D_OK;
}

// Reads every job's counters back; per universe: the step statistics, lost
// particles (an error) and the re-layout when too many particles wait.
template <typename T>
int batch_after(ipic3d_batch* b) {
    const auto& jobs = jobs_of<T>(b);
    const int nj = (int)jobs.size();
    if (nj == 0) return IPIC3D_OK;
    cudaStream_t st = b->stream;
    std::vector<JobStatus> hs(nj);
    int n = launch_batch_status<T>(reinterpret_cast<const PopJob<T>*>(b->d_jobs), nj, b->d_status, st);
    b->launches += (uint64_t)n;
    CU(cudaMemcpyAsync(hs.data(), b->d_status, nj * sizeof(JobStatus), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    for (size_t i = 0; i < b->inst.size(); ++i) {
        ipic3d_ctx* c = b->inst[i];
        const InstJob& I = b->ij[i];
        StepCounters tot{};
        uint64_t pending = 0;
        for (int j = I.job0; j < I.job0 + I.njobs; ++j) {
            const StepCounters& s = hs[j].c;
            tot.removed += s.removed;
            tot.migrated += s.migrated;
            tot.injected += s.injected;
            tot.lost += s.lost;
            tot.pending_out += s.pending_out;
            pending += hs[j].pending_in;
        }
        c->last = tot;
        c->pending_last = pending;
        if (tot.lost) return fail(IPIC3D_E_CAPACITY, "universe %zu: %u particles lost: pending list full", i, tot.lost);
        if (pending > I.pend_limit) {
            c->relayout_steps += 1;
            int rc = relayout(c);
            if (rc) return rc;
        }
    }
    return IPIC3D_OK;
}

template <typename T>
int batch_run(ipic3d_batch* b, uint64_t num_steps) {
    int rc;
    if ((rc = batch_tables<T>(b))) return rc;
    const bool use_graph = (b->cfg.flags & IPIC3D_F_USE_GRAPH) != 0;
    cudaStream_t st = b->stream;
    // the first batched run with particles tunes the push shape (or takes a
    // cached one)
    if (b->fp32 && b->cfg.block_size == 0 && !b->tune_started && !jobs_of<T>(b).empty()) {
        uint64_t particles = 0;
        int64_t cells = 0;
        for (auto* c : b->inst) {
            particles += c->particles_hint;
            cells += c->ncells();
        }
        if (particles > 0) {
            b->tune_started = true;
            batch_drop_graph(b);
            if (!tune_lookup(batch_tune_key(b, particles, cells), b->tuner))
                b->tuner.start(push32_blocks_per_sm(b->device));
        }
    }
    uint64_t watch_from = 0;
    for (uint64_t done = 0; done < num_steps;) {
        if (b->tuner.running()) {  // a trial step of the autotuner: outside the graph, push timed
            b->tune_timing = true;
            rc = batch_enqueue_step<T>(b);
            b->tune_timing = false;
            if (rc) return rc;
            CU(cudaEventSynchronize(b->tune_ev[1]));
            float ms = 0.f;
            CU(cudaEventElapsedTime(&ms, b->tune_ev[0], b->tune_ev[1]));
            b->tuner.record(ms);
            if (!b->tuner.running()) {
                uint64_t particles = 0;
                int64_t cells = 0;
                for (auto* c : b->inst) {
                    particles += c->particles_hint;
                    cells += c->ncells();
                }
                tune_store(batch_tune_key(b, particles, cells), b->tuner);
                batch_drop_graph(b);
            }
        } else if (use_graph) {
            if (!b->graph_valid) {
                cudaGraph_t graph = nullptr;
                CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                const uint64_t before = b->launches;
                rc = batch_enqueue_step<T>(b);
                b->graph_kernels = b->launches - before;
                b->launches = before;  // capturing runs nothing
                cudaError_t e = cudaStreamEndCapture(st, &graph);
                if (rc) {
                    if (graph) cudaGraphDestroy(graph);
                    return rc;
                }
                if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
                e = cudaGraphInstantiate(&b->graph, graph, 0);
                cudaGraphDestroy(graph);
                if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "batch graph instantiate: %s", cudaGetErrorString(e));
                b->graph_valid = true;
            }
            CU(cudaGraphLaunch(b->graph, st));
            b->launches += b->graph_kernels;
        } else if ((rc = batch_enqueue_step<T>(b))) {
            return rc;
        }
        const int slot = (int)(done & 1);
        CU(cudaMemcpyAsync(b->h_flag + slot, b->d_flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CU(cudaEventRecord(b->flag_ev[slot], st));
        ++done;
        ++b->steps;
        for (auto* c : b->inst) ++c->steps;
        // the previous step's flag (this step runs meanwhile)
        if (done >= 2 && done - 2 >= watch_from && done < num_steps) {
            const int ps = (int)((done - 2) & 1);
            CU(cudaEventSynchronize(b->flag_ev[ps]));
            if (b->h_flag[ps]) {
                if ((rc = batch_after<T>(b))) return rc;
                if ((rc = batch_tables<T>(b))) return rc;
                watch_from = done;
            }
        }
    }
    return batch_after<T>(b);
}

int batch_check(ipic3d_batch* b) {
    if (!b) return fail(IPIC3D_E_INVALID, "batch is NULL");
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return fail(IPIC3D_E_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    return IPIC3D_OK;
}

void batch_free(ipic3d_batch* b) {
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_drop_graph(b);
    for (auto* c : b->inst) {
        c->lent = false;
        destroy_impl(c);
    }
    b->inst.clear();
    dfree(b->d_jobs);
    dfree(b->d_inst);
    dfree(b->d_cta);
    dfree(b->d_place);
    dfree(b->d_status);
    dfree(b->d_flag);
    if (b->h_flag) cudaFreeHost(b->h_flag);
    for (auto& e : b->flag_ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : b->tune_ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : b->aux_ev)
        if (e) cudaEventDestroy(e);
    if (b->aux_stream) cudaStreamDestroy(b->aux_stream);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

}  // namespace

extern "C" {

int ipic3d_gpu_batch_create(uint32_t count, const ipic3d_props* props, const ipic3d_config* cfg,
                            ipic3d_batch** out) {
    if (!props || !cfg || !out) return fail(IPIC3D_E_INVALID, "NULL argument");
    *out = nullptr;
    if (count == 0 || count > 65535) return fail(IPIC3D_E_INVALID, "batch of %u universes (1 to 65535)", count);
    if (cfg->flags & IPIC3D_F_INJECT_LOW_X) return fail(IPIC3D_E_INVALID, "injection is not supported in a batch");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(IPIC3D_E_NODEVICE, "no CUDA device");
    auto* b = new (std::nothrow) ipic3d_batch();
    if (!b) return fail(IPIC3D_E_NOMEM, "host allocation");
    cudaGetDevice(&b->device);
    b->cfg = *cfg;
    b->fp32 = cfg->precision == IPIC3D_FP32;
    auto bail = [&](int rc) {
        batch_free(b);
        return rc;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_flag, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_flag, 0, sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_flag, 2 * sizeof(uint32_t));
    for (auto& ev : b->flag_ev)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    for (auto& ev : b->tune_ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->aux_stream, cudaStreamNonBlocking);
    for (auto& ev : b->aux_ev)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess)
        return bail(fail(e == cudaErrorMemoryAllocation ? IPIC3D_E_NOMEM : IPIC3D_E_CUDA, "batch: %s",
                         cudaGetErrorString(e)));
    b->h_flag[0] = b->h_flag[1] = 0;
    b->inst.reserve(count);
    for (uint32_t i = 0; i < count; ++i) {
        ipic3d_ctx* c = nullptr;
        int rc = create_impl(props + i, cfg, b->stream, &c);
        if (rc) {
            char msg[512];
            std::snprintf(msg, sizeof msg, "universe %u: %s", i, g_last_msg);
            bail(rc);
            return fail(rc, "%s", msg);
        }
        c->lent = true;
        b->inst.push_back(c);
    }
    *out = b;
    return IPIC3D_OK;
}

int ipic3d_gpu_batch_destroy(ipic3d_batch* b) {
    if (!b) return IPIC3D_OK;
    batch_free(b);
    return IPIC3D_OK;
}

int ipic3d_gpu_batch_size(ipic3d_batch* b, uint32_t* count) {
    int rc = batch_check(b);
    if (rc) return rc;
    if (!count) return fail(IPIC3D_E_INVALID, "count == NULL");
    *count = (uint32_t)b->inst.size();
    return IPIC3D_OK;
}

int ipic3d_gpu_batch_universe(ipic3d_batch* b, uint32_t index, ipic3d_ctx** out) {
    int rc = batch_check(b);
    if (rc) return rc;
    if (!out) return fail(IPIC3D_E_INVALID, "out == NULL");
    if (index >= b->inst.size()) return fail(IPIC3D_E_INVALID, "universe %u of %zu", index, b->inst.size());
    *out = b->inst[index];
    return IPIC3D_OK;
}

int ipic3d_gpu_batch_step(ipic3d_batch* b, uint64_t num_steps) {
    int rc = batch_check(b);
    if (rc) return rc;
    if (num_steps == 0) return IPIC3D_OK;
    // universes whose J is stale get their projection first, as in ipic3d_gpu_step
    if (b->cfg.projector == IPIC3D_PROJECT_CIC)
        for (auto* c : b->inst)
            if (!c->j_valid && (rc = project_impl(c))) return rc;
    return b->fp32 ? batch_run<float>(b, num_steps) : batch_run<double>(b, num_steps);
}

int ipic3d_gpu_batch_synchronize(ipic3d_batch* b) {
    int rc = batch_check(b);
    if (rc) return rc;
    CU(cudaStreamSynchronize(b->stream));
    return IPIC3D_OK;
}

void* ipic3d_gpu_batch_stream(ipic3d_batch* b) { return b ? (void*)b->stream : nullptr; }

int ipic3d_gpu_batch_stats(ipic3d_batch* b, ipic3d_stats* out) {
    int rc = batch_check(b);
    if (rc) return rc;
    if (!out) return fail(IPIC3D_E_INVALID, "out == NULL");
    std::memset(out, 0, sizeof(*out));
    for (auto* c : b->inst) {
        ipic3d_stats s;
        if ((rc = ipic3d_gpu_stats(c, &s))) return rc;
        out->particles += s.particles;
        out->capacity += s.capacity;
        out->migrated_last += s.migrated_last;
        out->removed_last += s.removed_last;
        out->injected_last += s.injected_last;
        out->rebuilds += s.rebuilds;
        out->pending_last += s.pending_last;
        out->relayout_steps += s.relayout_steps;
    }
    out->steps = b->steps;
    out->kernel_launches = b->launches;
    return IPIC3D_OK;
}

int ipic3d_gpu_batch_get_push_shape(ipic3d_batch* b, ipic3d_push_shape* out) {
    int rc = batch_check(b);
    if (rc) return rc;
    if (!out) return fail(IPIC3D_E_INVALID, "out == NULL");
    std::memset(out, 0, sizeof(*out));
    const PushShape& s = b->tuner.shape();
    out->item = s.item;
    out->item_cells = s.item_cells;
    out->blocks_per_sm = s.per_sm;
    out->tuned = b->tuner.tuned() ? 1 : 0;
    out->tuning = b->tuner.running() ? 1 : 0;
    out->trials = b->tuner.trials();
    out->push_ms = b->tuner.best_ms();
    return IPIC3D_OK;
}

}  // extern "C"
