// Particle initialisation on the device with the reference's own random
// streams: initCells(properties, numParticles, uniform<>) (cell.h:638-697),
// the universe of the reference's ":U:N" benchmark mode, and phase 2 of
// initCells<Distribution> (cell.h:596-632) for the .inp driver's
// uniform_pos_normal_speed distribution (src/ipic3d.cxx:76-82).
//
// initCells(uniform):
// Cell pos gets floor(N / cells) particles (+1 for the first N mod cells
// cells in row-major order); its positions come from a std::minstd_rand
// seeded with seed + 1 and its velocities from one seeded with seed + 2,
// seed = (uint32)((x * 1023 + y) * 1023 + z) (cell.h:663-674,
// generic_particle_generator and vector::uniform at cell.h:138-174, 262-330);
// each coordinate is a std::uniform_real_distribution<double>(lo, hi) draw.
// Here the streams are replayed in parallel: thread i of a cell jumps its two
// generators ahead by 6 i draws (x_{n+k} = a^k x_n mod m, a^k by squaring)
// and draws its particle's six coordinates. The arithmetic is the one the
// reference's standard library performs (libstdc++'s generate_canonical with
// two 31-bit draws, then lo + (hi - lo) * u), with every FP64 operation
// rounded separately (built with -fmad=false, explicit _rn intrinsics): the
// particles are bit-identical to the reference's.
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "../../include/ipic3d_types.h"
#include "launch.h"

namespace ipg {

namespace {

constexpr uint64_t kLcgA = 48271u, kLcgM = 2147483647u;  // std::minstd_rand
constexpr double kLcgRange = 2147483646.0;               // max - min + 1

__device__ __forceinline__ uint64_t lcg_mulmod(uint64_t a, uint64_t b) { return (a * b) % kLcgM; }

// a^k mod m
__device__ __forceinline__ uint64_t lcg_pow(uint64_t k) {
    uint64_t r = 1, b = kLcgA;
    while (k) {
        if (k & 1) r = lcg_mulmod(r, b);
        b = lcg_mulmod(b, b);
        k >>= 1;
    }
    return r;
}

// linear_congruential_engine::seed: s mod m, or 1 when that is 0
__device__ __forceinline__ uint64_t lcg_seed(uint32_t s) {
    const uint64_t x = (uint64_t)s % kLcgM;
    return x == 0 ? 1 : x;
}

// generate_canonical<double, 53>: k = 2 draws, sum (d_i - min) r^i, / r^2
__device__ __forceinline__ double canonical(uint64_t& x) {
    x = lcg_mulmod(x, kLcgA);
    double sum = __dadd_rn(0.0, (double)(x - 1));  // (d - min) * 1
    double tmp = kLcgRange;
    x = lcg_mulmod(x, kLcgA);
    sum = __dadd_rn(sum, __dmul_rn((double)(x - 1), tmp));
    tmp = __dmul_rn(tmp, kLcgRange);
    double ret = __ddiv_rn(sum, tmp);
    if (ret >= 1.0) ret = __longlong_as_double(0x3fefffffffffffffLL);  // nextafter(1, 0)
    return ret;
}

__device__ __forceinline__ double uniform_draw(uint64_t& x, double lo, double hi) {
    return __dadd_rn(__dmul_rn(canonical(x), __dsub_rn(hi, lo)), lo);
}

struct InitUniformArgs {
    int sx, sy, sz;
    double origin[3], w[3];
    uint64_t per_cell, remaining;  // N / cells, N mod cells
    ipic3d_particle* out;          // grouped by cell, row-major
};

// block b = cell b; its threads stride over the cell's particles
__global__ void k_init_uniform(InitUniformArgs A) {
    const int64_t c = blockIdx.x;
    const int z = (int)(c % A.sz), y = (int)((c / A.sz) % A.sy), x = (int)(c / ((int64_t)A.sy * A.sz));
    const int64_t n = (int64_t)A.per_cell + ((uint64_t)c < A.remaining ? 1 : 0);
    double lo[3], hi[3];
    const int pos[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = __dadd_rn(__dmul_rn(A.w[a], (double)pos[a]), A.origin[a]);
        hi[a] = __dadd_rn(lo[a], A.w[a]);
    }
    const uint32_t seed = (uint32_t)(((int64_t)x * 1023 + y) * 1023 + z);
    const uint64_t x0 = lcg_seed(seed + 1u), v0 = lcg_seed(seed + 2u);
    const int64_t s0 = c * (int64_t)A.per_cell + (c < (int64_t)A.remaining ? c : (int64_t)A.remaining);
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t jump = lcg_pow(6 * (uint64_t)i);  // 3 coordinates x 2 draws per particle
        uint64_t gp = lcg_mulmod(x0, jump), gv = lcg_mulmod(v0, jump);
        ipic3d_particle p;
#pragma unroll
        for (int a = 0; a < 3; ++a) p.position[a] = uniform_draw(gp, lo[a], hi[a]);
#pragma unroll
        for (int a = 0; a < 3; ++a) p.velocity[a] = uniform_draw(gv, -0.2, 0.2);
        p.q = -1.0;    // species::electron (cell.h:107-118)
        p.qom = -25.0;
        A.out[s0 + i] = p;
    }
}

// ---- initCells<uniform_pos_normal_speed> phase 2 (cell.h:596-632) --------
//
// Per cell, one thread replays the reference's loop: the cell's copy of the
// generator reseeded from seed = (uint32)((x * 1023 + y) * 1023 + z)
// (cell.h:608-612, generic_particle_generator::seed at cell.h:281-287: the
// position stream gets (1023 s) & s, the velocity stream ((1023 s) & s)
// transformed once more) draws each particle; its position is then replaced
// by a draw of the cell's own uniform stream seeded with seed
// (vector::uniform next_position, cell.h:615-621), so the generator's
// position draws never reach the output and are skipped here. Velocities are
// mean + stddev * z per component, z from the reference's Marsaglia-Tsang
// ziggurat (ziggurat_normal_distribution.h:8-127: 64-bit SHR3 state seeded
// 123456789 ^ seed, every draw through nfix()). Its tables are computed on
// the host with the reference's arithmetic (zigset, :101-125) and passed in.
// The ziggurat draws are sequential within a cell (rejection), so a cell is
// one thread. Every operation is rounded as the reference's build rounds it
// (FP32 where the reference computes in float, FP64 elsewhere, no fused
// multiply-adds); log and exp are the device library's, whose results agree
// with the host's on the rare paths that use them for the inputs tested.
struct ZigTables {
    uint64_t kn[128];
    float wn[128], fn[128];
};

struct Zig {
    uint64_t jsr;
    __device__ __forceinline__ uint64_t shr3() {
        const uint64_t jz = jsr;
        jsr ^= jsr << 13;
        jsr ^= jsr >> 17;
        jsr ^= jsr << 5;
        return jz + jsr;
    }
    __device__ __forceinline__ float uni() {
        return (float)__dadd_rn(0.5, __dmul_rn((double)(int32_t)(uint32_t)shr3(), .2328306e-9));
    }
    // log of a float argument, rounded to float
    __device__ __forceinline__ static float logf_(float v) { return (float)log((double)v); }
    __device__ float nfix(const ZigTables& T) {
        const float r = 3.442620f;
        int32_t hz = (int32_t)(uint32_t)shr3();
        uint32_t iz = (uint32_t)hz & 127u;
        if (fabs((double)hz) < (double)T.kn[iz]) return __fmul_rn((float)hz, T.wn[iz]);
        for (;;) {
            if (iz == 0) {
                float x, y;
                for (;;) {
                    x = (float)__dmul_rn(-0.2904764, (double)logf_(uni()));
                    y = -logf_(uni());
                    if (__fmul_rn(x, x) <= __fadd_rn(y, y)) break;
                }
                return hz <= 0 ? __fsub_rn(-r, x) : __fadd_rn(r, x);
            }
            const float x = __fmul_rn((float)hz, T.wn[iz]);
            const float f = __fadd_rn(T.fn[iz], __fmul_rn(uni(), __fsub_rn(T.fn[iz - 1], T.fn[iz])));
            if ((double)f < exp(__dmul_rn(__dmul_rn(-0.5, (double)x), (double)x))) return x;
            hz = (int32_t)(uint32_t)shr3();
            iz = (uint32_t)hz & 127u;
            if (fabs((double)hz) < (double)T.kn[iz]) return __fmul_rn((float)hz, T.wn[iz]);
        }
    }
};

struct InitNormalArgs {
    int sx, sy, sz;
    double origin[3], w[3];
    double mean[3], stddev[3];
    double q, qom;
    const uint64_t* count;  // particles per cell (phase 1)
    const int64_t* off;     // first output record of each cell
    ipic3d_particle* out;
};

__global__ void k_init_normal(const __grid_constant__ InitNormalArgs A, const __grid_constant__ ZigTables T) {
    const int64_t ncells = (int64_t)A.sx * A.sy * A.sz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int z = (int)(c % A.sz), y = (int)((c / A.sz) % A.sy), x = (int)(c / ((int64_t)A.sy * A.sz));
        double lo[3], hi[3];
        const int pos[3] = {x, y, z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = __dadd_rn(__dmul_rn(A.w[a], (double)pos[a]), A.origin[a]);
            hi[a] = __dadd_rn(lo[a], A.w[a]);
        }
        const uint32_t seed = (uint32_t)(((int64_t)x * 1023 + y) * 1023 + z);
        uint32_t s = (1023u * seed) & seed;  // the position stream's seed (its draws are overwritten)
        s = (1023u * s) & s;                 // the velocity stream's seed
        Zig zg{123456789ull ^ (uint64_t)s};
        uint64_t gp = lcg_seed(seed);  // next_position
        const uint64_t n = A.count[c];
        ipic3d_particle* o = A.out + A.off[c];
        for (uint64_t i = 0; i < n; ++i) {
            ipic3d_particle p;
#pragma unroll
            for (int a = 0; a < 3; ++a) p.velocity[a] = __dadd_rn(A.mean[a], __dmul_rn(A.stddev[a], (double)zg.nfix(T)));
#pragma unroll
            for (int a = 0; a < 3; ++a) p.position[a] = uniform_draw(gp, lo[a], hi[a]);
            p.q = A.q;
            p.qom = A.qom;
            o[i] = p;
        }
    }
}

// zigset (ziggurat_normal_distribution.h:101-125): the tables, with the
// host's libm as the reference computes them
ZigTables zig_tables() {
    ZigTables T;
    const double m1 = 2147483648.0;
    double dn = 3.442619855899, tn = dn, vn = 9.91256303526217e-3, q;
    q = vn / std::exp(-.5 * dn * dn);
    T.kn[0] = (uint64_t)((dn / q) * m1);
    T.kn[1] = 0;
    T.wn[0] = (float)(q / m1);
    T.wn[127] = (float)(dn / m1);
    T.fn[0] = 1.f;
    T.fn[127] = (float)(std::exp(-.5 * dn * dn));
    for (int i = 126; i >= 1; i--) {
        dn = std::sqrt(-2. * std::log(vn / dn + std::exp(-.5 * dn * dn)));
        T.kn[i + 1] = (uint64_t)((dn / tn) * m1);
        tn = dn;
        T.fn[i] = (float)(std::exp(-.5 * dn * dn));
        T.wn[i] = (float)(dn / m1);
    }
    return T;
}

}  // namespace

// Phase 1 of initCells<Distribution> (cell.h:505-590) on the host: 100
// pseudo-particles per cell from the distribution's position stream
// (vector::uniform over [low, hig), seeded 1: std::minstd_rand through
// std::uniform_real_distribution, the reference's own library classes),
// each redrawn until it lies in the universe (isInsideUniverse, cell.h:75-83)
// and binned with N / (100 cells) particles, then the remainder spread (every
// cell gets (N - sum) / cells more, the first (N - sum) % cells one more).
// The velocity draws of this phase do not influence the counts and are not
// made.
void init_normal_counts(const ipic3d_props& pr, uint64_t num_particles, const double low[3], const double hig[3],
                        std::vector<uint64_t>& counts) {
    const int64_t sx = pr.size[0], sy = pr.size[1], sz = pr.size[2];
    const int64_t cells = sx * sy * sz;
    counts.assign(cells, 0);
    std::minstd_rand g(1);
    std::uniform_real_distribution<> d[3] = {std::uniform_real_distribution<>(low[0], hig[0]),
                                             std::uniform_real_distribution<>(low[1], hig[1]),
                                             std::uniform_real_distribution<>(low[2], hig[2])};
    const int64_t pseudo = cells * 100;
    const uint64_t per = num_particles / (uint64_t)pseudo;
    const double top[3] = {pr.origin[0] + sx * pr.cell_width[0], pr.origin[1] + sy * pr.cell_width[1],
                           pr.origin[2] + sz * pr.cell_width[2]};
    for (int64_t i = 0; i < pseudo; ++i) {
        double p[3];
        for (;;) {
            for (int a = 0; a < 3; ++a) p[a] = d[a](g);
            bool in = true;
            for (int a = 0; a < 3; ++a) in = in && pr.origin[a] <= p[a] && p[a] < top[a];
            if (in) break;
        }
        int64_t c[3];
        for (int a = 0; a < 3; ++a) c[a] = (int64_t)((p[a] - pr.origin[a]) / pr.cell_width[a]);
        counts[(c[0] * sy + c[1]) * sz + c[2]] += per;
    }
    uint64_t sum = 0;
    for (auto n : counts) sum += n;
    const int64_t missing = (int64_t)num_particles - (int64_t)sum;
    if (missing != 0) {
        const int all_correct = (int)(missing / cells);
        const int remain_correct = (int)(missing % cells);
        for (int64_t c = 0; c < cells; ++c) {
            counts[c] += all_correct;
            if (c < remain_correct) counts[c] += 1;
        }
    }
}

int launch_init_normal(const ipic3d_props& pr, const double mean[3], const double stddev[3], double q, double qom,
                       const uint64_t* d_count, const int64_t* d_off, void* out, cudaStream_t st) {
    InitNormalArgs A;
    A.sx = (int)pr.size[0];
    A.sy = (int)pr.size[1];
    A.sz = (int)pr.size[2];
    for (int a = 0; a < 3; ++a) {
        A.origin[a] = pr.origin[a];
        A.w[a] = pr.cell_width[a];
        A.mean[a] = mean[a];
        A.stddev[a] = stddev[a];
    }
    A.q = q;
    A.qom = qom;
    A.count = d_count;
    A.off = d_off;
    A.out = static_cast<ipic3d_particle*>(out);
    const int64_t cells = pr.size[0] * pr.size[1] * pr.size[2];
    const int64_t blocks = std::min<int64_t>((cells + 127) / 128, 152 * 16);
    k_init_normal<<<(unsigned)(blocks > 0 ? blocks : 1), 128, 0, st>>>(A, zig_tables());
    return 1;
}

int launch_init_uniform(int sx, int sy, int sz, const double origin[3], const double w[3], uint64_t num_particles,
                        void* out, cudaStream_t st) {
    InitUniformArgs A;
    A.sx = sx;
    A.sy = sy;
    A.sz = sz;
    for (int a = 0; a < 3; ++a) {
        A.origin[a] = origin[a];
        A.w[a] = w[a];
    }
    const uint64_t cells = (uint64_t)sx * sy * sz;
    A.per_cell = num_particles / cells;
    A.remaining = num_particles % cells;
    A.out = static_cast<ipic3d_particle*>(out);
    k_init_uniform<<<(unsigned)cells, 256, 0, st>>>(A);
    return 1;
}

}  // namespace ipg
