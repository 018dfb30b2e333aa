// Particle initialisation on the device with the reference's own random
// streams: initCells(properties, numParticles, uniform<>) (cell.h:638-697),
// the universe of the reference's ":U:N" benchmark mode.
//
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
#include <cstdint>

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

}  // namespace

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
