// Device-side upload of the reference's particle layout (Universe::cells:
// AoS Particle records grouped by cell, cell.h:31-38) into the GPU layout
// (per species structure-of-arrays, grouped by cell with slack).
//
//   k_classify  species index of every particle from its (q, qom)
//   k_count     per species and cell counts (one warp per cell, ballots)
//   k_scatter   slot of every particle: start[s][c] + its rank among the
//               cell's particles of species s (ballot prefix), converting the
//               position to cell-relative FP32 where the context is FP32
#include "../../include/ipic3d_types.h"
#include "upload.h"

namespace ipg {
namespace {

__global__ void k_classify(const ipic3d_particle* __restrict__ p, int64_t n, SpeciesTable sp, uint8_t* sid,
                           int* unknown) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double q = p[i].q, qom = p[i].qom;
        int k = 0;
        for (; k < sp.n; ++k)
            if (sp.q[k] == q && sp.qom[k] == qom) break;
        if (k == sp.n) {
            atomicExch(unknown, 1);
            k = 0;
        }
        sid[i] = (uint8_t)k;
    }
}

__global__ void k_count(const uint8_t* __restrict__ sid, const int64_t* __restrict__ in_off, int ncells, int npop,
                        int32_t* counts /* [npop][ncells] */) {
    const int c = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= ncells) return;
    const int64_t a = in_off[c], b = in_off[c + 1];
    int mine = 0;  // lane s accumulates species s (npop <= 32)
    for (int64_t i0 = a; i0 < b; i0 += 32) {
        const int64_t i = i0 + lane;
        const int s = i < b ? (int)sid[i] : -1;
        for (int k = 0; k < npop; ++k) {
            const unsigned bal = __ballot_sync(0xffffffffu, s == k);
            if (lane == k) mine += __popc(bal);
        }
    }
    if (lane < npop) counts[(int64_t)lane * ncells + c] = mine;
}

template <typename T>
__global__ void k_scatter(const ipic3d_particle* __restrict__ p, const uint32_t* __restrict__ ids,
                          const uint8_t* __restrict__ sid, const int64_t* __restrict__ in_off, UploadPops<T> U,
                          UploadGeom g) {
    const int c = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= g.ncells) return;
    const int cz = c % g.sz, cy = (c / g.sz) % g.sy, cx = c / (g.sy * g.sz);
    const double ox = g.origin[0] + (double)cx * g.w[0];
    const double oy = g.origin[1] + (double)cy * g.w[1];
    const double oz = g.origin[2] + (double)cz * g.w[2];
    const int64_t a = in_off[c], b = in_off[c + 1];
    int base[kUploadMaxPops];
    for (int k = 0; k < U.npop; ++k) base[k] = 0;
    for (int64_t i0 = a; i0 < b; i0 += 32) {
        const int64_t i = i0 + lane;
        const int s = i < b ? (int)sid[i] : -1;
        for (int k = 0; k < U.npop; ++k) {
            const unsigned bal = __ballot_sync(0xffffffffu, s == k);
            if (s == k) {
                const int64_t slot = U.start[k][c] + base[k] + __popc(bal & ((1u << lane) - 1u));
                const ipic3d_particle& q = p[i];
                if (U.relative) {
                    U.x[k][slot] = (T)((q.position[0] - ox) / g.w[0]);
                    U.y[k][slot] = (T)((q.position[1] - oy) / g.w[1]);
                    U.z[k][slot] = (T)((q.position[2] - oz) / g.w[2]);
                } else {
                    U.x[k][slot] = (T)q.position[0];
                    U.y[k][slot] = (T)q.position[1];
                    U.z[k][slot] = (T)q.position[2];
                }
                U.u[k][slot] = (T)q.velocity[0];
                U.v[k][slot] = (T)q.velocity[1];
                U.w[k][slot] = (T)q.velocity[2];
                if (U.id[k]) U.id[k][slot] = ids ? ids[i] : (uint32_t)i;
            }
            base[k] += __popc(bal);
        }
    }
    if (lane < U.npop) U.count[lane][c] = base[lane];
}

}  // namespace

int launch_classify(const void* parts, int64_t n, const SpeciesTable& sp, uint8_t* sid, int* unknown,
                    cudaStream_t st) {
    if (n <= 0) return 0;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_classify<<<(unsigned)blocks, 256, 0, st>>>((const ipic3d_particle*)parts, n, sp, sid, unknown);
    return 1;
}

int launch_count(const uint8_t* sid, const int64_t* in_off, int ncells, int npop, int32_t* counts,
                 cudaStream_t st) {
    const int64_t threads = (int64_t)ncells * 32;
    k_count<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(sid, in_off, ncells, npop, counts);
    return 1;
}

template <typename T>
int launch_scatter(const void* parts, const uint32_t* ids, const uint8_t* sid, const int64_t* in_off,
                   const UploadPops<T>& U, const UploadGeom& g, cudaStream_t st) {
    const int64_t threads = (int64_t)g.ncells * 32;
    k_scatter<T><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>((const ipic3d_particle*)parts, ids, sid, in_off,
                                                                     U, g);
    return 1;
}
template int launch_scatter<float>(const void*, const uint32_t*, const uint8_t*, const int64_t*,
                                   const UploadPops<float>&, const UploadGeom&, cudaStream_t);
template int launch_scatter<double>(const void*, const uint32_t*, const uint8_t*, const int64_t*,
                                    const UploadPops<double>&, const UploadGeom&, cudaStream_t);

}  // namespace ipg
