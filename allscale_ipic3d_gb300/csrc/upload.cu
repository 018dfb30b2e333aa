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

// Centred cloud-in-cell moments of one particle with weight wq (the charge):
// acc[8 Q + m], Q in {u, v, w, 1}, m in {1, x, y, xy, z, xz, yz, xyz} about the
// cell centre (the layout of the FP32 push's deposit).
__device__ __forceinline__ void add_moments_q(float (&acc)[32], float x, float y, float z, float u, float v, float w,
                                              float wq) {
    x -= 0.5f; y -= 0.5f; z -= 0.5f;
    const float mono[8] = {1.f, x, y, x * y, z, x * z, y * z, x * y * z};
    const float Q[4] = {wq * u, wq * v, wq * w, wq};
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int m = 0; m < 8; ++m) acc[q * 8 + m] = fmaf(Q[q], mono[m], acc[q * 8 + m]);
}

template <bool kDeposit, typename T>
__global__ void k_upload_cells(const ipic3d_particle* __restrict__ p, const uint32_t* __restrict__ ids,
                               const int64_t* __restrict__ in_off, int c0, int c1, SpeciesTable sp, UploadPops<T> U,
                               UploadGeom g, UploadDeposit dep, int* flags) {
    const int c = c0 + (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= c1) return;
    const int cz = c % g.sz, cy = (c / g.sz) % g.sy, cx = c / (g.sy * g.sz);
    const double ox = g.origin[0] + (double)cx * g.w[0];
    const double oy = g.origin[1] + (double)cy * g.w[1];
    const double oz = g.origin[2] + (double)cz * g.w[2];
    const int64_t a = in_off[c], b = in_off[c + 1];
    int base[kUploadMaxPops], cap[kUploadMaxPops];
    int64_t start[kUploadMaxPops];
    for (int k = 0; k < U.npop; ++k) {
        base[k] = 0;
        start[k] = U.start[k][c];
        cap[k] = (int)(U.start[k][c + 1] - start[k]);
    }
    float acc[32];
    if (kDeposit) {
#pragma unroll
        for (int l = 0; l < 32; ++l) acc[l] = 0.f;
    }
    bool unknown = false, full = false;
    for (int64_t i0 = a; i0 < b; i0 += 32) {
        const int64_t i = i0 + lane;
        int s = -1;
        ipic3d_particle q;
        if (i < b) {
            q = p[i];
            for (int k = 0; k < sp.n; ++k)
                if (sp.q[k] == q.q && sp.qom[k] == q.qom) { s = k; break; }
            if (s < 0) unknown = true;
        }
        T x = 0, y = 0, z = 0;
        if (s >= 0) {
            if (U.relative) {
                x = (T)((q.position[0] - ox) / g.w[0]);
                y = (T)((q.position[1] - oy) / g.w[1]);
                z = (T)((q.position[2] - oz) / g.w[2]);
            } else {
                x = (T)q.position[0];
                y = (T)q.position[1];
                z = (T)q.position[2];
            }
        }
        for (int k = 0; k < U.npop; ++k) {
            const unsigned bal = __ballot_sync(0xffffffffu, s == k);
            if (s == k) {
                const int r = base[k] + __popc(bal & ((1u << lane) - 1u));
                if (r < cap[k]) {
                    const int64_t slot = start[k] + r;
                    U.x[k][slot] = x; U.y[k][slot] = y; U.z[k][slot] = z;
                    U.u[k][slot] = (T)q.velocity[0];
                    U.v[k][slot] = (T)q.velocity[1];
                    U.w[k][slot] = (T)q.velocity[2];
                    if (U.id[k]) U.id[k][slot] = ids ? ids[i] : (uint32_t)i;
                } else {
                    full = true;
                }
            }
            base[k] += __popc(bal);
        }
        if (kDeposit && s >= 0)
            add_moments_q(acc, (float)x, (float)y, (float)z, (float)q.velocity[0], (float)q.velocity[1],
                          (float)q.velocity[2], (float)sp.q[s]);
    }
    if (__any_sync(0xffffffffu, unknown) && lane == 0) atomicExch(flags, 1);
    if (__any_sync(0xffffffffu, full) && lane == 0) atomicExch(flags + 1, 1);
    if (lane < U.npop) U.count[lane][c] = base[lane] < cap[lane] ? base[lane] : cap[lane];
    if (kDeposit) {
        // lane v: summed moment v = 8 Q + m; three axis butterflies give the
        // corner sums (corner m, component Q); one FP64 atomic each
        float v[32];
#pragma unroll
        for (int l = 0; l < 32; ++l) v[l] = acc[l];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const bool upper = (lane & off) != 0;
#pragma unroll
            for (int j = 0; j < off; ++j) {
                const float send = upper ? v[j] : v[j + off];
                const float keep = upper ? v[j + off] : v[j];
                v[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
            }
        }
        float t = v[0];
        const int m = lane & 7, qq = lane >> 3;
#pragma unroll
        for (int bit = 1; bit < 8; bit <<= 1) {
            const float o = __shfl_xor_sync(0xffffffffu, t, bit);
            t = (m & bit) ? fmaf(0.5f, o, t) : fmaf(0.5f, t, -o);
        }
        if (t != 0.f) {
            const int64_t n = ((int64_t)(cx + (m & 1)) * (dep.sy + 1) + (cy + ((m >> 1) & 1))) * (dep.sz + 1) +
                              (cz + (m >> 2));
            if (qq < 3)
                atomicAdd(dep.J + 3 * n + qq, (double)t);
            else
                atomicAdd(dep.rho + n, (double)t);
        }
    }
}

}  // namespace

template <typename T>
int launch_upload_cells(const void* parts, const uint32_t* ids, const int64_t* in_off, int c0, int c1,
                        const SpeciesTable& sp, const UploadPops<T>& U, const UploadGeom& g, const UploadDeposit& dep,
                        int* flags, cudaStream_t st) {
    if (c1 <= c0) return 0;
    const int64_t threads = (int64_t)(c1 - c0) * 32;
    const unsigned blocks = (unsigned)((threads + 255) / 256);
    if (dep.on)
        k_upload_cells<true, T><<<blocks, 256, 0, st>>>((const ipic3d_particle*)parts, ids, in_off, c0, c1, sp, U, g,
                                                        dep, flags);
    else
        k_upload_cells<false, T><<<blocks, 256, 0, st>>>((const ipic3d_particle*)parts, ids, in_off, c0, c1, sp, U,
                                                         g, dep, flags);
    return 1;
}
template int launch_upload_cells<float>(const void*, const uint32_t*, const int64_t*, int, int, const SpeciesTable&,
                                        const UploadPops<float>&, const UploadGeom&, const UploadDeposit&, int*,
                                        cudaStream_t);
template int launch_upload_cells<double>(const void*, const uint32_t*, const int64_t*, int, int, const SpeciesTable&,
                                         const UploadPops<double>&, const UploadGeom&, const UploadDeposit&, int*,
                                         cudaStream_t);

namespace {
// One warp per cell of [c0, c1): every population's particles of the cell
// as AoS records at their output indices (consecutive lanes write
// consecutive 64-byte records).
template <typename T>
__global__ void k_pack_cells(PackPops<T> P, UploadGeom g, int c0, int c1, ipic3d_particle* __restrict__ out,
                             uint32_t* __restrict__ out_ids) {
    const int64_t c = c0 + ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= c1) return;
    const int cz = (int)(c % g.sz), cy = (int)((c / g.sz) % g.sy), cx = (int)(c / ((int64_t)g.sy * g.sz));
    const double ox = g.origin[0] + (double)cx * g.w[0];
    const double oy = g.origin[1] + (double)cy * g.w[1];
    const double oz = g.origin[2] + (double)cz * g.w[2];
    for (int k = 0; k < P.npop; ++k) {
        const int n = P.count[k][c];
        const int64_t s0 = P.start[k][c], d0 = P.dst[(int64_t)k * g.ncells + c];
        for (int i = lane; i < n; i += 32) {
            const int64_t s = s0 + i;
            ipic3d_particle r;
            if (P.relative) {
                r.position[0] = ox + (double)P.x[k][s] * g.w[0];
                r.position[1] = oy + (double)P.y[k][s] * g.w[1];
                r.position[2] = oz + (double)P.z[k][s] * g.w[2];
            } else {
                r.position[0] = (double)P.x[k][s];
                r.position[1] = (double)P.y[k][s];
                r.position[2] = (double)P.z[k][s];
            }
            if (P.positions_only) {
                double* o = reinterpret_cast<double*>(out) + 3 * (d0 + i);
                o[0] = r.position[0];
                o[1] = r.position[1];
                o[2] = r.position[2];
                continue;
            }
            r.velocity[0] = (double)P.u[k][s];
            r.velocity[1] = (double)P.v[k][s];
            r.velocity[2] = (double)P.w[k][s];
            r.q = P.q[k];
            r.qom = P.qom[k];
            double2* o = reinterpret_cast<double2*>(out + d0 + i);
            o[0] = make_double2(r.position[0], r.position[1]);
            o[1] = make_double2(r.position[2], r.velocity[0]);
            o[2] = make_double2(r.velocity[1], r.velocity[2]);
            o[3] = make_double2(r.q, r.qom);
            if (out_ids) out_ids[d0 + i] = P.id[k] ? P.id[k][s] : 0u;
        }
    }
}
}  // namespace

template <typename T>
int launch_pack_cells(const PackPops<T>& P, const UploadGeom& g, int c0, int c1, void* out, uint32_t* out_ids,
                      cudaStream_t st) {
    if (c1 <= c0) return 0;
    const int64_t threads = (int64_t)(c1 - c0) * 32;
    k_pack_cells<T><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(P, g, c0, c1,
                                                                        static_cast<ipic3d_particle*>(out), out_ids);
    return 1;
}
template int launch_pack_cells<float>(const PackPops<float>&, const UploadGeom&, int, int, void*, uint32_t*,
                                      cudaStream_t);
template int launch_pack_cells<double>(const PackPops<double>&, const UploadGeom&, int, int, void*, uint32_t*,
                                       cudaStream_t);

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
