// ipic3d_gpu_project_noalloc: the current projection (projectToDensityField
// over all nodes, cell.h:787-824) for callers that cannot allocate device
// memory -- code that runs where a cudaMalloc would stall the stream or is
// not allowed: inside a host that owns every byte of device memory through
// its own pool, or a per-step loop that must not synchronise the device.
// The caller passes the particles and the output grids; the FP64 node sums
// in between live in a file-scope device array, so no call here allocates.
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/ipic3d_gpu.h"
#include "launch.h"

namespace ipg {
namespace {

// Raw per-node sums (Jx, Jy, Jz, rho) before the periodic fold and the
// normalisation: room for grids of up to 32^3 cells ((32+1)^3 nodes,
// 1.15 MB). Every GPU that loads the library holds it until the process
// exits; every call shares it.
constexpr int64_t kNoAllocMaxNodes = 33LL * 33 * 33;
__device__ __align__(256) double g_noalloc_scratch[4 * kNoAllocMaxNodes];

// Device address of g_noalloc_scratch per device, resolved on the first
// call in each context. The address belongs to the context the module was
// loaded into: after cudaDeviceReset (a new primary context, the module
// loaded again) the next call looks it up again, keyed on the context's
// unique id (cuCtxGetId), so no call writes through a stale address.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

// The unique id of the calling thread's current context (driver entry
// points resolved through the runtime: the library links no libcuda).
cudaError_t current_context_id(unsigned long long* id) {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess) return e;
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return cudaErrorSymbolNotFound;
        get_current = reinterpret_cast<GetCurrent>(f1);
        get_id = reinterpret_cast<GetId>(f2);
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return cudaErrorDeviceUninitialized;
    if (get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorContextIsDestroyed;
    return cudaSuccess;
}

struct NAGeom {
    int sx, sy, sz;
    double origin[3], w[3], vol;
    int div8;
};

// One warp per cell: every lane sums the cloud-in-cell contributions of its
// particles to the cell's 8 corners (weights (1-r) / r per axis, cell.h:815),
// a warp transpose-reduction collects the 32 values, one FP64 atomic each.
__global__ void k_na_deposit(const ipic3d_particle* __restrict__ p, const uint64_t* __restrict__ off, NAGeom g,
                             double* __restrict__ acc) {
    const int64_t ncells = (int64_t)g.sx * g.sy * g.sz;
    const int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= ncells) return;
    const int cz = (int)(c % g.sz), cy = (int)((c / g.sz) % g.sy), cx = (int)(c / ((int64_t)g.sy * g.sz));
    const double ox = g.origin[0] + (double)cx * g.w[0];
    const double oy = g.origin[1] + (double)cy * g.w[1];
    const double oz = g.origin[2] + (double)cz * g.w[2];
    double v[32];
#pragma unroll
    for (int l = 0; l < 32; ++l) v[l] = 0.0;
    const uint64_t a = off[c], b = off[c + 1];
    for (uint64_t i = a + lane; i < b; i += 32) {
        const ipic3d_particle q = p[i];
        const double rx = (q.position[0] - ox) / g.w[0];
        const double ry = (q.position[1] - oy) / g.w[1];
        const double rz = (q.position[2] - oz) / g.w[2];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const double fac = ((k & 4) ? rx : 1 - rx) * ((k & 2) ? ry : 1 - ry) * ((k & 1) ? rz : 1 - rz);
            v[k * 4 + 0] += (q.q * q.velocity[0]) * fac;
            v[k * 4 + 1] += (q.q * q.velocity[1]) * fac;
            v[k * 4 + 2] += (q.q * q.velocity[2]) * fac;
            v[k * 4 + 3] += q.q * fac;
        }
    }
    if (a == b) return;  // warp-uniform
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
            const double send = upper ? v[i] : v[i + o];
            const double keep = upper ? v[i + o] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    const int corner = lane >> 2, comp = lane & 3;
    const int nx = cx + (corner >> 2), ny = cy + ((corner >> 1) & 1), nz = cz + (corner & 1);
    const int64_t node = ((int64_t)nx * (g.sy + 1) + ny) * (g.sz + 1) + nz;
    if (v[0] != 0.0) atomicAdd(acc + 4 * node + comp, v[0]);
}

// Final values: the periodic image set of a boundary node ({0, s} per axis,
// the cell wrap of cell.h:799-805) shares one sum; J = (sum / vol) [/ 8].
__global__ void k_na_finalize(NAGeom g, const double* __restrict__ acc, double* __restrict__ J,
                              double* __restrict__ rho) {
    const int64_t total = (int64_t)g.sx * g.sy * g.sz;
    const int ny = g.sy + 1, nz = g.sz + 1;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(t / ((int64_t)g.sy * g.sz)), y = (int)((t / g.sz) % g.sy), z = (int)(t % g.sz);
        const int nxs = x == 0 ? 2 : 1, nys = y == 0 ? 2 : 1, nzs = z == 0 ? 2 : 1;
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        for (int i = 0; i < nxs; ++i)
            for (int j = 0; j < nys; ++j)
                for (int k = 0; k < nzs; ++k) {
                    const int64_t n = ((int64_t)(i ? g.sx : x) * ny + (j ? g.sy : y)) * nz + (k ? g.sz : z);
                    for (int c = 0; c < 4; ++c) s[c] += acc[4 * n + c];
                }
        for (int c = 0; c < 4; ++c) {
            s[c] = s[c] / g.vol;
            if (g.div8) s[c] = s[c] / 8.0;
        }
        for (int i = 0; i < nxs; ++i)
            for (int j = 0; j < nys; ++j)
                for (int k = 0; k < nzs; ++k) {
                    const int64_t n = ((int64_t)(i ? g.sx : x) * ny + (j ? g.sy : y)) * nz + (k ? g.sz : z);
                    J[3 * n] = s[0];
                    J[3 * n + 1] = s[1];
                    J[3 * n + 2] = s[2];
                    if (rho) rho[n] = s[3];
                }
    }
}

int na_fail(int status, const char* msg) { return set_last_error(status, msg); }

}  // namespace
}  // namespace ipg

extern "C" {

int ipic3d_gpu_project_noalloc(const ipic3d_props* props, uint32_t flags, const ipic3d_particle* d_particles,
                               const uint64_t* d_cell_offsets, double* d_J, double* d_rho, void* stream) {
    using namespace ipg;
    if (!props || !d_cell_offsets || !d_J) return na_fail(IPIC3D_E_INVALID, "NULL argument");
    for (int a = 0; a < 3; ++a)
        if (props->size[a] <= 0 || !(props->cell_width[a] > 0)) return na_fail(IPIC3D_E_INVALID, "bad grid");
    // each axis on its own first, so the node count below cannot overflow
    for (int a = 0; a < 3; ++a)
        if (props->size[a] >= kNoAllocMaxNodes)
            return na_fail(IPIC3D_E_CAPACITY,
                           "ipic3d_gpu_project_noalloc: grid too large for its fixed scratch (at most (32+1)^3 nodes)");
    const int64_t nodes = (props->size[0] + 1) * (props->size[1] + 1) * (props->size[2] + 1);
    if (nodes > kNoAllocMaxNodes)
        return na_fail(IPIC3D_E_CAPACITY,
                       "ipic3d_gpu_project_noalloc: grid too large for its fixed scratch (at most (32+1)^3 nodes)");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return na_fail(IPIC3D_E_NODEVICE, "no current CUDA device");
    unsigned long long ctx_id = 0;
    {
        const cudaError_t e = current_context_id(&ctx_id);
        if (e != cudaSuccess) return na_fail(IPIC3D_E_NODEVICE, cudaGetErrorString(e));
    }
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx_id) {
            // first call in this context: the device address of the static array
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return na_fail(IPIC3D_E_CUDA, cudaGetErrorString(e));
            g_scratch_ptr[dev] = static_cast<double*>(p);
            g_scratch_ctx[dev] = ctx_id;
        }
        scratch = g_scratch_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    NAGeom g;
    g.sx = (int)props->size[0];
    g.sy = (int)props->size[1];
    g.sz = (int)props->size[2];
    for (int a = 0; a < 3; ++a) {
        g.origin[a] = props->origin[a];
        g.w[a] = props->cell_width[a];
    }
    g.vol = props->cell_width[0] * props->cell_width[1] * props->cell_width[2];
    g.div8 = (flags & IPIC3D_F_J_DIV8) ? 1 : 0;
    // the scratch keeps the previous call's sums: clear the part in use
    cudaError_t e = cudaMemsetAsync(scratch, 0, (size_t)nodes * 4 * sizeof(double), st);
    if (e != cudaSuccess) return na_fail(IPIC3D_E_CUDA, cudaGetErrorString(e));
    const int64_t ncells = props->size[0] * props->size[1] * props->size[2];
    if (d_particles) {
        const int64_t threads = ncells * 32;
        k_na_deposit<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(d_particles, d_cell_offsets, g, scratch);
    }
    int64_t blocks = (ncells + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_na_finalize<<<(unsigned)blocks, 256, 0, st>>>(g, scratch, d_J, d_rho);
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(IPIC3D_E_CUDA, cudaGetErrorString(e));
    return IPIC3D_OK;
}

}  // extern "C"
