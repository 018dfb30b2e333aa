// aggregateDensityContributions (cell.h:835-855) over every node of the
// (size+1)^3 current-density grid: the node at pos adds the contributions at
// 2 pos + {-1, 0}^3 that lie inside the (2 size)^3 contribution grid (the
// buffer the reference allocates at simulator.h:156) to its J, in the
// reference's i, j, k order, and divides the sum by the cell volume and by
// 8. Each contribution belongs to exactly one node, so one thread per node
// reads the contribution grid once, coalesced along z.
#include "../../include/ipic3d_gpu.h"
#include "launch.h"

namespace ipg {
namespace {

struct AggGeom {
    int64_t nx, ny, nz;  // nodes per axis: size + 1
    int64_t cx, cy, cz;  // contributions per axis: 2 size
    double vol;
};

__global__ void k_aggregate(const double* __restrict__ contrib, double* __restrict__ J, AggGeom g) {
    const int64_t nodes = g.nx * g.ny * g.nz;
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += (int64_t)gridDim.x * blockDim.x) {
        const int64_t z = n % g.nz, y = (n / g.nz) % g.ny, x = n / (g.nz * g.ny);
        double* j = J + 3 * n;
        double ax = j[0], ay = j[1], az = j[2];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int64_t c0 = 2 * x + i - 1, c1 = 2 * y + jj - 1, c2 = 2 * z + k - 1;
                    if (c0 < 0 || c0 >= g.cx || c1 < 0 || c1 >= g.cy || c2 < 0 || c2 >= g.cz) continue;
                    const double* q = contrib + 3 * ((c0 * g.cy + c1) * g.cz + c2);
                    ax = ax + __ldg(q);
                    ay = ay + __ldg(q + 1);
                    az = az + __ldg(q + 2);
                }
        j[0] = ax / g.vol / 8.0;
        j[1] = ay / g.vol / 8.0;
        j[2] = az / g.vol / 8.0;
    }
}

}  // namespace
}  // namespace ipg

extern "C" {

int ipic3d_gpu_aggregate_contributions(const ipic3d_props* props, const double* d_contributions, double* d_J,
                                       void* stream) {
    using namespace ipg;
    if (!props || !d_contributions || !d_J)
        return set_last_error(IPIC3D_E_INVALID, "ipic3d_gpu_aggregate_contributions: NULL argument");
    for (int a = 0; a < 3; ++a)
        if (props->size[a] <= 0 || props->size[a] > (1 << 20) || !(props->cell_width[a] > 0))
            return set_last_error(IPIC3D_E_INVALID, "ipic3d_gpu_aggregate_contributions: bad grid");
    AggGeom g;
    g.nx = props->size[0] + 1;
    g.ny = props->size[1] + 1;
    g.nz = props->size[2] + 1;
    g.cx = 2 * props->size[0];
    g.cy = 2 * props->size[1];
    g.cz = 2 * props->size[2];
    g.vol = props->cell_width[0] * props->cell_width[1] * props->cell_width[2];
    const int64_t nodes = g.nx * g.ny * g.nz;
    int64_t blocks = (nodes + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_aggregate<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(d_contributions, d_J, g);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? IPIC3D_OK : set_last_error(IPIC3D_E_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
