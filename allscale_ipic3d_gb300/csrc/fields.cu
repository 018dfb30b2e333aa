// Field-grid kernels of the GB300 path (FP64, built with -fmad=false so every
// expression rounds as the reference's does).
//
//   k_ghost        updateFieldsOnBoundaries (field.h:407-440)
//   k_leapfrog_e   solveFieldLeapfrog, E part   (field.h:359-363)
//   k_leapfrog_b   solveFieldLeapfrog, Bc part  (field.h:366-372)
//   k_forward_e/b  solveFieldForward            (field.h:294-337, curls 162-229)
//   k_interp_c2n   interpC2N                    (field.h:234-247)
//   k_j_finalize   J = (Js / vol) / 8           (cell.h:822-823) plus the
//                  periodic duplicate nodes of the gather form (cell.h:799-805)
//   k_node32       FP32 copy of node E, B for the FP32 gather
//   reductions     getFieldEnergy (field.h:443-459), particle sums
//                  (cell.h:1315-1355), Neumaier-compensated
//
// The reference's per-node solver updates E and then Bc in one in-place pass
// whose result depends on the visiting order; here E is updated everywhere
// first and Bc afterwards (the order-independent two-phase reading).
#include <cmath>

#include "launch.h"

namespace ipg {

namespace {

__device__ __forceinline__ int64_t fidx(int n, int x, int y, int z) { return ((int64_t)x * n + y) * n + z; }

// Copies the six ghost faces of a cubic grid of n^3 records of `per` doubles:
// index (a, b) in [1, n-1)^2 of each face (edges and corners stay).
__device__ __forceinline__ void ghost_body(double* g, int n, int per, int64_t t0, int64_t stride) {
    const int end = n - 1;
    const int64_t m = (int64_t)(end - 1) * (end - 1);
    for (int64_t t = t0; t < m * per; t += stride) {
        int a, b, comp;
        split3(t, end - 1, per, a, b, comp);  // t = (a' (end - 1) + b') per + comp
        a += 1;
        b += 1;
        g[fidx(n, 0, a, b) * per + comp] = g[fidx(n, end - 1, a, b) * per + comp];
        g[fidx(n, end, a, b) * per + comp] = g[fidx(n, 1, a, b) * per + comp];
        g[fidx(n, a, 0, b) * per + comp] = g[fidx(n, a, end - 1, b) * per + comp];
        g[fidx(n, a, end, b) * per + comp] = g[fidx(n, a, 1, b) * per + comp];
        g[fidx(n, a, b, 0) * per + comp] = g[fidx(n, a, b, end - 1) * per + comp];
        g[fidx(n, a, b, end) * per + comp] = g[fidx(n, a, b, 1) * per + comp];
    }
}

struct SolverArgs {
    int s;                // cells per axis (cubic)
    double dt, c;
    double wx, wy, wz;
    double iwx, iwy, iwz;  // 1 / w (the multiplying solvers)
    float4* n32;          // FP32 node copy {Ex,Ey,Ez,0},{Bx,By,Bz,0} kept current (FP32 path), or null
    double* field;        // (s+3)^3 x 9
    double* bc;           // (s+2)^3 x 3
    const double* J;      // (s+1)^3 x 3
    // J as the E update reads it: jmode 0, final (folded, normalised); else
    // raw node sums of the deposit, folded over the periodic images and
    // normalised on the read exactly as k_j_finalize (jmode 1: / vol [/ 8])
    // or k_j_finalize_mul (jmode 2: * jinv) would store them
    int jmode, jdiv8;
    double jvol, jinv;
};

// J of node m (per axis in [0, s]) as the J finalisation stores it: the sum
// over the node's images {0, s} on each axis where it lies on the boundary,
// in the finalisation's order, then normalised.
__device__ __forceinline__ void final_j(const SolverArgs& A, int mx, int my, int mz, double (&a)[3]) {
    const int s = A.s, nd = A.s + 1;
    const int x = mx == s ? 0 : mx, y = my == s ? 0 : my, z = mz == s ? 0 : mz;
    const int nxs = x == 0 ? 2 : 1, nys = y == 0 ? 2 : 1, nzs = z == 0 ? 2 : 1;
    a[0] = a[1] = a[2] = 0.0;
    for (int i = 0; i < nxs; ++i)
        for (int j = 0; j < nys; ++j)
            for (int k = 0; k < nzs; ++k) {
                const double* p = A.J + 3 * fidx(nd, i ? s : x, j ? s : y, k ? s : z);
                a[0] += p[0]; a[1] += p[1]; a[2] += p[2];
            }
    for (int c = 0; c < 3; ++c) {
        if (A.jmode == 1) {
            a[c] = a[c] / A.jvol;
            if (A.jdiv8) a[c] = a[c] / 8.0;
        } else {
            a[c] *= A.jinv;
        }
    }
}

__device__ __forceinline__ void read_j(const SolverArgs& A, int mx, int my, int mz, double (&a)[3]) {
    if (A.jmode == 0) {
        const double* p = A.J + 3 * fidx(A.s + 1, mx, my, mz);
        a[0] = p[0]; a[1] = p[1]; a[2] = p[2];
    } else {
        final_j(A, mx, my, mz, a);
    }
}

// d / w: the reference's division (kMul false) or the product with 1 / w
// (kMul: equal bit for bit when w is a power of two; the FP32 path's solver
// otherwise)
template <bool kMul>
__device__ __forceinline__ double over(double d, double w, double iw) {
    return kMul ? d * iw : d / w;
}

// E at pos in [1, s+2)^3 from Bc(pos), Bc(pos - e_i) and J(pos - 1).
template <bool kMul = false>
__device__ __forceinline__ void leapfrog_e_body(SolverArgs A, int64_t t0, int64_t stride) {
    const int n = A.s + 1;  // nodes per axis in the updated box
    const int64_t total = (int64_t)n * n * n;
    const double c2 = A.c * A.c;
    for (int64_t t = t0; t < total; t += stride) {
        int x, y, z;
        split3(t, n, n, x, y, z);
        ++x; ++y; ++z;
        const int nb = A.s + 2, nf = A.s + 3;
        const double* B0 = A.bc + 3 * fidx(nb, x, y, z);
        const double* Bxm = A.bc + 3 * fidx(nb, x - 1, y, z);
        const double* Bym = A.bc + 3 * fidx(nb, x, y - 1, z);
        const double* Bzm = A.bc + 3 * fidx(nb, x, y, z - 1);
        double J[3];
        read_j(A, x - 1, y - 1, z - 1, J);
        double* E = A.field + 9 * fidx(nf, x, y, z);
        E[0] = E[0] + A.dt * (c2 * (over<kMul>(B0[2] - Bym[2], A.wy, A.iwy) - over<kMul>(B0[1] - Bzm[1], A.wz, A.iwz)) -
                              J[0]);
        E[1] = E[1] + A.dt * (c2 * (over<kMul>(B0[0] - Bzm[0], A.wz, A.iwz) - over<kMul>(B0[2] - Bxm[2], A.wx, A.iwx)) -
                              J[1]);
        E[2] = E[2] + A.dt * (c2 * (over<kMul>(B0[1] - Bxm[1], A.wx, A.iwx) - over<kMul>(B0[0] - Bym[0], A.wy, A.iwy)) -
                              J[2]);
        if (A.n32) A.n32[2 * fidx(nf, x, y, z)] = make_float4((float)E[0], (float)E[1], (float)E[2], 0.f);
    }
}

// Bc at pos in [1, s+1)^3 from the new E at pos and pos + e_i.
template <bool kMul = false>
__device__ __forceinline__ void leapfrog_b_body(SolverArgs A, int64_t t0, int64_t stride) {
    const int n = A.s;
    const int64_t total = (int64_t)n * n * n;
    for (int64_t t = t0; t < total; t += stride) {
        int x, y, z;
        split3(t, n, n, x, y, z);
        ++x; ++y; ++z;
        const int nb = A.s + 2, nf = A.s + 3;
        const double* E0 = A.field + 9 * fidx(nf, x, y, z);
        const double* Ex = A.field + 9 * fidx(nf, x + 1, y, z);
        const double* Ey = A.field + 9 * fidx(nf, x, y + 1, z);
        const double* Ez = A.field + 9 * fidx(nf, x, y, z + 1);
        double* B = A.bc + 3 * fidx(nb, x, y, z);
        B[0] = B[0] - A.dt * (over<kMul>(Ey[2] - E0[2], A.wy, A.iwy) - over<kMul>(Ez[1] - E0[1], A.wz, A.iwz));
        B[1] = B[1] - A.dt * (over<kMul>(Ez[0] - E0[0], A.wz, A.iwz) - over<kMul>(Ex[2] - E0[2], A.wx, A.iwx));
        B[2] = B[2] - A.dt * (over<kMul>(Ex[1] - E0[1], A.wx, A.iwx) - over<kMul>(Ey[0] - E0[0], A.wy, A.iwy));
    }
}

// computeCurlB (field.h:162-193) at node pos from the 8 Bc at pos - (i,j,k).
__device__ __forceinline__ void curl_b(const SolverArgs& A, int x, int y, int z, double& cx, double& cy, double& cz) {
    const int nb = A.s + 2;
    double b[2][2][2][3];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const double* p = A.bc + 3 * fidx(nb, x - i, y - j, z - k);
                b[i][j][k][0] = p[0]; b[i][j][k][1] = p[1]; b[i][j][k][2] = p[2];
            }
    // d/dy of z: (j=0) - (j=1) over the 4 (i,k); d/dz of y: (k=0) - (k=1); ...
    double zdy = .25 * (b[0][0][0][2] - b[0][1][0][2] + b[0][0][1][2] - b[0][1][1][2] + b[1][0][0][2] - b[1][1][0][2] + b[1][0][1][2] - b[1][1][1][2]) / A.wy;
    double ydz = .25 * (b[0][0][0][1] - b[0][0][1][1] + b[1][0][0][1] - b[1][0][1][1] + b[0][1][0][1] - b[0][1][1][1] + b[1][1][0][1] - b[1][1][1][1]) / A.wz;
    cx = zdy - ydz;
    double xdz = .25 * (b[0][0][0][0] - b[0][0][1][0] + b[1][0][0][0] - b[1][0][1][0] + b[0][1][0][0] - b[0][1][1][0] + b[1][1][0][0] - b[1][1][1][0]) / A.wz;
    double zdx = .25 * (b[0][0][0][2] - b[1][0][0][2] + b[0][0][1][2] - b[1][0][1][2] + b[0][1][0][2] - b[1][1][0][2] + b[0][1][1][2] - b[1][1][1][2]) / A.wx;
    cy = xdz - zdx;
    double ydx = .25 * (b[0][0][0][1] - b[1][0][0][1] + b[0][0][1][1] - b[1][0][1][1] + b[0][1][0][1] - b[1][1][0][1] + b[0][1][1][1] - b[1][1][1][1]) / A.wx;
    double xdy = .25 * (b[0][0][0][0] - b[0][1][0][0] + b[0][0][1][0] - b[0][1][1][0] + b[1][0][0][0] - b[1][1][0][0] + b[1][0][1][0] - b[1][1][1][0]) / A.wy;
    cz = ydx - xdy;
}

// computeCurlE (field.h:198-229) at centre pos from the 8 node E at pos + (i,j,k).
__device__ __forceinline__ void curl_e(const SolverArgs& A, int x, int y, int z, double& cx, double& cy, double& cz) {
    const int nf = A.s + 3;
    double e[2][2][2][3];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const double* p = A.field + 9 * fidx(nf, x + i, y + j, z + k);
                e[i][j][k][0] = p[0]; e[i][j][k][1] = p[1]; e[i][j][k][2] = p[2];
            }
    double zdy = .25 * (e[0][1][0][2] - e[0][0][0][2] + e[0][1][1][2] - e[0][0][1][2] + e[1][1][0][2] - e[1][0][0][2] + e[1][1][1][2] - e[1][0][1][2]) / A.wy;
    double ydz = .25 * (e[0][0][1][1] - e[0][0][0][1] + e[1][0][1][1] - e[1][0][0][1] + e[0][1][1][1] - e[0][1][0][1] + e[1][1][1][1] - e[1][1][0][1]) / A.wz;
    cx = zdy - ydz;
    double xdz = .25 * (e[0][0][1][0] - e[0][0][0][0] + e[1][0][1][0] - e[1][0][0][0] + e[0][1][1][0] - e[0][1][0][0] + e[1][1][1][0] - e[1][1][0][0]) / A.wz;
    double zdx = .25 * (e[1][0][0][2] - e[0][0][0][2] + e[1][0][1][2] - e[0][0][1][2] + e[1][1][0][2] - e[0][1][0][2] + e[1][1][1][2] - e[0][1][1][2]) / A.wx;
    cy = xdz - zdx;
    double ydx = .25 * (e[1][0][0][1] - e[0][0][0][1] + e[1][0][1][1] - e[0][0][1][1] + e[1][1][0][1] - e[0][1][0][1] + e[1][1][1][1] - e[0][1][1][1]) / A.wx;
    double xdy = .25 * (e[0][1][0][0] - e[0][0][0][0] + e[0][1][1][0] - e[0][0][1][0] + e[1][1][0][0] - e[1][0][0][0] + e[1][1][1][0] - e[1][0][1][0]) / A.wy;
    cz = ydx - xdy;
}

__device__ __forceinline__ void forward_e_body(SolverArgs A, int64_t t0, int64_t stride) {
    const int n = A.s + 1;
    const int64_t total = (int64_t)n * n * n;
    for (int64_t t = t0; t < total; t += stride) {
        int x, y, z;
        split3(t, n, n, x, y, z);
        ++x; ++y; ++z;
        double cx, cy, cz;
        curl_b(A, x, y, z, cx, cy, cz);
        double J[3];
        read_j(A, x - 1, y - 1, z - 1, J);
        double* E = A.field + 9 * fidx(A.s + 3, x, y, z);
        E[0] += (A.c * cx - J[0]) * A.dt;
        E[1] += (A.c * cy - J[1]) * A.dt;
        E[2] += (A.c * cz - J[2]) * A.dt;
        if (A.n32) A.n32[2 * fidx(A.s + 3, x, y, z)] = make_float4((float)E[0], (float)E[1], (float)E[2], 0.f);
    }
}

__device__ __forceinline__ void forward_b_body(SolverArgs A, int64_t t0, int64_t stride) {
    const int n = A.s;
    const int64_t total = (int64_t)n * n * n;
    for (int64_t t = t0; t < total; t += stride) {
        int x, y, z;
        split3(t, n, n, x, y, z);
        ++x; ++y; ++z;
        double cx, cy, cz;
        curl_e(A, x, y, z, cx, cy, cz);
        double* B = A.bc + 3 * fidx(A.s + 2, x, y, z);
        B[0] -= A.c * cx * A.dt;
        B[1] -= A.c * cy * A.dt;
        B[2] -= A.c * cz * A.dt;
    }
}

// node B at pos in [1, s+2)^3 = 1/8 sum of Bc at pos - (i,j,k)
__device__ __forceinline__ void interp_c2n_body(SolverArgs A, int64_t t0, int64_t stride) {
    const int n = A.s + 1;
    const int64_t total = (int64_t)n * n * n;
    for (int64_t t = t0; t < total; t += stride) {
        int x, y, z;
        split3(t, n, n, x, y, z);
        ++x; ++y; ++z;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
                for (int k = 0; k < 2; k++) {
                    const double* p = A.bc + 3 * fidx(A.s + 2, x - i, y - j, z - k);
                    a0 = a0 + p[0]; a1 = a1 + p[1]; a2 = a2 + p[2];
                }
        double* B = A.field + 9 * fidx(A.s + 3, x, y, z) + 3;
        B[0] = .125 * a0; B[1] = .125 * a1; B[2] = .125 * a2;
        if (A.n32) A.n32[2 * fidx(A.s + 3, x, y, z) + 1] = make_float4((float)B[0], (float)B[1], (float)B[2], 0.f);
    }
}

// The gather form of the reference adds, at node index 0 and index s of an
// axis, the same two cells (periodic wrap of the cell index): the final value
// of a node is the sum of the raw deposits over its image set {0, s} on every
// axis where it lies on the boundary. Then J = (Js / vol) [/ 8].
__device__ __forceinline__ void j_finalize_body(int sx, int sy, int sz, double* J, double* rho, double vol, int div8,
                                                int64_t t0, int64_t stride) {
    const int64_t total = (int64_t)sx * sy * sz;
    const int ny = sy + 1, nz = sz + 1;
    for (int64_t t = t0; t < total; t += stride) {
        int x, y, z;
        split3(t, sy, sz, x, y, z);
        const int nxs = x == 0 ? 2 : 1, nys = y == 0 ? 2 : 1, nzs = z == 0 ? 2 : 1;
        double a[4] = {0.0, 0.0, 0.0, 0.0};
        for (int i = 0; i < nxs; ++i)
            for (int j = 0; j < nys; ++j)
                for (int k = 0; k < nzs; ++k) {
                    const int64_t n = ((int64_t)(i ? sx : x) * ny + (j ? sy : y)) * nz + (k ? sz : z);
                    a[0] += J[3 * n]; a[1] += J[3 * n + 1]; a[2] += J[3 * n + 2]; a[3] += rho[n];
                }
        for (int c = 0; c < 4; ++c) {
            a[c] = a[c] / vol;
            if (div8) a[c] = a[c] / 8.0;
        }
        for (int i = 0; i < nxs; ++i)
            for (int j = 0; j < nys; ++j)
                for (int k = 0; k < nzs; ++k) {
                    const int64_t n = ((int64_t)(i ? sx : x) * ny + (j ? sy : y)) * nz + (k ? sz : z);
                    J[3 * n] = a[0]; J[3 * n + 1] = a[1]; J[3 * n + 2] = a[2]; rho[n] = a[3];
                }
    }
}

__global__ void k_node32(const double* field, float4* node32, int64_t nodes) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nodes; t += (int64_t)gridDim.x * blockDim.x) {
        const double* f = field + 9 * t;
        node32[2 * t] = make_float4((float)f[0], (float)f[1], (float)f[2], 0.f);
        node32[2 * t + 1] = make_float4((float)f[3], (float)f[4], (float)f[5], 0.f);
    }
}

__device__ __forceinline__ int64_t grid_t0() { return blockIdx.x * (int64_t)blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t grid_stride() { return (int64_t)gridDim.x * blockDim.x; }

__host__ __device__ inline SolverArgs solver_args(const Geom& g) {
    SolverArgs A;
    A.s = g.sx;
    A.dt = g.dt;
    A.c = g.c;
    A.wx = g.w[0];
    A.wy = g.w[1];
    A.wz = g.w[2];
    A.iwx = 1.0 / g.w[0];
    A.iwy = 1.0 / g.w[1];
    A.iwz = 1.0 / g.w[2];
    A.field = g.field;
    A.bc = g.bcfield;
    A.J = g.J;
    A.n32 = g.node32;
    A.jmode = 0;
    A.jdiv8 = 0;
    A.jvol = g.vol;
    A.jinv = 1.0;
    return A;
}

// single-universe kernels
// both grids' ghost faces in one launch: threads [0, nf_items) the field,
// the rest the Bc grid
__global__ void k_ghost2(double* field, int nf, double* bc, int nb) {
    const int64_t mf = (int64_t)(nf - 2) * (nf - 2) * 9;
    const int64_t t = grid_t0();
    if (t < mf)
        ghost_body(field, nf, 9, t, mf);
    else
        ghost_body(bc, nb, 3, t - mf, (int64_t)(nb - 2) * (nb - 2) * 3);
}
template <bool kMul>
__global__ void k_leapfrog_e(SolverArgs A) { leapfrog_e_body<kMul>(A, grid_t0(), grid_stride()); }
template <bool kMul>
__global__ void k_leapfrog_b(SolverArgs A) { leapfrog_b_body<kMul>(A, grid_t0(), grid_stride()); }
__global__ void k_forward_e(SolverArgs A) { forward_e_body(A, grid_t0(), grid_stride()); }
__global__ void k_forward_b(SolverArgs A) { forward_b_body(A, grid_t0(), grid_stride()); }
__global__ void k_interp_c2n(SolverArgs A) { interp_c2n_body(A, grid_t0(), grid_stride()); }
__global__ void k_j_finalize(int sx, int sy, int sz, double* J, double* rho, double vol, int div8) {
    j_finalize_body(sx, sy, sz, J, rho, vol, div8, grid_t0(), grid_stride());
}
// The same with the normalisation as one multiplication by `inv` (1 / vol
// [/ 8]): for the FP32 path, and wherever vol is a power of two (then the
// product equals the reference's quotients bit for bit).
__global__ void k_j_finalize_mul(int sx, int sy, int sz, double* J, double* rho, double inv) {
    const int64_t total = (int64_t)sx * sy * sz;
    const int ny = sy + 1, nz = sz + 1;
    for (int64_t t = grid_t0(); t < total; t += grid_stride()) {
        int x, y, z;
        split3(t, sy, sz, x, y, z);
        const int nxs = x == 0 ? 2 : 1, nys = y == 0 ? 2 : 1, nzs = z == 0 ? 2 : 1;
        double a[4] = {0.0, 0.0, 0.0, 0.0};
        for (int i = 0; i < nxs; ++i)
            for (int j = 0; j < nys; ++j)
                for (int k = 0; k < nzs; ++k) {
                    const int64_t n = ((int64_t)(i ? sx : x) * ny + (j ? sy : y)) * nz + (k ? sz : z);
                    a[0] += J[3 * n]; a[1] += J[3 * n + 1]; a[2] += J[3 * n + 2]; a[3] += rho[n];
                }
        for (int c = 0; c < 4; ++c) a[c] *= inv;
        for (int i = 0; i < nxs; ++i)
            for (int j = 0; j < nys; ++j)
                for (int k = 0; k < nzs; ++k) {
                    const int64_t n = ((int64_t)(i ? sx : x) * ny + (j ? sy : y)) * nz + (k ? sz : z);
                    J[3 * n] = a[0]; J[3 * n + 1] = a[1]; J[3 * n + 2] = a[2]; rho[n] = a[3];
                }
    }
}

// batched kernels: blockIdx.y is the universe, blockIdx.x strides over its
// items (the grid is sized for the largest universe of the batch)
__global__ void k_ghost_batch(const InstJob* jobs) {
    const Geom& g = jobs[blockIdx.y].g;
    ghost_body(g.field, g.sx + 3, 9, grid_t0(), grid_stride());
    ghost_body(g.bcfield, g.sx + 2, 3, grid_t0(), grid_stride());
}
__global__ void k_leapfrog_e_batch(const InstJob* jobs) {
    leapfrog_e_body(solver_args(jobs[blockIdx.y].g), grid_t0(), grid_stride());
}
__global__ void k_leapfrog_b_batch(const InstJob* jobs) {
    leapfrog_b_body(solver_args(jobs[blockIdx.y].g), grid_t0(), grid_stride());
}
__global__ void k_forward_e_batch(const InstJob* jobs) {
    forward_e_body(solver_args(jobs[blockIdx.y].g), grid_t0(), grid_stride());
}
__global__ void k_forward_b_batch(const InstJob* jobs) {
    forward_b_body(solver_args(jobs[blockIdx.y].g), grid_t0(), grid_stride());
}
__global__ void k_interp_c2n_batch(const InstJob* jobs) {
    interp_c2n_body(solver_args(jobs[blockIdx.y].g), grid_t0(), grid_stride());
}
__global__ void k_j_finalize_batch(const InstJob* jobs) {
    const InstJob& b = jobs[blockIdx.y];
    j_finalize_body(b.g.sx, b.g.sy, b.g.sz, b.g.J, b.g.rho, b.g.vol, b.div8, grid_t0(), grid_stride());
}

// ---- compensated reductions ----------------------------------------------------
// Neumaier's improved Kahan summation: (s, c) with s + c the running sum.
struct Neu {
    double s, c;
    __device__ void add(double x) {
        double t = s + x;
        if (fabs(s) >= fabs(x)) c += (s - t) + x;
        else c += (x - t) + s;
        s = t;
    }
    __device__ void merge(const Neu& o) {
        add(o.s);
        c += o.c;
    }
};

__device__ __forceinline__ Neu shfl_neu(Neu a, int off) {
    Neu b;
    b.s = __shfl_down_sync(0xffffffffu, a.s, off);
    b.c = __shfl_down_sync(0xffffffffu, a.c, off);
    return b;
}

// Block-level merge of kQ compensated sums; thread 0 writes 2*kQ doubles.
template <int kQ>
__device__ void block_merge(Neu (&acc)[kQ], double* out) {
    __shared__ Neu sm[32][kQ];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kQ; ++q)
        for (int off = 16; off > 0; off >>= 1) acc[q].merge(shfl_neu(acc[q], off));
    if (lane == 0)
        for (int q = 0; q < kQ; ++q) sm[wid][q] = acc[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) / 32;
        for (int q = 0; q < kQ; ++q) {
            Neu t = {0.0, 0.0};
            for (int w = 0; w < nw; ++w) t.merge(sm[w][q]);
            out[2 * q] = t.s;
            out[2 * q + 1] = t.c;
        }
    }
}

// Particle sums of one population: sum (q/qom)|v|, sum 1/2 (q/qom)|v|^2,
// sum q (cell.h:1315-1338), over the particles in slots (slots beyond
// count[c] are skipped) and those waiting in the pending list.
template <typename T>
__device__ __forceinline__ void add_particle(Neu (&acc)[3], double m, double q, T u, T v, T w) {
    const double a = (double)u, b = (double)v, d = (double)w;
    double ss = a * a;
    ss += b * b;
    ss += d * d;
    acc[0].add(m * sqrt(ss));
    acc[1].add(0.5 * m * ss);
    acc[2].add(q);
}

template <typename T>
__global__ void k_reduce_particles(const T* u, const T* v, const T* w, const int64_t* start, const int32_t* count,
                                   int ncells, const Mover<T>* pend, const uint32_t* npend, double q, double qom,
                                   double* partial) {
    Neu acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    const double m = q / qom;
    for (int c = blockIdx.x; c < ncells; c += gridDim.x) {
        const int64_t s0 = start[c];
        const int n = count[c];
        for (int i = threadIdx.x; i < n; i += blockDim.x) add_particle<T>(acc, m, q, u[s0 + i], v[s0 + i], w[s0 + i]);
    }
    const uint32_t np = *npend;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x)
        add_particle<T>(acc, m, q, pend[i].u, pend[i].v, pend[i].w);
    block_merge<3>(acc, partial + 6 * blockIdx.x);
}

// Field energies over [1, s+2)^3: vol * |E|^2 / 4pi and vol * |B + Bext|^2 /
// 4pi with vol = cell volume / 2 (field.h:443-459).
__global__ void k_reduce_fields(const double* field, int s, double vol, double four_pi, double* partial) {
    Neu acc[2] = {{0, 0}, {0, 0}};
    const int n = s + 1, nf = s + 3;
    const int64_t total = (int64_t)n * n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int x, y, z;
        split3(t, n, n, x, y, z);
        ++x; ++y; ++z;
        const double* f = field + 9 * fidx(nf, x, y, z);
        double e = f[0] * f[0];
        e += f[1] * f[1];
        e += f[2] * f[2];
        const double b0 = f[3] + f[6], b1 = f[4] + f[7], b2 = f[5] + f[8];
        double b = b0 * b0;
        b += b1 * b1;
        b += b2 * b2;
        acc[0].add(vol * e / four_pi);
        acc[1].add(vol * b / four_pi);
    }
    block_merge<2>(acc, partial + 4 * blockIdx.x);
}

// Final merge of `blocks` partial records of kq (s, c) pairs: warp q merges
// quantity q, lane l the records l, l + 32, ... in order, then the lanes'
// sums in a fixed shuffle tree (the same order every call).
__global__ void k_reduce_final(const double* partial, int blocks, int kq, double* out) {
    const int lane = threadIdx.x & 31, q = threadIdx.x >> 5;
    if (blockIdx.x != 0 || q >= kq) return;
    Neu t = {0.0, 0.0};
    for (int b = lane; b < blocks; b += 32) {
        t.add(partial[2 * kq * b + 2 * q]);
        t.c += partial[2 * kq * b + 2 * q + 1];
    }
    for (int off = 16; off > 0; off >>= 1) t.merge(shfl_neu(t, off));
    if (lane == 0) out[q] = t.s + t.c;
}

inline int grid_for(int64_t n, int threads, int64_t max_blocks = 152 * 32) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (int)b;
}


}  // namespace

// ---- host launchers ------------------------------------------------------------

int launch_ghost(const Geom& g, cudaStream_t st) {
    const int nf = g.sx + 3, nb = g.sx + 2;
    const int64_t items = (int64_t)(nf - 2) * (nf - 2) * 9 + (int64_t)(nb - 2) * (nb - 2) * 3;
    k_ghost2<<<(unsigned)((items + 255) / 256), 256, 0, st>>>(g.field, nf, g.bcfield, nb);
    return 1;
}

static bool pow2(double v) {
    int e = 0;
    return std::frexp(v, &e) == 0.5;
}

// raw J: read as the J finalisation (div8 / exact as launch_j_finalize's)
// would store it
static void set_raw_j(SolverArgs& A, const Geom& g, bool div8, bool exact);

int launch_leapfrog(const Geom& g, bool refresh_node_b, bool exact, cudaStream_t st, bool raw_j, bool div8,
                    cudaEvent_t after_e) {
    SolverArgs A = solver_args(g);
    if (raw_j) set_raw_j(A, g, div8, exact);
    const int64_t ne = (int64_t)(g.sx + 1) * (g.sx + 1) * (g.sx + 1);
    const bool mul = !exact || (pow2(g.w[0]) && pow2(g.w[1]) && pow2(g.w[2]));
    if (mul) {
        k_leapfrog_e<true><<<grid_for(ne, 256), 256, 0, st>>>(A);
        if (after_e) cudaEventRecord(after_e, st);
        k_leapfrog_b<true><<<grid_for((int64_t)g.sx * g.sx * g.sx, 256), 256, 0, st>>>(A);
    } else {
        k_leapfrog_e<false><<<grid_for(ne, 256), 256, 0, st>>>(A);
        if (after_e) cudaEventRecord(after_e, st);
        k_leapfrog_b<false><<<grid_for((int64_t)g.sx * g.sx * g.sx, 256), 256, 0, st>>>(A);
    }
    if (refresh_node_b) {
        k_interp_c2n<<<grid_for(ne, 256), 256, 0, st>>>(A);
        return 3;
    }
    return 2;
}

int launch_forward(const Geom& g, cudaStream_t st, bool raw_j, bool div8, bool exact, cudaEvent_t after_e) {
    SolverArgs A = solver_args(g);
    if (raw_j) set_raw_j(A, g, div8, exact);
    const int64_t ne = (int64_t)(g.sx + 1) * (g.sx + 1) * (g.sx + 1);
    k_forward_e<<<grid_for(ne, 256), 256, 0, st>>>(A);
    if (after_e) cudaEventRecord(after_e, st);
    k_forward_b<<<grid_for((int64_t)g.sx * g.sx * g.sx, 256), 256, 0, st>>>(A);
    k_interp_c2n<<<grid_for(ne, 256), 256, 0, st>>>(A);
    return 3;
}

static void set_raw_j(SolverArgs& A, const Geom& g, bool div8, bool exact) {
    A.jdiv8 = div8 ? 1 : 0;
    A.jvol = g.vol;
    A.jinv = div8 ? 1.0 / g.vol / 8.0 : 1.0 / g.vol;
    A.jmode = exact && !pow2(g.vol) ? 1 : 2;  // launch_j_finalize's choice
}

int launch_j_finalize(const Geom& g, bool div8, bool exact, cudaStream_t st) {
    if (exact && !pow2(g.vol)) {  // vol = 2^k: 1 / vol is exact
        k_j_finalize<<<grid_for((int64_t)g.sx * g.sy * g.sz, 256), 256, 0, st>>>(g.sx, g.sy, g.sz, g.J, g.rho,
                                                                                 g.vol, div8 ? 1 : 0);
    } else {
        const double inv = div8 ? 1.0 / g.vol / 8.0 : 1.0 / g.vol;
        k_j_finalize_mul<<<grid_for((int64_t)g.sx * g.sy * g.sz, 256), 256, 0, st>>>(g.sx, g.sy, g.sz, g.J, g.rho,
                                                                                     inv);
    }
    return 1;
}

int launch_node32(const Geom& g, float4* node32, cudaStream_t st) {
    const int64_t nodes = (int64_t)(g.sx + 3) * (g.sy + 3) * (g.sz + 3);
    k_node32<<<grid_for(nodes, 256), 256, 0, st>>>(g.field, node32, nodes);
    return 1;
}

// batched launchers: `ninst` universes, `max_s` the largest cells per axis
int launch_ghost_batch(const InstJob* jobs, int ninst, int max_s, cudaStream_t st) {
    const int64_t m = (int64_t)(max_s + 1) * (max_s + 1) * 9;
    k_ghost_batch<<<dim3(grid_for(m, 256, 64), ninst), 256, 0, st>>>(jobs);
    return 1;
}

int launch_leapfrog_batch(const InstJob* jobs, int ninst, int max_s, bool refresh_node_b, cudaStream_t st) {
    const int64_t ne = (int64_t)(max_s + 1) * (max_s + 1) * (max_s + 1);
    const unsigned gx = grid_for(ne, 256, 64);
    k_leapfrog_e_batch<<<dim3(gx, ninst), 256, 0, st>>>(jobs);
    k_leapfrog_b_batch<<<dim3(gx, ninst), 256, 0, st>>>(jobs);
    if (!refresh_node_b) return 2;
    k_interp_c2n_batch<<<dim3(gx, ninst), 256, 0, st>>>(jobs);
    return 3;
}

int launch_forward_batch(const InstJob* jobs, int ninst, int max_s, cudaStream_t st) {
    const int64_t ne = (int64_t)(max_s + 1) * (max_s + 1) * (max_s + 1);
    const unsigned gx = grid_for(ne, 256, 64);
    k_forward_e_batch<<<dim3(gx, ninst), 256, 0, st>>>(jobs);
    k_forward_b_batch<<<dim3(gx, ninst), 256, 0, st>>>(jobs);
    k_interp_c2n_batch<<<dim3(gx, ninst), 256, 0, st>>>(jobs);
    return 3;
}

int launch_j_finalize_batch(const InstJob* jobs, int ninst, int64_t max_cells, cudaStream_t st) {
    k_j_finalize_batch<<<dim3(grid_for(max_cells, 256, 64), ninst), 256, 0, st>>>(jobs);
    return 1;
}

int reduce_blocks() { return 152 * 4; }

template <typename T>
int launch_reduce_particles(const Pop<T>& P, int ncells, double* partial, cudaStream_t st) {
    k_reduce_particles<T><<<reduce_blocks(), 256, 0, st>>>(P.u, P.v, P.w, P.start, P.count, ncells, P.pending_in,
                                                            P.pending_in_count, P.q, P.qom, partial);
    return 1;
}
template int launch_reduce_particles<float>(const Pop<float>&, int, double*, cudaStream_t);
template int launch_reduce_particles<double>(const Pop<double>&, int, double*, cudaStream_t);

int launch_reduce_fields(const Geom& g, double* partial, cudaStream_t st) {
    const double vol = 0.5 * g.w[0] * g.w[1] * g.w[2];
    const double four_pi = 16.0 * atan(1.0);
    k_reduce_fields<<<reduce_blocks(), 256, 0, st>>>(g.field, g.sx, vol, four_pi, partial);
    return 1;
}

int launch_reduce_final(const double* partial, int blocks, int kq, double* out, cudaStream_t st) {
    k_reduce_final<<<1, 32 * kq, 0, st>>>(partial, blocks, kq, out);
    return 1;
}

}  // namespace ipg
