// FP32 particle physics shared by the FP32 kernels, and the kernels that use
// it one particle at a time: particles waiting for a slot (k_push_pending32)
// and the per-cell field polynomial (k_cell_coef / k_cell_coef32). The bulk
// push is push32_pipe.cuh.
//   * fields: per-cell trilinear polynomial f = c0 + c1 x + c2 y + c3 z +
//     c4 xy + c5 xz + c6 yz + c7 xyz of every E and B component (the
//     expansion of trilinearInterpolationF2P, cell.h:867-885, with node
//     values from the cell's 8 corners as in cell.h:905-937): 7 FMAs per
//     component;
//   * dipole: |r|^-5 from one rsqrt;
//   * sub-cycles (cell.h:947-952): dt/dt_sub = K |B|^2 with K per species.
#pragma once

#include "particle_kernels.cuh"

namespace ipg {

// E (and B) at cell-relative r from the cell's coefficients: component q
// (Ex, Ey, Ez, Bx, By, Bz) owns coef[q * 8 + m], m = 1, x, y, z, xy, xz, yz,
// xyz: two float4 per component, evaluated one component at a time.
__device__ __forceinline__ void eval_fields(const float* __restrict__ coef, float x, float y, float z, float (&f)[6]) {
    const float4* c4 = reinterpret_cast<const float4*>(coef);
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const float4 lo = __ldg(c4 + 2 * q), hi = __ldg(c4 + 2 * q + 1);
        // lo = (c0, cx, cy, cz), hi = (cxy, cxz, cyz, cxyz)
        const float a = fmaf(y, hi.w, hi.y);     // x z terms
        float b = fmaf(y, hi.x, lo.y);           // x terms
        b = fmaf(z, a, b);
        const float gz = fmaf(z, hi.z, lo.z);    // y terms
        float r = fmaf(y, gz, lo.x);
        r = fmaf(z, lo.w, r);
        f[q] = fmaf(x, b, r);
    }
}

// mover + export of one particle (FP32, cell-relative); same outcomes as
// step_particle(..., PState<float>&, ...).
__device__ __forceinline__ int step32(const Geom& g, const Push32Const& pc, const float* __restrict__ coef, int cx,
                                      int cy, int cz, float ox, float oy, float oz, PState<float>& p, int& dest) {
    float E[6];
    if (g.mover == 1) {
        eval_fields(coef, p.x, p.y, p.z, E);
    } else {
#pragma unroll
        for (int q = 0; q < 6; ++q) E[q] = 0.f;
    }
    if (g.mover != 1 || (g.flags & 4u)) {
        const float X = fmaf(p.x, pc.w[0], ox), Y = fmaf(p.y, pc.w[1], oy), Z = fmaf(p.z, pc.w[2], oz);
        const float r2 = fmaf(X, X, fmaf(Y, Y, Z * Z));
        const float ir = rsqrtf(r2), ir2 = ir * ir;
        const float fac1 = pc.mft * (ir2 * ir2 * ir);
        E[3] = fmaf(3.f * X * Z, fac1, E[3]);
        E[4] = fmaf(3.f * Y * Z, fac1, E[4]);
        E[5] = fmaf(fmaf(2.f * Z, Z, -fmaf(X, X, Y * Y)), fac1, E[5]);
    }
    const float bmag = fmaf(E[3], E[3], fmaf(E[4], E[4], E[5] * E[5]));
    const float ratio = pc.k_sub * bmag;
    int ns = 0;
    if (ratio >= 0.f && ratio < 2147483647.f) {
        ns = (int)ratio + 1;
        ns = ns < 100 ? ns : 100;
    }
    if (ns > 0) {
        const float dts = __fdividef(pc.dt, (float)ns);
        const float k = pc.qom * 0.5f * dts;
        const float tx = k * E[3], ty = k * E[4], tz = k * E[5];
        // the rotation factor 2 / (1 + |t|^2) keeps |v| through the rotation:
        // correctly rounded reciprocal here
        const float inv = __frcp_rn(fmaf(tx, tx, fmaf(ty, ty, fmaf(tz, tz, 1.f))));
        const float sx = 2.f * tx * inv, sy = 2.f * ty * inv, sz = 2.f * tz * inv;
        const float kex = k * E[0], key = k * E[1], kez = k * E[2];
        const float ax = dts * pc.inv_w[0], ay = dts * pc.inv_w[1], az = dts * pc.inv_w[2];
        for (int s = 0; s < ns; ++s) {
            const float mx = p.u + kex, my = p.v + key, mz = p.w + kez;
            const float px = mx + (my * tz - mz * ty);
            const float py = my + (mz * tx - mx * tz);
            const float pz = mz + (mx * ty - my * tx);
            p.u = mx + (py * sz - pz * sy) + kex;
            p.v = my + (pz * sx - px * sz) + key;
            p.w = mz + (px * sy - py * sx) + kez;
            p.x = fmaf(p.u, ax, p.x);
            p.y = fmaf(p.v, ay, p.y);
            p.z = fmaf(p.w, az, p.z);
        }
    }
    // export (cell.h:1093-1146) in cell-relative coordinates
    const int pos[3] = {cx, cy, cz};
    const int size[3] = {g.sx, g.sy, g.sz};
    float R[3] = {p.x, p.y, p.z};
    bool invert = false, drop = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (pos[a] == 0 && R[a] < 0.f) {
            if (g.bc_lo[a] == 0) { invert = true; R[a] += 0.5f; }
            else if (g.bc_lo[a] == 2) drop = true;
        } else if (pos[a] == size[a] - 1 && R[a] > 1.f) {
            if (g.bc_hi[a] == 0) { invert = true; R[a] -= 0.5f; }
            else if (g.bc_hi[a] == 2) drop = true;
        }
    }
    if (invert) { p.u = -p.u; p.v = -p.v; p.w = -p.w; }
    if (drop) return kDrop;
    {
        const float dx = fmaf(R[0], pc.w[0], ox - pc.center[0]);
        const float dy = fmaf(R[1], pc.w[1], oy - pc.center[1]);
        const float dz = fmaf(R[2], pc.w[2], oz - pc.center[2]);
        if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= pc.planet_r2) return kDrop;  // cell.h:1123-1128
    }
    int d[3];
    bool out = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        d[a] = R[a] < 0.f ? -1 : (R[a] > 1.f ? 1 : 0);
        out |= d[a] != 0;
        R[a] -= (float)d[a];
    }
    p.x = R[0]; p.y = R[1]; p.z = R[2];
    if (!out) return kStay;
    int n[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int t = pos[a] + d[a];
        n[a] = t < 0 ? t + size[a] : (t >= size[a] ? t - size[a] : t);
    }
    dest = cell_id(g, n[0], n[1], n[2]);
    return kMove;
}

// Pending particles (no slot last step) with the same physics; threads
// t0, t0 + stride, ... of the pending list.
__device__ __forceinline__ void push_pending32_body(const Geom& g, const Pop<float>& P, const Push32Const& pc,
                                                    uint32_t t0, uint32_t stride) {
    const uint32_t n = *P.pending_in_count;
    for (uint32_t i = t0; i < n; i += stride) {
        Mover<float> m = P.pending_in[i];
        PState<float> p = {m.x, m.y, m.z, m.u, m.v, m.w};
        int cx, cy, cz;
        cell_coords(g, m.cell, cx, cy, cz);
        const float ox = fmaf((float)cx, pc.w[0], pc.origin[0]);
        const float oy = fmaf((float)cy, pc.w[1], pc.origin[1]);
        const float oz = fmaf((float)cz, pc.w[2], pc.origin[2]);
        int dest = m.cell;
        const int outcome = step32(g, pc, g.cellcoef + (size_t)m.cell * 48, cx, cy, cz, ox, oy, oz, p, dest);
        if (outcome == kDrop) {
            atomicAdd(&P.ctr->removed, 1u);
            continue;
        }
        if (outcome == kMove) atomicAdd(&P.ctr->migrated, 1u);
        Mover<float> o = {dest, m.id, p.x, p.y, p.z, p.u, p.v, p.w};
        const uint32_t k = atomicAdd(&P.ctr->outbox, 1u);
        if (k < P.outbox_cap) {
            P.outbox[k] = o;
            register_arrival(P, k, o);
        } else {
            atomicAdd(&P.ctr->lost, 1u);
        }
        if (g.deposit) deposit_one<float>(g, dest, p, P.q);
    }
}

// population blockIdx.y of the set, pc.c[blockIdx.y] its push constants
__global__ void k_push_pending32(Geom g, const __grid_constant__ PopSet<float> S,
                                 const __grid_constant__ Push32Set pc) {
    push_pending32_body(g, S.p[blockIdx.y], pc.c[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x,
                        gridDim.x * blockDim.x);
}

// Cell coefficients of the trilinear field polynomial, stored FP32:
// coefficient m of component q (Ex, Ey, Ez, Bx, By, Bz) of cell c at
// coef[c * 48 + q * 8 + m]; monomials m = 1, x, y, z, xy, xz, yz, xyz. One
// thread per (cell, component): the seven corner differences from corner
// (0,0,0) are taken in FP64 and rounded once, the mixed terms are then FP32
// sums of those differences (a few FP64 operations per coefficient instead
// of an FP64 polynomial: GB300's FP64 rate is a small fraction of FP32's).
__device__ __forceinline__ void cell_coef_body(const double* __restrict__ field, int sx, int sy, int sz, double scale,
                                               float* coef, int64_t t0, int64_t stride) {
    const int64_t total = (int64_t)sx * sy * sz * 6;
    const float fs = (float)scale;
    for (int64_t t = t0; t < total; t += stride) {
        const int q = (int)(t % 6);
        const int64_t c = t / 6;
        int x, y, z;
        split3(c, sy, sz, x, y, z);
        const int64_t sy3 = sy + 3, sz3 = sz + 3;
        const double* f0 = field + 9 * (((int64_t)(x + 1) * sy3 + (y + 1)) * sz3 + (z + 1)) + q;
        const int64_t dx = 9 * sy3 * sz3, dy = 9 * sz3, dz = 9;
        const double f000 = __ldg(f0);
        const float d100 = (float)(__ldg(f0 + dx) - f000), d010 = (float)(__ldg(f0 + dy) - f000);
        const float d001 = (float)(__ldg(f0 + dz) - f000), d110 = (float)(__ldg(f0 + dx + dy) - f000);
        const float d101 = (float)(__ldg(f0 + dx + dz) - f000), d011 = (float)(__ldg(f0 + dy + dz) - f000);
        const float d111 = (float)(__ldg(f0 + dx + dy + dz) - f000);
        float m[8];
        m[0] = (float)f000;
        m[1] = d100;
        m[2] = d010;
        m[3] = d001;
        m[4] = d110 - d100 - d010;
        m[5] = d101 - d100 - d001;
        m[6] = d011 - d010 - d001;
        m[7] = ((d111 - d110) - (d101 + d011)) + (d100 + d010 + d001);
        if (scale != 1.0) {
            m[0] = (float)(f000 * scale);
#pragma unroll
            for (int k = 1; k < 8; ++k) m[k] *= fs;
        }
        float4* out = reinterpret_cast<float4*>(coef + c * 48 + q * 8);
        out[0] = make_float4(m[0], m[1], m[2], m[3]);
        out[1] = make_float4(m[4], m[5], m[6], m[7]);
    }
}

__global__ void k_cell_coef(const double* __restrict__ field, int sx, int sy, int sz, double scale, float* coef) {
    cell_coef_body(field, sx, sy, sz, scale, coef, blockIdx.x * (int64_t)blockDim.x + threadIdx.x,
                   (int64_t)gridDim.x * blockDim.x);
}

// The same coefficients from the FP32 node copy (n32: {Ex,Ey,Ez,0},
// {Bx,By,Bz,0} per node of the (s+3)^3 field grid), one thread per cell:
// sixteen 16-byte loads and FP32 corner differences.
__global__ void k_cell_coef32(const float4* __restrict__ n32, int sx, int sy, int sz, float scale, float* coef) {
    const int64_t total = (int64_t)sx * sy * sz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < total;
         c += (int64_t)gridDim.x * blockDim.x) {
        int x, y, z;
        split3(c, sy, sz, x, y, z);
        const int64_t sy3 = sy + 3, sz3 = sz + 3;
        const int64_t n0 = ((int64_t)(x + 1) * sy3 + (y + 1)) * sz3 + (z + 1);
        const int64_t dx = sy3 * sz3, dy = sz3;
        float f[8][6];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int64_t n = n0 + ((k & 1) ? dx : 0) + ((k & 2) ? dy : 0) + ((k & 4) ? 1 : 0);
            const float4 e = __ldg(n32 + 2 * n), b = __ldg(n32 + 2 * n + 1);
            f[k][0] = e.x; f[k][1] = e.y; f[k][2] = e.z;
            f[k][3] = b.x; f[k][4] = b.y; f[k][5] = b.z;
        }
        float4* out = reinterpret_cast<float4*>(coef + c * 48);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            // corner k = i + 2 j + 4 l at (x + i, y + j, z + l)
            const float f000 = f[0][q], d100 = f[1][q] - f000, d010 = f[2][q] - f000, d001 = f[4][q] - f000;
            const float d110 = f[3][q] - f000, d101 = f[5][q] - f000, d011 = f[6][q] - f000, d111 = f[7][q] - f000;
            const float m1 = d100, m2 = d010, m3 = d001;
            const float m4 = d110 - d100 - d010, m5 = d101 - d100 - d001, m6 = d011 - d010 - d001;
            const float m7 = ((d111 - d110) - (d101 + d011)) + (d100 + d010 + d001);
            out[2 * q] = make_float4(f000 * scale, m1 * scale, m2 * scale, m3 * scale);
            out[2 * q + 1] = make_float4(m4 * scale, m5 * scale, m6 * scale, m7 * scale);
        }
    }
}

// ---- batched ensemble (tables as in particles_impl.cuh) ---------------------
__global__ void k_push_pending32_batch(const PopJob<float>* __restrict__ jobs) {
    const PopJob<float>& J = jobs[blockIdx.y];
    push_pending32_body(J.g, J.P, J.pc, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// blockIdx.y = universe
__global__ void k_cell_coef_batch(const InstJob* __restrict__ inst) {
    const InstJob& b = inst[blockIdx.y];
    cell_coef_body(b.g.field, b.g.sx, b.g.sy, b.g.sz, b.coef_scale, b.cellcoef,
                   blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

}  // namespace ipg
