// FP32 particle physics shared by the FP32 kernels -- the bulk push
// (push32_pipe.cuh) and the particles waiting for a slot (k_push_pending32)
// run the same functions, so a particle's arithmetic does not depend on the
// path it takes -- and the per-cell field polynomial (k_cell_coef /
// k_cell_coef32).
//   * fields: per-cell trilinear polynomial f = c0 + c1 x + c2 y + c3 z +
//     c4 xy + c5 xz + c6 yz + c7 xyz of every E and B component (the
//     expansion of trilinearInterpolationF2P, cell.h:867-885, with node
//     values from the cell's 8 corners as in cell.h:905-937): 7 packed
//     FP32-pair FMAs per two components;
//   * dipole: |r|^-5 from one rsqrt;
//   * sub-cycles (cell.h:947-952): dt/dt_sub = K |B|^2 with K per species.
#pragma once

#include "particle_kernels.cuh"

namespace ipg {

// What the push needs to know about a particle's cell (four registers).
struct CellInfo {
    float ox, oy, oz;  // cell origin, relative to the dipole centre (0, 0, 0)
    int flags;         // kCell* bits
};
enum : int {
    kCellNear = 1,    // the planet test can remove a particle that stays in the cell
    kCellEdge = 2,    // a face of the cell lies on a reflecting or open domain face
    kCellLoX = 4,     // bits 2..4: the cell is the first along x, y, z; bits 5..7: the last
    kCellHiX = 32,
};

// Cell coordinates of a cell index (no 64-bit division for the sizes the
// push handles).
__device__ __forceinline__ int3 cell_xyz(const Geom& g, const Push32Const& pc, int cell) {
    int3 c;
    if (g.ncells < (1 << 24) && g.sy < 4096 && g.sz < 4096) {
        const int t = fast_div(cell, g.sz, pc.inv_sz);
        c.z = cell - t * g.sz;
        c.x = fast_div(t, g.sy, pc.inv_sy);
        c.y = t - c.x * g.sy;
    } else {
        cell_coords(g, cell, c.x, c.y, c.z);
    }
    return c;
}

__device__ __forceinline__ CellInfo cell_info(const Geom& g, const Push32Const& pc, int cell) {
    const int3 x = cell_xyz(g, pc, cell);
    CellInfo c;
    c.ox = fmaf((float)x.x, pc.w[0], pc.origin[0]);
    c.oy = fmaf((float)x.y, pc.w[1], pc.origin[1]);
    c.oz = fmaf((float)x.z, pc.w[2], pc.origin[2]);
    const int pos[3] = {x.x, x.y, x.z};
    const int size[3] = {g.sx, g.sy, g.sz};
    int f = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (pos[a] == 0 && g.bc_lo[a] != 1) f |= kCellLoX << a;
        if (pos[a] == size[a] - 1 && g.bc_hi[a] != 1) f |= kCellHiX << a;
    }
    if (f) f |= kCellEdge;
    // squared distance of the closed cell box from the planet centre against
    // the planet radius plus 1/64 of the widest cell side: a particle that
    // stays in a cell that is not near lies outside the planet whatever the
    // rounding of the test (cell.h:1123-1128)
    const float lo[3] = {c.ox - pc.center[0], c.oy - pc.center[1], c.oz - pc.center[2]};
    float d2 = 0.f, wmax = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float hi = lo[a] + pc.w[a];
        const float t = lo[a] > 0.f ? lo[a] : (hi < 0.f ? -hi : 0.f);
        d2 = fmaf(t, t, d2);
        wmax = fmaxf(wmax, pc.w[a]);
    }
    const float r = sqrtf(pc.planet_r2) + wmax * (1.f / 64.f);
    if (d2 <= r * r) f |= kCellNear;
    c.flags = f;
    return c;
}

// The CellInfo of lane `src` (warp-wide).
__device__ __forceinline__ CellInfo shfl_cell_info(const CellInfo& c, int src) {
    CellInfo r;
    r.ox = __shfl_sync(0xffffffffu, c.ox, src);
    r.oy = __shfl_sync(0xffffffffu, c.oy, src);
    r.oz = __shfl_sync(0xffffffffu, c.oz, src);
    r.flags = __shfl_sync(0xffffffffu, c.flags, src);
    return r;
}

// Packed FP32 pairs (sm_100+: one instruction for two lanes' worth of
// work; each component rounds exactly as the scalar operation does).
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }

// Two components (a, b) of the cell's trilinear field polynomial at
// (x, y, z), seven packed FMAs; c4 holds the pair's coefficients
// interleaved: (c0a, c0b, cxa, cxb), (cya, cyb, cza, czb),
// (cxya, cxyb, cxza, cxzb), (cyza, cyzb, cxyza, cxyzb).
__device__ __forceinline__ float2 poly32x2(const float4& c01, const float4& c23, const float4& c45, const float4& c67,
                                           float2 x, float2 y, float2 z) {
    const float2 c0 = make_float2(c01.x, c01.y), cx = make_float2(c01.z, c01.w);
    const float2 cy = make_float2(c23.x, c23.y), cz = make_float2(c23.z, c23.w);
    const float2 cxy = make_float2(c45.x, c45.y), cxz = make_float2(c45.z, c45.w);
    const float2 cyz = make_float2(c67.x, c67.y), cxyz = make_float2(c67.z, c67.w);
    const float2 a = fma2(y, cxyz, cxz);  // x z terms
    float2 b = fma2(y, cxy, cx);          // x terms
    b = fma2(z, a, b);
    const float2 gz = fma2(z, cyz, cy);   // y terms
    float2 r = fma2(y, gz, c0);
    r = fma2(z, cz, r);
    return fma2(x, b, r);
}

// Coefficient m (monomials 1, x, y, z, xy, xz, yz, xyz) of component q (Ex,
// Ey, Ez, Bx, By, Bz) within a cell's 48: components in pairs (Ex, Ey),
// (Bx, By), (Ez, Bz) -- the pairs the mover works on -- each pair's
// coefficients interleaved.
__host__ __device__ constexpr int coef_pair(int q) { return q == 2 || q == 5 ? 2 : q / 3; }
__host__ __device__ constexpr int coef_slot(int q) { return q == 5 ? 1 : (q == 2 ? 0 : q % 3); }
__host__ __device__ constexpr int coef_index(int q, int m) { return coef_pair(q) * 16 + m * 2 + coef_slot(q); }
// The inverse: component and monomial stored at position p of a cell's 48.
__host__ __device__ constexpr int coef_comp(int p) {
    return p / 16 == 0 ? (p % 2) : (p / 16 == 1 ? 3 + p % 2 : (p % 2 ? 5 : 2));
}
__host__ __device__ constexpr int coef_mono(int p) { return (p % 16) / 2; }
constexpr bool coef_layout_is_a_bijection() {
    for (int p = 0; p < 48; ++p)
        if (coef_index(coef_comp(p), coef_mono(p)) != p) return false;
    return true;
}
static_assert(coef_layout_is_a_bijection(), "coef_index and its inverse disagree");

// E and B of a particle from its cell's polynomial coefficients (kSmem:
// staged in shared memory; else read from global memory).
template <bool kSmem>
__device__ __forceinline__ void fields_one(const float* __restrict__ coef, const PState<float>& a, float (&E)[6]) {
    const float4* c4 = reinterpret_cast<const float4*>(coef);
    const float2 x = dup2(a.x), y = dup2(a.y), z = dup2(a.z);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float4 c01 = kSmem ? c4[4 * q] : __ldg(c4 + 4 * q);
        const float4 c23 = kSmem ? c4[4 * q + 1] : __ldg(c4 + 4 * q + 1);
        const float4 c45 = kSmem ? c4[4 * q + 2] : __ldg(c4 + 4 * q + 2);
        const float4 c67 = kSmem ? c4[4 * q + 3] : __ldg(c4 + 4 * q + 3);
        const float2 e = poly32x2(c01, c23, c45, c67, x, y, z);
        E[coef_comp(16 * q)] = e.x;
        E[coef_comp(16 * q + 1)] = e.y;
    }
}

// The analytic dipole (cell.h:939-945) added to B: B += (3xz, 3yz,
// 2z^2 - x^2 - y^2) mft / |r|^5, |r|^-5 from one reciprocal square root.
__device__ __forceinline__ void add_dipole(const Push32Const& pc, const CellInfo& ci, const PState<float>& p,
                                           float (&E)[6]) {
    const float2 XY = fma2(make_float2(p.x, p.y), make_float2(pc.w[0], pc.w[1]), make_float2(ci.ox, ci.oy));
    const float X = XY.x, Y = XY.y, Z = fmaf(p.z, pc.w[2], ci.oz);
    const float r2 = fmaf(X, X, fmaf(Y, Y, Z * Z));
    const float ir = rsqrtf(r2), ir2 = ir * ir;
    const float fac1 = pc.mft * (ir2 * ir2 * ir);
    // (3 X Z, 3 Y Z) fac1 added to (Bx, By)
    const float2 b = fma2(mul2(mul2(dup2(3.f), XY), dup2(Z)), dup2(fac1), make_float2(E[3], E[4]));
    E[3] = b.x;
    E[4] = b.y;
    E[5] = fmaf(fmaf(2.f * Z, Z, -fmaf(X, X, Y * Y)), fac1, E[5]);
}

// dt / dt_sub of cell.h:947-952: K |B|^2 with K = k_sub of the species
__device__ __forceinline__ float sub_ratio(float k_sub, const float (&E)[6]) {
    return k_sub * fmaf(E[3], E[3], fmaf(E[4], E[4], E[5] * E[5]));
}

// `ns` Boris sub-cycles (particle.h:24-49) with k = q/m dts / 2 and
// a = dts / w (positions in cell widths): t = k B, s = 2 t / (1 + |t|^2),
// v- = v + k E, v' = v- + v- x t, v+ = v- + v' x s, v = v+ + k E,
// x += v dts. The cross products are fused multiply-adds; the rotation
// factor 2 / (1 + |t|^2) is the hardware reciprocal (relative error ~2^-22:
// |v| changes by that times |t|^2 per rotation, far below the FP32 path's
// stated error).
template <int kFixedNs>
__device__ __forceinline__ void boris32(float k, float ax, float ay, float az, const float (&E)[6], PState<float>& p,
                                        int ns = kFixedNs) {
    const float2 k2 = dup2(k);
    const float2 txy = mul2(k2, make_float2(E[3], E[4]));
    // k E as separate roundings: the adds below must not fuse with them in
    // one kernel and not in another (the batched and single-universe
    // kernels give the same particles bit for bit)
    const float2 kexy = mul2(k2, make_float2(E[0], E[1]));
    const float2 kez_tz = mul2(k2, make_float2(E[2], E[5]));
    const float tx = txy.x, ty = txy.y, tz = kez_tz.y, kez = kez_tz.x;
    const float den = fmaf(tx, tx, fmaf(ty, ty, fmaf(tz, tz, 1.f)));
    const float f = __fdividef(2.f, den);
    const float2 sxy = mul2(txy, dup2(f));
    const float sx = sxy.x, sy = sxy.y, sz = tz * f;
    const float2 axy = make_float2(ax, ay);
    int s = 0;
    do {
        const float2 mxy = add2(make_float2(p.u, p.v), kexy);
        const float mx = mxy.x, my = mxy.y, mz = p.w + kez;
        const float qx = fmaf(my, tz, fmaf(-mz, ty, mx));
        const float qy = fmaf(mz, tx, fmaf(-mx, tz, my));
        const float qz = fmaf(mx, ty, fmaf(-my, tx, mz));
        const float2 uv = add2(make_float2(fmaf(qy, sz, fmaf(-qz, sy, mx)), fmaf(qz, sx, fmaf(-qx, sz, my))), kexy);
        p.u = uv.x;
        p.v = uv.y;
        p.w = fmaf(qx, sy, fmaf(-qy, sx, mz)) + kez;
        const float2 xy = fma2(uv, axy, make_float2(p.x, p.y));
        p.x = xy.x;
        p.y = xy.y;
        p.z = fmaf(p.w, az, p.z);
    } while (kFixedNs == 0 && ++s < ns);
}

// The reference's sub-cycling rule (cell.h:947-952): ns = min(int(ratio) +
// 1, 100) Boris steps of dt / ns; a quotient beyond the int range (or NaN)
// leaves the particle unmoved, as the reference's x86 conversion does. For
// ns = 1 the constants equal the species' one-step constants (k1, a1) bit
// for bit, whichever path a particle takes.
__device__ __forceinline__ void boris_sub(const Push32Const& pc, const Push32Const& sp, float ratio,
                                          const float (&E)[6], PState<float>& p) {
    if (!(ratio < 2147483647.f)) return;
    int ns = (int)ratio + 1;
    ns = ns < 100 ? ns : 100;
    const float dts = ns == 1 ? pc.dt : __fdividef(pc.dt, (float)ns);
    boris32<0>(sp.qom * 0.5f * dts, dts * pc.inv_w[0], dts * pc.inv_w[1], dts * pc.inv_w[2], E, p, ns);
}

// Export of one moved particle (cell.h:1093-1146) in cell-relative
// coordinates: the walls of reflecting / open domain faces (cells on such a
// face only), the planet (cells near it, and every particle that left its
// cell), then the move to a neighbour: kStay, kDrop, or kMove with the move
// in `dir` as (dx + 1) | (dy + 1) << 2 | (dz + 1) << 4 and the position made
// relative to the destination cell. NaN coordinates stay (no axis moves).
__device__ __forceinline__ int export32(const Geom& g, const Push32Const& pc, const CellInfo& ci, PState<float>& p,
                                        int& dir) {
    if (ci.flags & kCellEdge) {
        float* R[3] = {&p.x, &p.y, &p.z};
        bool invert = false, drop = false;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if ((ci.flags & (kCellLoX << a)) && *R[a] < 0.f) {  // a reflecting / open low face
                if (g.bc_lo[a] == 0) { invert = true; *R[a] += 0.5f; }
                else if (g.bc_lo[a] == 2) drop = true;
            } else if ((ci.flags & (kCellHiX << a)) && *R[a] > 1.f) {
                if (g.bc_hi[a] == 0) { invert = true; *R[a] -= 0.5f; }
                else if (g.bc_hi[a] == 2) drop = true;
            }
        }
        if (invert) { p.u = -p.u; p.v = -p.v; p.w = -p.w; }
        if (drop) return kDrop;
    }
    const bool in = p.x >= 0.f && p.x <= 1.f && p.y >= 0.f && p.y <= 1.f && p.z >= 0.f && p.z <= 1.f;
    if ((ci.flags & kCellNear) || !in) {
        const float dx = fmaf(p.x, pc.w[0], ci.ox - pc.center[0]);
        const float dy = fmaf(p.y, pc.w[1], ci.oy - pc.center[1]);
        const float dz = fmaf(p.z, pc.w[2], ci.oz - pc.center[2]);
        if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= pc.planet_r2) return kDrop;  // cell.h:1123-1128
    }
    if (in) return kStay;
    const float fx = p.x < 0.f ? -1.f : (p.x > 1.f ? 1.f : 0.f);
    const float fy = p.y < 0.f ? -1.f : (p.y > 1.f ? 1.f : 0.f);
    const float fz = p.z < 0.f ? -1.f : (p.z > 1.f ? 1.f : 0.f);
    p.x -= fx;
    p.y -= fy;
    p.z -= fz;
    if (fx == 0.f && fy == 0.f && fz == 0.f) return kStay;
    dir = ((int)fx + 1) | (((int)fy + 1) << 2) | (((int)fz + 1) << 4);
    return kMove;
}

// Mover + export of one particle: fields, sub-cycled Boris, export.
template <bool kSmemCoef, bool kGather, bool kDipole>
__device__ __forceinline__ int step32f(const Geom& g, const Push32Const& pc, const Push32Const& sp,
                                       const float* __restrict__ coef, const CellInfo& ci, PState<float>& p,
                                       int& dir) {
    float E[6];
    if (kGather) {
        fields_one<kSmemCoef>(coef, p, E);
    } else {
#pragma unroll
        for (int q = 0; q < 6; ++q) E[q] = 0.f;
    }
    if (kDipole) add_dipole(pc, ci, p, E);
    const float ratio = sub_ratio(sp.k_sub, E);
    if (ratio < 1.f)
        boris32<1>(sp.k1, pc.a1[0], pc.a1[1], pc.a1[2], E, p);
    else
        boris_sub(pc, sp, ratio, E, p);
    return export32(g, pc, ci, p, dir);
}

// Mover + export of one particle with the policy read at run time (the
// particles that waited for a slot): the same arithmetic as the bulk push.
__device__ __forceinline__ int step32_any(const Geom& g, const Push32Const& pc, const float* __restrict__ coef,
                                          const CellInfo& ci, PState<float>& p, int& dir) {
    if (g.mover == 1) {
        if (g.flags & 4u) return step32f<false, true, true>(g, pc, pc, coef, ci, p, dir);
        return step32f<false, true, false>(g, pc, pc, coef, ci, p, dir);
    }
    return step32f<false, false, true>(g, pc, pc, coef, ci, p, dir);
}

// Pending particles (no slot last step) with the same physics; threads
// t0, t0 + stride, ... of the pending list.
__device__ __forceinline__ void push_pending32_body(const Geom& g, const Pop<float>& P, const Push32Const& pc,
                                                    uint32_t t0, uint32_t stride) {
    const uint32_t n = *P.pending_in_count;
    for (uint32_t i = t0; i < n; i += stride) {
        Mover<float> m = P.pending_in[i];
        PState<float> p = {m.x, m.y, m.z, m.u, m.v, m.w};
        const CellInfo ci = cell_info(g, pc, m.cell);
        int dir = 0;
        const int outcome = step32_any(g, pc, g.cellcoef + (size_t)m.cell * 48, ci, p, dir);
        int dest = m.cell;
        if (outcome == kMove) {
            const int3 c = cell_xyz(g, pc, m.cell);
            int n[3] = {c.x + (dir & 3) - 1, c.y + ((dir >> 2) & 3) - 1, c.z + ((dir >> 4) & 3) - 1};
            const int size[3] = {g.sx, g.sy, g.sz};
#pragma unroll
            for (int a = 0; a < 3; ++a) n[a] = n[a] < 0 ? n[a] + size[a] : (n[a] >= size[a] ? n[a] - size[a] : n[a]);
            dest = cell_id(g, n[0], n[1], n[2]);
        }
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
// coef[c * 48 + coef_index(q, m)]; monomials m = 1, x, y, z, xy, xz, yz, xyz. One
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
        float* out = coef + c * 48;
#pragma unroll
        for (int k = 0; k < 8; ++k) out[coef_index(q, k)] = m[k];
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
        float m[6][8];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            // corner k = i + 2 j + 4 l at (x + i, y + j, z + l)
            const float f000 = f[0][q], d100 = f[1][q] - f000, d010 = f[2][q] - f000, d001 = f[4][q] - f000;
            const float d110 = f[3][q] - f000, d101 = f[5][q] - f000, d011 = f[6][q] - f000, d111 = f[7][q] - f000;
            const float m1 = d100, m2 = d010, m3 = d001;
            const float m4 = d110 - d100 - d010, m5 = d101 - d100 - d001, m6 = d011 - d010 - d001;
            const float m7 = ((d111 - d110) - (d101 + d011)) + (d100 + d010 + d001);
            m[q][0] = f000 * scale; m[q][1] = m1 * scale; m[q][2] = m2 * scale; m[q][3] = m3 * scale;
            m[q][4] = m4 * scale; m[q][5] = m5 * scale; m[q][6] = m6 * scale; m[q][7] = m7 * scale;
        }
        float4* out = reinterpret_cast<float4*>(coef + c * 48);
#pragma unroll
        for (int v = 0; v < 12; ++v)
            out[v] = make_float4(m[coef_comp(4 * v)][coef_mono(4 * v)], m[coef_comp(4 * v + 1)][coef_mono(4 * v + 1)],
                                 m[coef_comp(4 * v + 2)][coef_mono(4 * v + 2)],
                                 m[coef_comp(4 * v + 3)][coef_mono(4 * v + 3)]);
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
