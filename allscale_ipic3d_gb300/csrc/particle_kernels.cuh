// Particle kernels of the GB300 path, templated on the storage type:
//   T = double : absolute FP64 positions, the reference's arithmetic order
//                (compiled with -fmad=false so no product is fused);
//   T = float  : FP32 positions relative to the cell origin in cell widths.
//
// One step of the reference's active loop (simulator.h:214-223) is
//   k_push      mover (cell.h:896-964) + export (cell.h:975-1159), in place,
//               fused with the cloud-in-cell deposit of the moved particles
//               (cell.h:787-824, scatter form) for the next step's solver;
//               leavers go to an outbox (the TransferBuffers of
//               transfer_buffer.h:48-95, compacted with warp ballots);
//   k_push_pending  the same for particles that found no slot last step;
//   k_inject    x=0 injection (not in the reference);
//   k_place     import (cell.h:1195-1310): one warp per cell fills the holes
//               left by leavers with arrivals and compacts the cell.
#pragma once

#include <type_traits>

#include "device.cuh"

namespace ipg {

// ---- r^2.5 correctly rounded (FP64) ----------------------------------------
// The reference evaluates pow(|x|^2, 2.5) with the host libm (cell.h:940),
// whose result is the correctly rounded one in all but rare cases. CUDA's pow
// is not correctly rounded, so the FP64 path evaluates a^2.5 = a^2 * sqrt(a)
// in double-double arithmetic and rounds once at the end. sqrt(a) = s + ds
// to ~2^-100 relative comes from the reciprocal square root y (error <= 1
// ulp): s0 = a y, then s = s0 + (a - s0^2) y / 2, the correctly rounded root
// (exact when a is a square), and ds = (a - s^2) y / 2, with the residuals
// exact through fma; a^2 = p + pe and p s = h + l are Dekker's exact
// products. The result is the correctly rounded one unless a^2.5 lies within
// ~2^-100 relative of a rounding boundary (exact midpoints, from squares,
// round to even). Inputs in [2^400, 2^410) are scaled by 2^-400 (exactly)
// and the result by 2^1000; from 2^410 on a^2.5 overflows. Below 2^-400 the
// result is subnormal or zero and is rounded twice.
__device__ __forceinline__ double pow25_core(double a) {
    const double y = rsqrt(a);
    double s = __dmul_rn(a, y);
    double e = __fma_rn(-s, s, a);
    s = __dadd_rn(s, __dmul_rn(__dmul_rn(e, y), 0.5));
    e = __fma_rn(-s, s, a);
    const double ds = __dmul_rn(__dmul_rn(e, y), 0.5);
    const double p = __dmul_rn(a, a);
    const double pe = __fma_rn(a, a, -p);  // a*a = p + pe exactly
    const double h = __dmul_rn(p, s);
    double l = __fma_rn(p, s, -h);         // p*s = h + l exactly
    l = __dadd_rn(l, __dadd_rn(__dmul_rn(p, ds), __dmul_rn(pe, s)));
    return __dadd_rn(h, l);
}

__device__ __forceinline__ double pow25_rn(double a) {
    if (a >= 0x1p-400 && a < 0x1p400) return pow25_core(a);
    if (a != a) return a;
    if (a < 0.0) return __longlong_as_double(0x7ff8000000000000LL);
    if (a < 0x1p-800) return 0.0;  // a^2.5 < 2^-2000 (and a == 0)
    if (a < 0x1p-400) return __dmul_rn(pow25_core(__dmul_rn(a, 0x1p400)), 0x1p-1000);
    if (a < 0x1p410) return __dmul_rn(pow25_core(__dmul_rn(a, 0x1p-400)), 0x1p1000);
    return __longlong_as_double(0x7ff0000000000000LL);  // +inf
}

// ---- the Boris rotation (Particle::updateVelocity, particle.h:31-49) -------
template <typename T>
__device__ __forceinline__ void boris(T& u, T& v, T& w, T ex, T ey, T ez, T bx, T by, T bz, T qom, T dt) {
    T k = qom * T(0.5) * dt;
    T tx = k * bx, ty = k * by, tz = k * bz;
    T t_mag2 = tx * tx;
    t_mag2 += ty * ty;
    t_mag2 += tz * tz;
    T den = T(1.0) + t_mag2;
    T sx = (T(2.0) * tx) / den, sy = (T(2.0) * ty) / den, sz = (T(2.0) * tz) / den;
    T kex = k * ex, key = k * ey, kez = k * ez;
    T mx = u + kex, my = v + key, mz = w + kez;            // v_minus
    T px = mx + (my * tz - mz * ty);                        // v_prime = v_minus + v_minus x t
    T py = my + (mz * tx - mx * tz);
    T pz = mz + (mx * ty - my * tx);
    T qx = mx + (py * sz - pz * sy);                        // v_plus = v_minus + v_prime x s
    T qy = my + (pz * sx - px * sz);
    T qz = mz + (px * sy - py * sx);
    u = qx + kex;
    v = qy + key;
    w = qz + kez;
}

// x + z for z = k * 0 = +-0 (k finite, z negative when k is): x itself,
// except -0 + +0 = +0. Integer work in place of the FP64 addition.
__device__ __forceinline__ double add_zero(double x, bool z_negative) {
    return (!z_negative && __double_as_longlong(x) == (long long)0x8000000000000000ULL) ? 0.0 : x;
}

// Particle::updateVelocity (particle.h:31-49) in FP64 for E = 0 (the dipole
// mover, the tracer): boris<double> with the k E terms (+-0 for finite k)
// applied as add_zero, bit for bit the same velocities.
__device__ __forceinline__ void boris_e0(double& u, double& v, double& w, double bx, double by, double bz,
                                         double qom, double dt) {
    const double k = qom * 0.5 * dt;
    if (!isfinite(k)) {  // k E is NaN: the general routine
        boris<double>(u, v, w, 0.0, 0.0, 0.0, bx, by, bz, qom, dt);
        return;
    }
    const bool kneg = signbit(k);
    const double tx = k * bx, ty = k * by, tz = k * bz;
    double t_mag2 = tx * tx;
    t_mag2 += ty * ty;
    t_mag2 += tz * tz;
    const double den = 1.0 + t_mag2;
    const double sx = (2.0 * tx) / den, sy = (2.0 * ty) / den, sz = (2.0 * tz) / den;
    const double mx = add_zero(u, kneg), my = add_zero(v, kneg), mz = add_zero(w, kneg);  // v_minus
    const double px = mx + (my * tz - mz * ty);  // v_prime = v_minus + v_minus x t
    const double py = my + (mz * tx - mx * tz);
    const double pz = mz + (mx * ty - my * tx);
    u = add_zero(mx + (py * sz - pz * sy), kneg);  // v_plus + k E
    v = add_zero(my + (pz * sx - px * sz), kneg);
    w = add_zero(mz + (px * sy - py * sx), kneg);
}

// Sub-cycle count of moveParticles (cell.h:947-952): min(int(dt/dt_sub)+1,
// 100) with dt_sub = pi c / (4 |qom| |B|^2). Quotients outside the int range
// (and NaN) convert to INT_MIN on the reference's x86 build, which leaves the
// particle unmoved; that outcome is returned as 0.
template <typename T>
__device__ __forceinline__ int sub_cycles(T dt, T c, T qom, T bmag) {
    T dt_sub = T(3.14159265358979323846) * c / (T(4.0) * fabs(qom) * bmag);
    T ratio = dt / dt_sub;
    if (!(ratio >= T(-2147483648.0) && ratio < T(2147483647.0))) return 0;
    int n = (int)ratio + 1;
    return n < 100 ? n : 100;
}

// The FP64 sub-cycle count and step together: dt / dt_sub is first
// estimated from its product form dt (4 |qom| |B|^2) / (pi c), with inv_pic
// = 1 / (pi c) rounded any way; below 1/2 the reference's two roundings of
// the quotient cannot reach 1, so the count is 1 and the step dt (dt / 1.0
// == dt), without a division. Otherwise sub_cycles and dt / n.
__device__ __forceinline__ int sub_cycles_dt(double dt, double c, double inv_pic, double qom, double bmag,
                                             double& dts) {
    const double est = (dt * ((4.0 * fabs(qom)) * bmag)) * inv_pic;
    // |est| < 0.5 on the bit pattern (NaN compares above): integer work in
    // place of an FP64 comparison
    if ((__double_as_longlong(est) & 0x7fffffffffffffffLL) < 0x3fe0000000000000LL) {
        dts = dt;
        return 1;
    }
    const int ns = sub_cycles<double>(dt, c, qom, bmag);
    dts = dt / double(ns);
    return ns;
}

// Outcome of one particle's mover + export step.
enum : int { kStay = 0, kMove = 1, kDrop = 2 };

template <typename T>
struct PState {
    T x, y, z, u, v, w;
};

// Trilinear field gather at fractional position r inside cell (cx,cy,cz):
// trilinearInterpolationF2P (cell.h:867-885) applied to the node E and B of
// the cell's 8 corners as in the commented mover (cell.h:905-937).
__device__ __forceinline__ void gather64(const Geom& g, int cx, int cy, int cz, double rx, double ry, double rz,
                                         double& ex, double& ey, double& ez, double& bx, double& by, double& bz) {
    ex = ey = ez = bx = by = bz = 0.0;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                double fac = (i == 0 ? (1 - rx) : rx) * (j == 0 ? (1 - ry) : ry) * (k == 0 ? (1 - rz) : rz);
                const double* n = g.field + 9 * field_index(g, cx + i + 1, cy + j + 1, cz + k + 1);
                ex = ex + __ldg(n + 0) * fac;
                ey = ey + __ldg(n + 1) * fac;
                ez = ez + __ldg(n + 2) * fac;
                bx = bx + __ldg(n + 3) * fac;
                by = by + __ldg(n + 4) * fac;
                bz = bz + __ldg(n + 5) * fac;
            }
    if (g.flags & 2u /*IPIC3D_F_GATHER_DIV_VOL*/) {
        ex = ex / g.vol; ey = ey / g.vol; ez = ez / g.vol;
        bx = bx / g.vol; by = by / g.vol; bz = bz / g.vol;
    }
}

__device__ __forceinline__ void gather32(const Geom& g, int cx, int cy, int cz, float rx, float ry, float rz, float& ex,
                                         float& ey, float& ez, float& bx, float& by, float& bz) {
    ex = ey = ez = bx = by = bz = 0.f;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                float fac = (i == 0 ? (1.f - rx) : rx) * (j == 0 ? (1.f - ry) : ry) * (k == 0 ? (1.f - rz) : rz);
                int64_t n = field_index(g, cx + i + 1, cy + j + 1, cz + k + 1);
                float4 e = __ldg(g.node32 + 2 * n), b = __ldg(g.node32 + 2 * n + 1);
                ex += e.x * fac; ey += e.y * fac; ez += e.z * fac;
                bx += b.x * fac; by += b.y * fac; bz += b.z * fac;
            }
    if (g.flags & 2u) {
        float iv = (float)(1.0 / g.vol);
        ex *= iv; ey *= iv; ez *= iv; bx *= iv; by *= iv; bz *= iv;
    }
}

// ---- mover + export for one particle ---------------------------------------
// FP64: absolute position; the expressions follow cell.h term by term.
__device__ __forceinline__ int step_particle(const Geom& g, int cx, int cy, int cz, double qom, PState<double>& p,
                                             int& dest) {
    // -- moveParticles (cell.h:896-964) --
    double ex = 0.0, ey = 0.0, ez = 0.0, bx = 0.0, by = 0.0, bz = 0.0;
    const bool field_mover = g.mover == 1;
    if (field_mover) {
        double ox = g.origin[0] + (double)cx * g.w[0], oy = g.origin[1] + (double)cy * g.w[1],
               oz = g.origin[2] + (double)cz * g.w[2];
        gather64(g, cx, cy, cz, (p.x - ox) / g.w[0], (p.y - oy) / g.w[1], (p.z - oz) / g.w[2], ex, ey, ez, bx, by, bz);
    }
    if (!field_mover || (g.flags & 4u /*IPIC3D_F_DIPOLE_IN_GATHER*/)) {
        double r2 = p.x * p.x;
        r2 += p.y * p.y;
        r2 += p.z * p.z;
        double fac1 = g.mft / pow25_rn(r2);
        double dbx = 3.0 * p.x * p.z * fac1;
        double dby = 3.0 * p.y * p.z * fac1;
        double dbz = (2.0 * (p.z * p.z) - (p.x * p.x) - (p.y * p.y)) * fac1;
        if (field_mover) {
            bx = bx + dbx; by = by + dby; bz = bz + dbz;
        } else {
            bx = dbx; by = dby; bz = dbz;
        }
    }
    double bmag = bx * bx;
    bmag += by * by;
    bmag += bz * bz;
    double dts;
    const int ns = sub_cycles_dt(g.dt, g.c, g.inv_pic, qom, bmag, dts);
    for (int s = 0; s < ns; ++s) {
        if (field_mover)
            boris<double>(p.u, p.v, p.w, ex, ey, ez, bx, by, bz, qom, dts);
        else
            boris_e0(p.u, p.v, p.w, bx, by, bz, qom, dts);
        p.x = p.x + p.u * dts;  // updatePosition (particle.h:24-26)
        p.y = p.y + p.v * dts;
        p.z = p.z + p.w * dts;
    }
    // -- exportParticles (cell.h:1093-1146) --
    const int pos[3] = {cx, cy, cz};
    const int size[3] = {g.sx, g.sy, g.sz};
    double P[3] = {p.x, p.y, p.z};
    double center[3], rel[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        center[a] = (g.origin[a] + (double)pos[a] * g.w[a]) + g.w[a] / 2.0;
        rel[a] = P[a] - center[a];
    }
    bool invert = false, drop = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (pos[a] == 0 && rel[a] < -g.half_w[a]) {
            if (g.bc_lo[a] == 0) { invert = true; P[a] = P[a] + g.half_w[a]; }
            else if (g.bc_lo[a] == 2) drop = true;
        } else if (pos[a] == size[a] - 1 && rel[a] > g.half_w[a]) {
            if (g.bc_hi[a] == 0) { invert = true; P[a] = P[a] - g.half_w[a]; }
            else if (g.bc_hi[a] == 2) drop = true;
        }
    }
    if (invert) { p.u = p.u * -1.0; p.v = p.v * -1.0; p.w = p.w * -1.0; }
    if (drop) return kDrop;
    double dx = P[0] - g.object_center[0], dy = P[1] - g.object_center[1], dz = P[2] - g.object_center[2];
    double r2 = dx * dx;
    r2 += dy * dy;
    r2 += dz * dz;
    if (r2 <= g.planet_r2) return kDrop;
    int d[3];
    bool out = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        rel[a] = P[a] - center[a];
        out |= fabs(rel[a]) > g.half_w[a];
        d[a] = rel[a] < -g.half_w[a] ? -1 : (rel[a] > g.half_w[a] ? 1 : 0);
    }
    p.x = P[0]; p.y = P[1]; p.z = P[2];
    if (!out) return kStay;
    int n[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int t = pos[a] + d[a];
        if (t < 0) {
            t += size[a];
            if (g.bc_lo[a] == 1) P[a] += (double)size[a] * g.w[a];
        } else if (t >= size[a]) {
            t -= size[a];
            if (g.bc_hi[a] == 1) P[a] -= (double)size[a] * g.w[a];
        }
        n[a] = t;
    }
    p.x = P[0]; p.y = P[1]; p.z = P[2];
    dest = cell_id(g, n[0], n[1], n[2]);
    return kMove;
}

// FP32: position relative to the cell origin in cell widths; inside <=> [0,1]
// on every axis, which is the reference's |relPos| <= halfWidth test.
__device__ __forceinline__ int step_particle(const Geom& g, int cx, int cy, int cz, float qom, PState<float>& p,
                                             int& dest) {
    const float w0 = (float)g.w[0], w1 = (float)g.w[1], w2 = (float)g.w[2];
    const float iw0 = (float)g.inv_w[0], iw1 = (float)g.inv_w[1], iw2 = (float)g.inv_w[2];
    float ex = 0.f, ey = 0.f, ez = 0.f, bx0 = 0.f, by0 = 0.f, bz0 = 0.f;
    const bool field_mover = g.mover == 1;
    const bool with_dipole = !field_mover || (g.flags & 4u);
    if (field_mover) gather32(g, cx, cy, cz, p.x, p.y, p.z, ex, ey, ez, bx0, by0, bz0);
    // cell origin relative to the dipole centre (the origin of coordinates)
    const float ox = (float)(g.origin[0] + (double)cx * g.w[0]);
    const float oy = (float)(g.origin[1] + (double)cy * g.w[1]);
    const float oz = (float)(g.origin[2] + (double)cz * g.w[2]);
    const float mft = (float)g.mft;
    const float dt = (float)g.dt, c = (float)g.c;
    // the dipole B of the reference mover is evaluated at the particle before
    // the sub-cycles (cell.h:940-945)
    float bx = bx0, by = by0, bz = bz0;
    if (with_dipole) {
        float X = ox + p.x * w0, Y = oy + p.y * w1, Z = oz + p.z * w2;
        float r2 = X * X + Y * Y + Z * Z;
        float fac1 = mft / (r2 * r2 * sqrtf(r2));
        bx += 3.f * X * Z * fac1;
        by += 3.f * Y * Z * fac1;
        bz += (2.f * Z * Z - X * X - Y * Y) * fac1;
    }
    int ns = sub_cycles<float>(dt, c, qom, bx * bx + by * by + bz * bz);
    float dts = dt / (float)ns;
    float sx = dts * iw0, sy = dts * iw1, sz = dts * iw2;
    for (int s = 0; s < ns; ++s) {
        boris<float>(p.u, p.v, p.w, ex, ey, ez, bx, by, bz, qom, dts);
        p.x += p.u * sx;
        p.y += p.v * sy;
        p.z += p.w * sz;
    }
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
        float dx = (float)(g.origin[0] + (double)cx * g.w[0] - g.object_center[0]) + R[0] * w0;
        float dy = (float)(g.origin[1] + (double)cy * g.w[1] - g.object_center[1]) + R[1] * w1;
        float dz = (float)(g.origin[2] + (double)cz * g.w[2] - g.object_center[2]) + R[2] * w2;
        if (dx * dx + dy * dy + dz * dz <= (float)g.planet_r2) return kDrop;  // cell.h:1123-1128
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

// ---- deposit -----------------------------------------------------------------
// Cloud-in-cell weights of projectToDensityField (cell.h:810-816): a particle
// at fractional position r in cell c adds q v fac and q fac to node c+(i,j,k)
// with fac = prod (i ? r : 1-r). Index l = corner*4 + comp, comp 3 = rho.
template <typename T>
__device__ __forceinline__ void frac_in_cell(const Geom& g, int cx, int cy, int cz, const PState<T>& p, T& rx, T& ry,
                                             T& rz) {
    if constexpr (std::is_same<T, double>::value) {
        rx = (p.x - (g.origin[0] + (double)cx * g.w[0])) / g.w[0];
        ry = (p.y - (g.origin[1] + (double)cy * g.w[1])) / g.w[1];
        rz = (p.z - (g.origin[2] + (double)cz * g.w[2])) / g.w[2];
    } else {
        rx = p.x; ry = p.y; rz = p.z;
    }
}

template <typename T>
__device__ __forceinline__ T cic_weight(int corner, T rx, T ry, T rz) {
    int i = corner >> 2, j = (corner >> 1) & 1, k = corner & 1;
    return (i == 0 ? (1 - rx) : rx) * (j == 0 ? (1 - ry) : ry) * (k == 0 ? (1 - rz) : rz);
}

__device__ __forceinline__ void node_atomic_add(const Geom& g, int cx, int cy, int cz, int l, double val) {
    if (val == 0.0) return;
    int corner = l >> 2, comp = l & 3;
    int64_t n = node_index(g, cx + (corner >> 2), cy + ((corner >> 1) & 1), cz + (corner & 1));
    if (comp < 3)
        atomicAdd(g.J + 3 * n + comp, val);
    else
        atomicAdd(g.rho + n, val);
}

// Direct deposit of one particle (rare paths: migrants, pending, injected).
template <typename T>
__device__ __forceinline__ void deposit_one(const Geom& g, int c, const PState<T>& p, double q) {
    int cx, cy, cz;
    cell_coords(g, c, cx, cy, cz);
    T rx, ry, rz;
    frac_in_cell(g, cx, cy, cz, p, rx, ry, rz);
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
        double fac = (double)cic_weight<T>(corner, rx, ry, rz);
        node_atomic_add(g, cx, cy, cz, corner * 4 + 0, (q * (double)p.u) * fac);
        node_atomic_add(g, cx, cy, cz, corner * 4 + 1, (q * (double)p.v) * fac);
        node_atomic_add(g, cx, cy, cz, corner * 4 + 2, (q * (double)p.w) * fac);
        node_atomic_add(g, cx, cy, cz, corner * 4 + 3, q * fac);
    }
}

// Deposit of the warp's leavers into their destination cells, one leaver at
// a time: lane l adds value l (corner l & 7, component l >> 3) of the leaver's
// cloud-in-cell contribution, the same values deposit_one adds one by one, so
// a leaver costs one 32-lane atomic instead of 32 serial ones. Every lane of
// the warp must call it.
template <typename T>
__device__ __forceinline__ void warp_deposit_leavers(const Geom& g, bool leave, int dest, const PState<T>& p,
                                                     double q) {
    unsigned m = __ballot_sync(0xffffffffu, leave);
    const int lane = threadIdx.x & 31, corner = lane & 7, comp = lane >> 3;
    while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const int c = __shfl_sync(0xffffffffu, dest, src);
        PState<T> s;
        s.x = __shfl_sync(0xffffffffu, p.x, src);
        s.y = __shfl_sync(0xffffffffu, p.y, src);
        s.z = __shfl_sync(0xffffffffu, p.z, src);
        s.u = __shfl_sync(0xffffffffu, p.u, src);
        s.v = __shfl_sync(0xffffffffu, p.v, src);
        s.w = __shfl_sync(0xffffffffu, p.w, src);
        int cx, cy, cz;
        cell_coords(g, c, cx, cy, cz);
        T rx, ry, rz;
        frac_in_cell(g, cx, cy, cz, s, rx, ry, rz);
        const double fac = (double)cic_weight<T>(corner, rx, ry, rz);
        const double Q = comp == 0 ? (double)s.u : (comp == 1 ? (double)s.v : (double)s.w);
        node_atomic_add(g, cx, cy, cz, corner * 4 + comp, comp < 3 ? (q * Q) * fac : q * fac);
    }
}

// Warp transpose-reduction: every lane holds 32 values; afterwards lane l
// holds the warp-wide sum of value l (31 exchanges in total).
template <typename T>
__device__ __forceinline__ T warp_transpose_sum(T (&v)[32]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < off; ++i) {
            T send = upper ? v[i] : v[i + off];
            T keep = upper ? v[i + off] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    return v[0];
}

// ---- slot / outbox helpers -------------------------------------------------
template <typename T>
__device__ __forceinline__ void write_slot(const Pop<T>& P, int64_t slot, const Mover<T>& m) {
    P.x[slot] = m.x; P.y[slot] = m.y; P.z[slot] = m.z;
    P.u[slot] = m.u; P.v[slot] = m.v; P.w[slot] = m.w;
    if (P.id) P.id[slot] = m.id;
}

template <typename T>
__device__ __forceinline__ void move_slot(const Pop<T>& P, int64_t from, int64_t to) {
    P.x[to] = P.x[from]; P.y[to] = P.y[from]; P.z[to] = P.z[from];
    P.u[to] = P.u[from]; P.v[to] = P.v[from]; P.w[to] = P.w[from];
    if (P.id) P.id[to] = P.id[from];
}

// Files an outbox entry as an arrival of its destination cell: slot k of the
// cell's arrival list, or the pending list when the cell's slots are short.
template <typename T>
__device__ __forceinline__ void register_arrival(const Pop<T>& P, uint32_t o, const Mover<T>& m) {
    int k = atomicAdd(P.arr_cnt + m.cell, 1);
    mark_dirty(P, m.cell);
    int64_t s = P.start[m.cell];
    if (k < (int)(P.start[m.cell + 1] - s)) {
        P.arr_list[s + k] = (int32_t)o;
    } else {
        uint32_t pi = atomicAdd(&P.ctr->pending_out, 1u);
        if (pi < P.pending_cap) P.pending_out[pi] = m;
        else atomicAdd(&P.ctr->lost, 1u);
    }
}

// ---- the fused push kernel ----------------------------------------------------
// CTA b covers slots [b*kSlotsPerCta, (b+1)*kSlotsPerCta) of one population;
// thread t the 4 slots from 4t (one cell, start[] is 4-aligned). mode 0 =
// step (mover + export + deposit), mode 1 = deposit only (the projector over
// the stored particles, cell.h:787-824).
// push_body is the work of CTA `blk`; the single-universe kernel passes its
// block index, the batched kernel the block index within its job.
template <typename T>
__device__ __forceinline__ void push_body(const Geom& g, const Pop<T>& P, int64_t blk, int mode) {
    __shared__ int64_t s_start[kMaxCellsPerCta + 1];
    __shared__ int s_count[kMaxCellsPerCta];
    const int64_t base = blk * kSlotsPerCta;
    // the cells this CTA's slots belong to (fixed between re-layouts)
    const int2 cc = __ldg(P.cta_cells + blk);
    const int c0 = cc.x, nc = cc.y;
    for (int i = threadIdx.x; i <= nc; i += blockDim.x) s_start[i] = P.start[c0 + i];
    for (int i = threadIdx.x; i < nc; i += blockDim.x) s_count[i] = P.count[c0 + i];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int64_t s0 = base + (int64_t)threadIdx.x * kVec;
    int lc = 0;
    {
        int lo = 0, hi = nc - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (s_start[mid] <= s0) lo = mid; else hi = mid - 1;
        }
        lc = lo;
    }
    const int cell = c0 + lc;
    int nv = 0;
    if (s0 < P.capacity) {
        int64_t e = s_start[lc] + s_count[lc] - s0;
        nv = e <= 0 ? 0 : (e >= kVec ? kVec : (int)e);
    }
    int cx, cy, cz;
    cell_coords(g, cell, cx, cy, cz);
    const T qom = (T)P.qom;
    const double q = P.q;

    PState<T> ps[kVec];
    if (nv > 0) {
        if constexpr (std::is_same<T, float>::value) {
            float4 X = *reinterpret_cast<const float4*>(P.x + s0), Y = *reinterpret_cast<const float4*>(P.y + s0),
                   Z = *reinterpret_cast<const float4*>(P.z + s0), U = *reinterpret_cast<const float4*>(P.u + s0),
                   V = *reinterpret_cast<const float4*>(P.v + s0), W = *reinterpret_cast<const float4*>(P.w + s0);
            ps[0] = {X.x, Y.x, Z.x, U.x, V.x, W.x};
            ps[1] = {X.y, Y.y, Z.y, U.y, V.y, W.y};
            ps[2] = {X.z, Y.z, Z.z, U.z, V.z, W.z};
            ps[3] = {X.w, Y.w, Z.w, U.w, V.w, W.w};
        } else {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                double2 X = *reinterpret_cast<const double2*>(P.x + s0 + 2 * h);
                double2 Y = *reinterpret_cast<const double2*>(P.y + s0 + 2 * h);
                double2 Z = *reinterpret_cast<const double2*>(P.z + s0 + 2 * h);
                double2 U = *reinterpret_cast<const double2*>(P.u + s0 + 2 * h);
                double2 V = *reinterpret_cast<const double2*>(P.v + s0 + 2 * h);
                double2 W = *reinterpret_cast<const double2*>(P.w + s0 + 2 * h);
                ps[2 * h] = {X.x, Y.x, Z.x, U.x, V.x, W.x};
                ps[2 * h + 1] = {X.y, Y.y, Z.y, U.y, V.y, W.y};
            }
        }
    }

    const bool deposit = g.deposit != 0;
    // per-thread node sums of its (up to 4) staying particles: FP32 for the
    // FP32 path, FP64 otherwise; the node accumulation itself is FP64
    T acc[32];
#pragma unroll
    for (int l = 0; l < 32; ++l) acc[l] = T(0);
    bool has_acc = false;
    int outc[kVec], dst[kVec];

#pragma unroll
    for (int j = 0; j < kVec; ++j) {
        outc[j] = -1;
        dst[j] = cell;
        if (j >= nv) continue;
        int outcome = kStay, dest = cell;
        if (mode == 0) outcome = step_particle(g, cx, cy, cz, qom, ps[j], dest);
        outc[j] = outcome;
        dst[j] = dest;
        if (outcome == kStay && deposit) {
            T rx, ry, rz;
            frac_in_cell(g, cx, cy, cz, ps[j], rx, ry, rz);
#pragma unroll
            for (int corner = 0; corner < 8; ++corner) {
                T fac = cic_weight<T>(corner, rx, ry, rz);
                if constexpr (std::is_same<T, double>::value) {
                    acc[corner * 4 + 0] += (q * ps[j].u) * fac;
                    acc[corner * 4 + 1] += (q * ps[j].v) * fac;
                    acc[corner * 4 + 2] += (q * ps[j].w) * fac;
                    acc[corner * 4 + 3] += q * fac;
                } else {
                    const float qf = (float)q;
                    acc[corner * 4 + 0] += qf * ps[j].u * fac;
                    acc[corner * 4 + 1] += qf * ps[j].v * fac;
                    acc[corner * 4 + 2] += qf * ps[j].w * fac;
                    acc[corner * 4 + 3] += qf * fac;
                }
            }
            has_acc = true;
        }
    }

    // leavers -> outbox (one warp-aggregated append per vector lane), arrival
    // lists of the destination cells, deposit relative to the destination
    uint32_t nmig = 0, nrem = 0;
#pragma unroll
    for (int j = 0; j < kVec; ++j) {
        const bool leave = outc[j] == kMove;
        const uint32_t o = warp_append(&P.ctr->outbox, leave);
        if (leave) {
            Mover<T> m;
            m.cell = dst[j];
            m.id = P.id ? P.id[s0 + j] : 0u;
            m.x = ps[j].x; m.y = ps[j].y; m.z = ps[j].z;
            m.u = ps[j].u; m.v = ps[j].v; m.w = ps[j].w;
            if (o < P.outbox_cap) {  // sized for one entry per slot: never full
                P.outbox[o] = m;
                register_arrival(P, o, m);
            } else {
                atomicAdd(&P.ctr->lost, 1u);
            }
            ++nmig;
        }
        if (outc[j] == kMove || outc[j] == kDrop) {
            file_hole(P, cell, s_start[lc], s0 + j);
            if (outc[j] == kDrop) ++nrem;
        }
    }
    if (deposit) {
#pragma unroll
        for (int j = 0; j < kVec; ++j) warp_deposit_leavers<T>(g, outc[j] == kMove, dst[j], ps[j], q);
    }
    nmig = __reduce_add_sync(0xffffffffu, nmig);
    nrem = __reduce_add_sync(0xffffffffu, nrem);
    if (lane == 0) {
        if (nmig) atomicAdd(&P.ctr->migrated, nmig);
        if (nrem) atomicAdd(&P.ctr->removed, nrem);
    }

    // stayers: write the updated state back in place (vector stores)
    if (mode == 0 && nv > 0) {
        if constexpr (std::is_same<T, float>::value) {
            *reinterpret_cast<float4*>(P.x + s0) = make_float4(ps[0].x, ps[1].x, ps[2].x, ps[3].x);
            *reinterpret_cast<float4*>(P.y + s0) = make_float4(ps[0].y, ps[1].y, ps[2].y, ps[3].y);
            *reinterpret_cast<float4*>(P.z + s0) = make_float4(ps[0].z, ps[1].z, ps[2].z, ps[3].z);
            *reinterpret_cast<float4*>(P.u + s0) = make_float4(ps[0].u, ps[1].u, ps[2].u, ps[3].u);
            *reinterpret_cast<float4*>(P.v + s0) = make_float4(ps[0].v, ps[1].v, ps[2].v, ps[3].v);
            *reinterpret_cast<float4*>(P.w + s0) = make_float4(ps[0].w, ps[1].w, ps[2].w, ps[3].w);
        } else {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                *reinterpret_cast<double2*>(P.x + s0 + 2 * h) = make_double2(ps[2 * h].x, ps[2 * h + 1].x);
                *reinterpret_cast<double2*>(P.y + s0 + 2 * h) = make_double2(ps[2 * h].y, ps[2 * h + 1].y);
                *reinterpret_cast<double2*>(P.z + s0 + 2 * h) = make_double2(ps[2 * h].z, ps[2 * h + 1].z);
                *reinterpret_cast<double2*>(P.u + s0 + 2 * h) = make_double2(ps[2 * h].u, ps[2 * h + 1].u);
                *reinterpret_cast<double2*>(P.v + s0 + 2 * h) = make_double2(ps[2 * h].v, ps[2 * h + 1].v);
                *reinterpret_cast<double2*>(P.w + s0 + 2 * h) = make_double2(ps[2 * h].w, ps[2 * h + 1].w);
            }
        }
    }

    // stayers' deposit: group lanes by cell, transpose-reduce the 32 node
    // components, one FP64 atomic per lane and group
    if (deposit) {
        unsigned todo = __ballot_sync(0xffffffffu, has_acc);
        while (todo) {
            const int leader = __ffs(todo) - 1;
            const int gcell = __shfl_sync(0xffffffffu, cell, leader);
            const bool mine = has_acc && cell == gcell;
            const unsigned grp = __ballot_sync(0xffffffffu, mine);
            T v[32];
#pragma unroll
            for (int l = 0; l < 32; ++l) v[l] = mine ? acc[l] : T(0);
            const double tot = (double)warp_transpose_sum<T>(v);
            int gx, gy, gz;
            cell_coords(g, gcell, gx, gy, gz);
            node_atomic_add(g, gx, gy, gz, lane, tot);
            todo &= ~grp;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kPushThreads) k_push(Geom g, Pop<T> P, int mode) {
    push_body<T>(g, P, blockIdx.x, mode);
}

// ---- particles that waited for a slot --------------------------------------
// Entries t0, t0 + stride, ... of the pending list.
template <typename T>
__device__ __forceinline__ void push_pending_body(const Geom& g, const Pop<T>& P, uint32_t t0, uint32_t stride) {
    const uint32_t n = *P.pending_in_count;
    const double q = P.q;
    for (uint32_t i = t0; i < n; i += stride) {
        Mover<T> m = P.pending_in[i];
        PState<T> p = {m.x, m.y, m.z, m.u, m.v, m.w};
        int cx, cy, cz;
        cell_coords(g, m.cell, cx, cy, cz);
        int dest = m.cell;
        int outcome = step_particle(g, cx, cy, cz, (T)P.qom, p, dest);
        if (outcome == kDrop) {
            atomicAdd(&P.ctr->removed, 1u);
            continue;
        }
        if (outcome == kMove) atomicAdd(&P.ctr->migrated, 1u);
        Mover<T> o = {dest, m.id, p.x, p.y, p.z, p.u, p.v, p.w};
        uint32_t k = atomicAdd(&P.ctr->outbox, 1u);
        if (k < P.outbox_cap) {
            P.outbox[k] = o;
            register_arrival(P, k, o);
        } else {
            atomicAdd(&P.ctr->lost, 1u);
        }
        if (g.deposit) deposit_one<T>(g, dest, p, q);
    }
}

template <typename T>
__global__ void k_push_pending(Geom g, const __grid_constant__ PopSet<T> S) {
    push_pending_body<T>(g, S.p[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// ---- injection at the x = 0 face (not in the reference) ---------------------
// MurmurHash3's 64-bit finaliser (fmix64, A. Appleby, public domain) drives a
// counter-based generator keyed by (seed, step, cell, draw); the CPU oracle
// uses the same keys. Per face cell: floor(rate + u) particles, positions
// uniform in the cell, velocities drift + vth * Box-Muller normals.
__device__ __forceinline__ uint64_t fmix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}
__device__ __forceinline__ uint64_t inj_key(uint64_t seed, uint64_t step, uint64_t cell, uint64_t draw) {
    return fmix64(fmix64(seed ^ (step * 0x9E3779B97F4A7C15ULL)) ^ (cell * 0xD1B54A32D192ED03ULL + draw));
}
__device__ __forceinline__ double u01(uint64_t key) { return (double)(key >> 11) * (1.0 / 9007199254740992.0); }

struct InjectParams {
    double per_cell, drift[3], vth[3];
    uint64_t seed;
    const uint64_t* step;  // device step counter
};

template <typename T>
__global__ void k_inject(Geom g, Pop<T> P, InjectParams ip) {
    // one thread per face cell; the warp takes its cells' particles one round
    // at a time (warp-aggregated outbox appends, cooperative deposit)
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int j = 0, k = 0, c = 0, n = 0;
    const uint64_t step = *ip.step;
    if (f < g.sy * g.sz) {
        j = f / g.sz;
        k = f - j * g.sz;
        c = cell_id(g, 0, j, k);
        n = (int)floor(ip.per_cell + u01(inj_key(ip.seed, step, (uint64_t)c, 0)));
    }
    const int nmax = __reduce_max_sync(0xffffffffu, n);
    for (int m = 0; m < nmax; ++m) {
        const bool has = m < n;
        PState<T> p = {};
        Mover<T> mv = {};
        if (has) {
            const uint64_t d = 1 + 8 * (uint64_t)m;
            double u[7];
#pragma unroll
            for (int t = 0; t < 7; ++t) u[t] = u01(inj_key(ip.seed, step, (uint64_t)c, d + t));
            if constexpr (std::is_same<T, double>::value) {
                const double g1 = sqrt(-2.0 * log(1.0 - u[3])), th1 = 2.0 * 3.14159265358979323846 * u[4];
                const double g2 = sqrt(-2.0 * log(1.0 - u[5])), th2 = 2.0 * 3.14159265358979323846 * u[6];
                p.x = g.origin[0] + u[0] * g.w[0];
                p.y = g.origin[1] + ((double)j + u[1]) * g.w[1];
                p.z = g.origin[2] + ((double)k + u[2]) * g.w[2];
                p.u = ip.drift[0] + ip.vth[0] * (g1 * cos(th1));
                p.v = ip.drift[1] + ip.vth[1] * (g1 * sin(th1));
                p.w = ip.drift[2] + ip.vth[2] * (g2 * cos(th2));
            } else {
                // the same draws, Box-Muller in FP32 (GB300's FP64
                // transcendentals would dominate this kernel)
                const float g1 = sqrtf(-2.f * logf(1.f - (float)u[3])), g2 = sqrtf(-2.f * logf(1.f - (float)u[5]));
                float s1, c1, s2, c2;
                sincospif(2.f * (float)u[4], &s1, &c1);
                sincospif(2.f * (float)u[6], &s2, &c2);
                p.x = (float)u[0]; p.y = (float)u[1]; p.z = (float)u[2];
                p.u = (float)ip.drift[0] + (float)ip.vth[0] * (g1 * c1);
                p.v = (float)ip.drift[1] + (float)ip.vth[1] * (g1 * s1);
                p.w = (float)ip.drift[2] + (float)ip.vth[2] * (g2 * c2);
            }
            mv = {c, 0xffffffffu, p.x, p.y, p.z, p.u, p.v, p.w};
        }
        const uint32_t o = warp_append(&P.ctr->outbox, has);
        if (has) {
            if (o < P.outbox_cap) {
                P.outbox[o] = mv;
                register_arrival(P, o, mv);
            } else {
                atomicAdd(&P.ctr->lost, 1u);
            }
        }
        if (g.deposit) warp_deposit_leavers<T>(g, has, c, p, P.q);
    }
    const int tot = __reduce_add_sync(0xffffffffu, n);
    if (lane == 0 && tot) atomicAdd(&P.ctr->injected, (uint32_t)tot);
}

// ---- import: one warp per cell ------------------------------------------------
// Fills the cell's holes (sorted ascending) with its arrivals; surplus
// arrivals append after the last particle, surplus holes are closed by moving
// the cell's last particles into them. Arrivals beyond the cell's slots go to
// the pending list and are pushed and placed again next step.
// place_body is the work of a group of kG lanes (kG = 8: four cells per warp
// at once; the kernel waits on memory, so four cells' loads in flight per
// warp) on cell c (uniform within the group).
constexpr int kPlaceLanes = 8;

template <typename T, int kG = kPlaceLanes>
__device__ __forceinline__ void place_body(const Geom& g, const Pop<T>& P, int32_t* sort_tmp, int c) {
    static_assert(kG == 8 || kG == 16 || kG == 32, "group of 8, 16 or 32 lanes");
    const int wl = threadIdx.x & 31, lane = wl & (kG - 1);
    const unsigned gmask = (kG == 32 ? 0xffffffffu : ((1u << kG) - 1u)) << (wl & ~(kG - 1));
    if (c >= g.ncells) return;
    const int nh = P.hole_cnt[c], na_all = P.arr_cnt[c];
    if (nh == 0 && na_all == 0) {  // nothing to place: only the flag to clear
        if (lane == 0) P.dirty_flag[c] = 0;
        return;
    }
    const int64_t s0 = P.start[c];
    const int cap = (int)(P.start[c + 1] - s0);
    const int cnt = P.count[c];
    const int na = na_all < cap ? na_all : cap;
    const int free_slots = cap - (cnt - nh);
    const int np = na < free_slots ? na : free_slots;
    for (int i = np + lane; i < na; i += kG) {
        const Mover<T> m = P.outbox[P.arr_list[s0 + i]];
        uint32_t pi = atomicAdd(&P.ctr->pending_out, 1u);
        if (pi < P.pending_cap) P.pending_out[pi] = m;
        else atomicAdd(&P.ctr->lost, 1u);
    }
    // holes in ascending order (rank sort; hole counts are small; one hole
    // is sorted already)
    if (nh > 1) {
        for (int i = lane; i < nh; i += kG) {
            const int32_t h = P.hole_list[s0 + i];
            int r = 0;
            for (int j = 0; j < nh; ++j) r += P.hole_list[s0 + j] < h;
            sort_tmp[s0 + r] = h;
        }
        __syncwarp(gmask);
    }
    const int32_t* H = (nh > 1 ? sort_tmp : P.hole_list) + s0;
    const int m = nh < np ? nh : np;
    for (int i = lane; i < m; i += kG) write_slot(P, H[i], P.outbox[P.arr_list[s0 + i]]);
    for (int i = nh + lane; i < np; i += kG) write_slot(P, s0 + cnt + (i - nh), P.outbox[P.arr_list[s0 + i]]);
    const int newcount = cnt - nh + np;
    if (nh > np) {
        const int64_t lim = s0 + newcount, end = s0 + cnt;
        // remaining holes H[np, nh): the first L are below lim
        int lo = np, hi = nh;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (H[mid] < lim) lo = mid + 1; else hi = mid;
        }
        const int L0 = lo;  // H[np, L0) < lim <= H[L0, nh)
        int filled = 0;
        for (int64_t b = lim; b < end; b += kG) {
            const int64_t t = b + lane;
            bool valid = false;
            if (t < end) {
                int a = L0, z = nh;  // is t one of the holes H[L0, nh)?
                while (a < z) {
                    int mid = (a + z) >> 1;
                    if (H[mid] < t) a = mid + 1; else z = mid;
                }
                valid = !(a < nh && H[a] == t);
            }
            const unsigned bal = __ballot_sync(gmask, valid);  // bits of this group's lanes only
            const int idx = filled + __popc(bal & ((1u << wl) - 1u));
            if (valid) move_slot(P, t, H[np + idx]);
            filled += __popc(bal);
        }
    }
    if (lane == 0) {
        P.count[c] = newcount;
        P.hole_cnt[c] = 0;
        P.arr_cnt[c] = 0;
        P.dirty_flag[c] = 0;
    }
}

// Lists the cells flagged this step (holes or arrivals) of cells [c0, c1) of
// population P on its dirty list (order: warp by warp, ascending within a
// warp; the placement does not depend on the order). 32 x n threads from
// thread t0 with stride `stride`.
template <typename T>
__device__ __forceinline__ void dirty_compact_body(const Pop<T>& P, int c0, int c1, int64_t t0, int64_t stride) {
    const int lane = threadIdx.x & 31;
    for (int64_t base = t0 - lane; base + c0 < c1; base += stride) {
        const int c = (int)(c0 + base + lane);
        const bool d = c < c1 && P.dirty_flag[c] != 0;
        const unsigned b = __ballot_sync(0xffffffffu, d);
        if (!b) continue;
        uint32_t o = 0;
        if (lane == 0) o = atomicAdd(&P.ctr->dirty, (uint32_t)__popc(b));
        o = __shfl_sync(0xffffffffu, o, 0) + __popc(b & ((1u << lane) - 1u));
        if (d) P.dirty_list[o] = c;
    }
}

template <typename T>
__global__ void k_dirty_compact(int ncells, const __grid_constant__ PopSet<T> S) {
    dirty_compact_body<T>(S.p[blockIdx.y], 0, ncells, blockIdx.x * (int64_t)blockDim.x + threadIdx.x,
                          (int64_t)gridDim.x * blockDim.x);
}

// The cells of the step's dirty lists (the only ones with holes or
// arrivals), one group of kPlaceLanes lanes per cell, groups striding over
// the list of population blockIdx.y.
template <typename T>
__global__ void k_place(Geom g, const __grid_constant__ PopSet<T> S) {
    const Pop<T>& P = S.p[blockIdx.y];
    int32_t* sort_tmp = S.sort_tmp[blockIdx.y];
    const uint32_t n = P.ctr->dirty;
    const uint32_t g0 = (blockIdx.x * blockDim.x + threadIdx.x) / kPlaceLanes,
                   ng = (gridDim.x * blockDim.x) / kPlaceLanes;
    for (uint32_t i = g0; i < n; i += ng) place_body<T>(g, P, sort_tmp, P.dirty_list[i]);
}

// Moves this step's pending list to the next step's input (thread t0 = 0
// also sets the count).
template <typename T>
__device__ __forceinline__ void pending_rotate_body(const Pop<T>& P, uint32_t* pending_in_count, uint32_t t0,
                                                    uint32_t stride) {
    uint32_t n = P.ctr->pending_out;
    if (n > P.pending_cap) n = P.pending_cap;
    for (uint32_t i = t0; i < n; i += stride) P.pending_in[i] = P.pending_out[i];
    if (t0 == 0) *pending_in_count = n;
}

// Population blockIdx.y; thread 0 of population 0 also advances the device
// step counter (`step`, may be null), which keys the injection generator.
template <typename T>
__global__ void k_pending_rotate(const __grid_constant__ PopSet<T> S, uint64_t* step) {
    pending_rotate_body<T>(S.p[blockIdx.y], S.pend_count[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x,
                           gridDim.x * blockDim.x);
    if (step && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *step += 1;
}

// ---- re-layout (cells ran out of slack) ---------------------------------------
// Pending particles per cell.
template <typename T>
__global__ void k_pending_count(const Mover<T>* pend, const uint32_t* n_pend, int32_t* per_cell) {
    const uint32_t n = *n_pend;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(per_cell + pend[i].cell, 1);
}

// One warp per cell: the cell's particles move to the new slot range.
template <typename T>
__global__ void k_relayout_copy(Pop<T> from, Pop<T> to, int ncells) {
    const int c = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= ncells) return;
    const int64_t a = from.start[c], b = to.start[c];
    const int n = from.count[c];
    for (int i = lane; i < n; i += 32) {
        to.x[b + i] = from.x[a + i]; to.y[b + i] = from.y[a + i]; to.z[b + i] = from.z[a + i];
        to.u[b + i] = from.u[a + i]; to.v[b + i] = from.v[a + i]; to.w[b + i] = from.w[a + i];
        if (to.id) to.id[b + i] = from.id[a + i];
    }
    if (lane == 0) to.count[c] = n;
}

// Pending particles go after the copied ones (the new capacities hold them).
template <typename T>
__global__ void k_pending_place(const Mover<T>* pend, const uint32_t* n_pend, Pop<T> to) {
    const uint32_t n = *n_pend;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Mover<T> m = pend[i];
        const int k = atomicAdd(to.count + m.cell, 1);
        write_slot(to, to.start[m.cell] + k, m);
    }
}

}  // namespace ipg
