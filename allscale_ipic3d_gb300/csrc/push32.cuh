// The FP32 push kernel: mover + export + deposit for particles stored as
// FP32 positions relative to their cell origin (in cell widths).
//
// Same step as k_push<T> (particle_kernels.cuh), arranged for instruction
// count:
//   * fields: per-cell trilinear polynomial f = c0 + c1 x + c2 y + c3 z +
//     c4 xy + c5 xz + c6 yz + c7 xyz of every E and B component (the
//     expansion of trilinearInterpolationF2P, cell.h:867-885, with node
//     values from the cell's 8 corners as in cell.h:905-937), precomputed by
//     k_cell_coef after every field change: 7 FMAs per component;
//   * dipole: |r|^-5 from one rsqrt;
//   * sub-cycles (cell.h:947-952): dt/dt_sub = K |B|^2 with K per species;
//   * deposit (cell.h:810-816 in scatter form): per thread the monomial
//     moments sum_p Q m(r_p), Q in {u, v, w, 1}, m in {1, x, y, z, xy, xz,
//     yz, xyz}; one butterfly per axis turns them into the 8 corner weights
//     (1-t, t); each warp sums them per cell in shared memory and issues
//     one FP64 atomic per cell, corner and component.
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

// The body of the FP32 push for CTA `blk` of population P (shared by the
// single-universe kernel and the batched one, which loads g / P / pc from
// its job table).
__device__ __forceinline__ void push32_body(const Geom& g, const Pop<float>& P, const Push32Const& pc, int64_t blk,
                                            int mode) {
    __shared__ int64_t s_start[kMaxCellsPerCta + 1];
    __shared__ int s_count[kMaxCellsPerCta];
    // deposit staging, one tile per warp: value l of lane t at [l * 33 + t]
    // (the odd stride puts a lane's 32 values, and a value's 32 lanes, in 32
    // different banks)
    __shared__ float s_acc[kPushThreads / 32][32 * 33];
    const int64_t base = blk * kSlotsPerCta;
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
            const int mid = (lo + hi + 1) >> 1;
            if (s_start[mid] <= s0) lo = mid; else hi = mid - 1;
        }
        lc = lo;
    }
    const int cell = c0 + lc;
    int nv = 0;
    if (s0 < P.capacity) {
        const int64_t e = s_start[lc] + s_count[lc] - s0;
        nv = e <= 0 ? 0 : (e >= kVec ? kVec : (int)e);
    }
    int cx, cy, cz;
    if (g.ncells < (1 << 24) && g.sy < 4096 && g.sz < 4096) {
        const int t = fast_div(cell, g.sz, pc.inv_sz);
        cz = cell - t * g.sz;
        cx = fast_div(t, g.sy, pc.inv_sy);
        cy = t - cx * g.sy;
    } else {
        cell_coords(g, cell, cx, cy, cz);
    }
    // cell origin relative to the dipole centre (the coordinate origin)
    const float ox = fmaf((float)cx, pc.w[0], pc.origin[0]);
    const float oy = fmaf((float)cy, pc.w[1], pc.origin[1]);
    const float oz = fmaf((float)cz, pc.w[2], pc.origin[2]);
    const float* coef = g.cellcoef + (size_t)cell * 48;

    PState<float> ps[kVec];
    if (nv > 0) {
        const float4 X = *reinterpret_cast<const float4*>(P.x + s0), Y = *reinterpret_cast<const float4*>(P.y + s0),
                     Z = *reinterpret_cast<const float4*>(P.z + s0), U = *reinterpret_cast<const float4*>(P.u + s0),
                     V = *reinterpret_cast<const float4*>(P.v + s0), W = *reinterpret_cast<const float4*>(P.w + s0);
        ps[0] = {X.x, Y.x, Z.x, U.x, V.x, W.x};
        ps[1] = {X.y, Y.y, Z.y, U.y, V.y, W.y};
        ps[2] = {X.z, Y.z, Z.z, U.z, V.z, W.z};
        ps[3] = {X.w, Y.w, Z.w, U.w, V.w, W.w};
    }

    const bool deposit = g.deposit != 0;
    // monomial moments: acc[q * 8 + m], q in {u, v, w, 1}, m in {1, x, y, z, xy, xz, yz, xyz}
    float acc[32];
#pragma unroll
    for (int l = 0; l < 32; ++l) acc[l] = 0.f;
    bool has_acc = false;
    int outc[kVec], dst[kVec];
#pragma unroll
    for (int j = 0; j < kVec; ++j) {
        outc[j] = -1;
        dst[j] = cell;
    }
    // one particle per iteration, not unrolled: the physics is emitted once;
    // the four register slots rotate so every index stays static
#pragma unroll 1
    for (int j = 0; j < kVec; ++j) {
        PState<float> p = ps[0];
        int outcome = -1, dest = cell;
        if (j < nv) {
            outcome = mode == 0 ? step32(g, pc, coef, cx, cy, cz, ox, oy, oz, p, dest) : kStay;
            if (outcome == kStay && deposit) {
                const float x = p.x, y = p.y, z = p.z;
                const float xy = x * y, xz = x * z, yz = y * z, xyz = xy * z;
                const float Q[4] = {p.u, p.v, p.w, 1.f};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    acc[q * 8 + 0] += Q[q];
                    acc[q * 8 + 1] = fmaf(Q[q], x, acc[q * 8 + 1]);
                    acc[q * 8 + 2] = fmaf(Q[q], y, acc[q * 8 + 2]);
                    acc[q * 8 + 3] = fmaf(Q[q], z, acc[q * 8 + 3]);
                    acc[q * 8 + 4] = fmaf(Q[q], xy, acc[q * 8 + 4]);
                    acc[q * 8 + 5] = fmaf(Q[q], xz, acc[q * 8 + 5]);
                    acc[q * 8 + 6] = fmaf(Q[q], yz, acc[q * 8 + 6]);
                    acc[q * 8 + 7] = fmaf(Q[q], xyz, acc[q * 8 + 7]);
                }
                has_acc = true;
            }
        }
        ps[0] = ps[1]; ps[1] = ps[2]; ps[2] = ps[3]; ps[3] = p;
        outc[0] = outc[1]; outc[1] = outc[2]; outc[2] = outc[3]; outc[3] = outcome;
        dst[0] = dst[1]; dst[1] = dst[2]; dst[2] = dst[3]; dst[3] = dest;
    }

    uint32_t nmig = 0, nrem = 0;
#pragma unroll
    for (int j = 0; j < kVec; ++j) {
        const bool leave = outc[j] == kMove;
        const uint32_t o = warp_append(&P.ctr->outbox, leave);
        if (leave) {
            Mover<float> m;
            m.cell = dst[j];
            m.id = P.id ? P.id[s0 + j] : 0u;
            m.x = ps[j].x; m.y = ps[j].y; m.z = ps[j].z;
            m.u = ps[j].u; m.v = ps[j].v; m.w = ps[j].w;
            if (o < P.outbox_cap) {
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
        for (int j = 0; j < kVec; ++j) warp_deposit_leavers<float>(g, outc[j] == kMove, dst[j], ps[j], P.q);
    }
    nmig = __reduce_add_sync(0xffffffffu, nmig);
    nrem = __reduce_add_sync(0xffffffffu, nrem);
    if (lane == 0) {
        if (nmig) atomicAdd(&P.ctr->migrated, nmig);
        if (nrem) atomicAdd(&P.ctr->removed, nrem);
    }

    if (mode == 0 && nv > 0) {
        *reinterpret_cast<float4*>(P.x + s0) = make_float4(ps[0].x, ps[1].x, ps[2].x, ps[3].x);
        *reinterpret_cast<float4*>(P.y + s0) = make_float4(ps[0].y, ps[1].y, ps[2].y, ps[3].y);
        *reinterpret_cast<float4*>(P.z + s0) = make_float4(ps[0].z, ps[1].z, ps[2].z, ps[3].z);
        *reinterpret_cast<float4*>(P.u + s0) = make_float4(ps[0].u, ps[1].u, ps[2].u, ps[3].u);
        *reinterpret_cast<float4*>(P.v + s0) = make_float4(ps[0].v, ps[1].v, ps[2].v, ps[3].v);
        *reinterpret_cast<float4*>(P.w + s0) = make_float4(ps[0].w, ps[1].w, ps[2].w, ps[3].w);
    }

    if (deposit) {
        // monomials -> corner weights: along each axis (a, b) -> (a - b, b),
        // i.e. sum Q (1 - t) and sum Q t; corner bits (i, j, k) = (x, y, z)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float* m = acc + q * 8;
            // m: [1, x, y, z, xy, xz, yz, xyz] -> node order c = i*4 + j*2 + k
            const float a000 = m[0], a100 = m[1], a010 = m[2], a001 = m[3];
            const float a110 = m[4], a101 = m[5], a011 = m[6], a111 = m[7];
            // x axis
            const float b000 = a000 - a100, b100 = a100, b010 = a010 - a110, b110 = a110;
            const float b001 = a001 - a101, b101 = a101, b011 = a011 - a111, b111 = a111;
            // y axis
            const float c000 = b000 - b010, c010 = b010, c100 = b100 - b110, c110 = b110;
            const float c001 = b001 - b011, c011 = b011, c101 = b101 - b111, c111 = b111;
            // z axis
            m[0] = c000 - c001; m[1] = c001;  // corners (0,0,0), (0,0,1)
            m[2] = c010 - c011; m[3] = c011;  // (0,1,0), (0,1,1)
            m[4] = c100 - c101; m[5] = c101;  // (1,0,0), (1,0,1)
            m[6] = c110 - c111; m[7] = c111;  // (1,1,0), (1,1,1)
        }
        // per cell of the warp and value l = q * 8 + corner: lane l sums value
        // l over the cell's lanes (a contiguous run: slots are grouped by
        // cell), then one FP64 atomic per lane and cell (node_atomic_add index
        // corner * 4 + comp with comp = q). Warp-local: no CTA barrier.
        float* tile = s_acc[threadIdx.x >> 5];
#pragma unroll
        for (int l = 0; l < 32; ++l) tile[l * 33 + lane] = acc[l];
        const unsigned todo = __ballot_sync(0xffffffffu, has_acc);
        // first lane of every run of lanes with the same cell
        const int prev_cell = __shfl_up_sync(0xffffffffu, cell, 1);
        unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev_cell != cell);
        __syncwarp();
        const float* row = tile + lane * 33;
        while (heads) {
            const int a = __ffs(heads) - 1;
            heads &= heads - 1;
            const int b = heads ? __ffs(heads) - 1 : 32;  // run [a, b)
            if (!(todo & (((b < 32 ? (1u << b) : 0u) - 1u) & ~((1u << a) - 1u)))) continue;
            float sum = 0.f;
            for (int t = a; t < b; ++t) sum += row[t];
            const int gcell = __shfl_sync(0xffffffffu, cell, a);
            int gx, gy, gz;
            if (g.ncells < (1 << 24) && g.sy < 4096 && g.sz < 4096) {
                const int u = fast_div(gcell, g.sz, pc.inv_sz);
                gz = gcell - u * g.sz;
                gx = fast_div(u, g.sy, pc.inv_sy);
                gy = u - gx * g.sy;
            } else {
                cell_coords(g, gcell, gx, gy, gz);
            }
            node_atomic_add(g, gx, gy, gz, (lane & 7) * 4 + (lane >> 3), (double)sum * P.q);
        }
    }
}

template <int kMinBlocks>
__global__ void __launch_bounds__(kPushThreads, kMinBlocks)
    k_push32(Geom g, Pop<float> P, Push32Const pc, int mode) {
    push32_body(g, P, pc, blockIdx.x, mode);
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
template <int kMinBlocks>
__global__ void __launch_bounds__(kPushThreads, kMinBlocks)
    k_push32_batch(const PopJob<float>* __restrict__ jobs, const int2* __restrict__ cta_job, int mode) {
    __shared__ PopJob<float> job;
    const int2 cj = __ldg(cta_job + blockIdx.x);
    load_job(job, jobs + cj.x);
    push32_body(job.g, job.P, job.pc, cj.y, mode);
}

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
