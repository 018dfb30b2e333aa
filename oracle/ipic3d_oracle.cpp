// CPU oracle of the GB300 particle path. TEST INFRASTRUCTURE ONLY: the tests,
// the smoke check and bench.py's CPU baseline use it as the checker / as the
// reference implementation timed on the host cores; the shipped library never
// links it.
//
// It restates the AllScale iPIC3D reference's algorithms in plain C++ with the
// reference's data organisation (one AoS vector of 64-byte particles per cell,
// 26 migration mailboxes per cell, OpenMP loop over cells), so its timing is a
// fair stand-in for the reference's shared-memory CPU run. Arithmetic follows
// the reference expression by expression; build with -ffp-contract=off so no
// multiply-add is fused, as on the reference's x86 build.
//
// Citations are to code/app/include/ipic3d/app/ in the reference unless a
// path says otherwise. Features that the reference does not have (periodic and
// open particle boundaries, injection, charge density, the field-gather mover
// running in a loop) are marked EXTENSION: their parity is not pinned by the
// reference.
#include "ipic3d_oracle.h"

#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V3 {
    double x, y, z;
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scale(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }  // s * v
inline V3 scale(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }  // v * s
inline double sum_sq(V3 a) {
    double r = 0.0;
    r += a.x * a.x;
    r += a.y * a.y;
    r += a.z * a.z;
    return r;
}
inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

struct Part {
    V3 pos, vel;
    double q, qom;
    uint32_t id;
};

// Particle::updatePosition (particle.h:24-26).
inline void push_position(Part& p, double dt) { p.pos = add(p.pos, scale(p.vel, dt)); }

}  // namespace

namespace {

// Particle::updateVelocity, the Boris rotation (particle.h:31-49).
inline void boris(Part& p, V3 E, V3 B, double dt) {
    double k = p.qom * 0.5 * dt;
    V3 t = scale(k, B);
    double t_mag2 = sum_sq(t);
    V3 t2 = scale(2.0, t);
    V3 s = {t2.x / (1.0 + t_mag2), t2.y / (1.0 + t_mag2), t2.z / (1.0 + t_mag2)};
    V3 v_minus = add(p.vel, scale(k, E));
    V3 v_prime = add(v_minus, cross(v_minus, t));
    V3 v_plus = add(v_minus, cross(v_prime, s));
    p.vel = add(v_plus, scale(k, E));
}

// MurmurHash3's 64-bit finaliser (fmix64, A. Appleby, public domain): the
// counter-based generator behind the x=0 injection (EXTENSION). The GPU uses
// the same key schedule, so both inject the same particles.
inline uint64_t fmix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}
inline uint64_t inj_key(uint64_t seed, uint64_t step, uint64_t cell, uint64_t draw) {
    return fmix64(fmix64(seed ^ (step * 0x9E3779B97F4A7C15ULL)) ^ (cell * 0xD1B54A32D192ED03ULL + draw));
}
inline double u01(uint64_t key) { return (double)(key >> 11) * (1.0 / 9007199254740992.0); }

// Reference conversion of the sub-cycle count, int(dt / dt_sub) + 1
// (cell.h:950), with the x86 behaviour of the out-of-range cases spelled out:
// a quotient outside int (or NaN) converts to INT_MIN, so after the "+ 1" and
// the min with 100 the loop runs zero times and the particle stays put.
inline int sub_cycle_count(double ratio) {
    int sc;
    if (ratio >= -2147483648.0 && ratio < 2147483647.0)
        sc = (int)ratio + 1;
    else
        sc = INT_MIN + 1;
    return sc < 100 ? sc : 100;
}

}  // namespace

struct oracle_sim {
    ipic3d_props props;
    ipic3d_config cfg;
    int64_t sx, sy, sz;
    int64_t ncells;
    std::vector<std::vector<Part>> cells;
    // TransferBuffers (transfer_buffer.h:48-95): box[dir][cell], dir = x*9+y*3+z
    // with 0 = predecessor, 1 = centre, 2 = successor, held per receiving cell.
    std::vector<std::vector<Part>> mail;
    std::vector<double> field;    // (s+3)^3 x 9   E,B,Bext
    std::vector<double> bcfield;  // (s+2)^3 x 3   Bc
    std::vector<double> density;  // (s+1)^3 x 3   J
    std::vector<double> rho;      // (s+1)^3       charge density (EXTENSION)
    uint64_t step_index = 0;
    uint64_t migrated = 0, removed = 0, injected = 0;

    int64_t fidx(int64_t x, int64_t y, int64_t z) const { return ((x * (sy + 3)) + y) * (sz + 3) + z; }
    int64_t bidx(int64_t x, int64_t y, int64_t z) const { return ((x * (sy + 2)) + y) * (sz + 2) + z; }
    int64_t didx(int64_t x, int64_t y, int64_t z) const { return ((x * (sy + 1)) + y) * (sz + 1) + z; }
    int64_t cidx(int64_t x, int64_t y, int64_t z) const { return ((x * sy) + y) * sz + z; }
    V3 E(int64_t i) const { return {field[9 * i], field[9 * i + 1], field[9 * i + 2]}; }
    V3 B(int64_t i) const { return {field[9 * i + 3], field[9 * i + 4], field[9 * i + 5]}; }
    V3 Bext(int64_t i) const { return {field[9 * i + 6], field[9 * i + 7], field[9 * i + 8]}; }
    V3 Bc(int64_t i) const { return {bcfield[3 * i], bcfield[3 * i + 1], bcfield[3 * i + 2]}; }
};

namespace {

V3 width(const oracle_sim* s) { return {s->props.cell_width[0], s->props.cell_width[1], s->props.cell_width[2]}; }

// getOriginOfCell (universe_properties.h:125-130): origin + pos * width.
V3 cell_origin(const oracle_sim* s, int64_t x, int64_t y, int64_t z) {
    return {s->props.origin[0] + (double)x * s->props.cell_width[0],
            s->props.origin[1] + (double)y * s->props.cell_width[1],
            s->props.origin[2] + (double)z * s->props.cell_width[2]};
}
// getCenterOfCell (universe_properties.h:139-142): origin of cell + width / 2.
V3 cell_center(const oracle_sim* s, int64_t x, int64_t y, int64_t z) {
    V3 o = cell_origin(s, x, y, z);
    return {o.x + s->props.cell_width[0] / 2.0, o.y + s->props.cell_width[1] / 2.0, o.z + s->props.cell_width[2] / 2.0};
}

// Analytic Earth dipole at the particle position (cell.h:939-945), with
// magneticFieldTemp = -Bext.z * pow(R, 3) (cell.h:923).
V3 dipole_b(const Part& p, double mft) {
    double fac1 = mft / pow(sum_sq(p.pos), 2.5);
    V3 B;
    B.x = 3.0 * p.pos.x * p.pos.z * fac1;
    B.y = 3.0 * p.pos.y * p.pos.z * fac1;
    B.z = (2.0 * pow(p.pos.z, 2) - pow(p.pos.x, 2) - pow(p.pos.y, 2)) * fac1;
    return B;
}

// trilinearInterpolationF2P (cell.h:867-885): corners[i][j][k], weights
// (1-r) for index 0 and r for index 1 per axis, optionally / vol.
V3 trilinear(const V3 c[2][2][2], V3 r, double vol, bool div_vol) {
    V3 res = {0.0, 0.0, 0.0};
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 2; ++k) {
                double fac = (i == 0 ? (1 - r.x) : r.x) * (j == 0 ? (1 - r.y) : r.y) * (k == 0 ? (1 - r.z) : r.z);
                res = add(res, scale(c[i][j][k], fac));
            }
    if (div_vol) res = res / vol;
    return res;
}

// moveParticles (cell.h:896-964) for one cell; with the FIELD mover the
// fields come from the commented gather of cell.h:905-937 instead.
void move_cell(oracle_sim* s, int64_t x, int64_t y, int64_t z, std::vector<Part>& ps) {
    if (ps.empty()) return;
    const ipic3d_props& P = s->props;
    const bool field_mover = s->cfg.mover == IPIC3D_MOVER_FIELD;
    const bool with_dipole = !field_mover || (s->cfg.flags & IPIC3D_F_DIPOLE_IN_GATHER);
    double magneticFieldTemp = -P.external_b[2] * pow(P.planet_radius, 3);
    V3 Es[2][2][2], Bs[2][2][2];
    V3 corigin = cell_origin(s, x, y, z);
    V3 w = width(s);
    double vol = w.x * w.y * w.z;
    if (field_mover) {
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
                for (int k = 0; k < 2; k++) {
                    int64_t n = s->fidx(x + i + 1, y + j + 1, z + k + 1);
                    Es[i][j][k] = s->E(n);
                    Bs[i][j][k] = s->B(n);
                }
    }
    for (Part& p : ps) {
        V3 E = {0.0, 0.0, 0.0}, B = {0.0, 0.0, 0.0};
        if (field_mover) {
            V3 rel = {(p.pos.x - corigin.x) / w.x, (p.pos.y - corigin.y) / w.y, (p.pos.z - corigin.z) / w.z};
            bool dv = (s->cfg.flags & IPIC3D_F_GATHER_DIV_VOL) != 0;
            E = trilinear(Es, rel, vol, dv);
            B = trilinear(Bs, rel, vol, dv);
        }
        if (with_dipole) {
            V3 Bd = dipole_b(p, magneticFieldTemp);
            B = field_mover ? add(B, Bd) : Bd;
        }
        // adaptive sub-cycling (cell.h:947-960); |B|^2 as the reference uses
        double B_mag = sum_sq(B);
        double dt_sub = M_PI * P.speed_of_light / (4.0 * fabs(p.qom) * B_mag);
        int sub_cycles = sub_cycle_count(P.dt / dt_sub);
        dt_sub = P.dt / double(sub_cycles);
        for (int c = 0; c < sub_cycles; c++) {
            boris(p, E, B, dt_sub);
            push_position(p, dt_sub);
        }
    }
}

// Receiving-side slot of a move in direction (i,j,k) in {0,1,2}^3: the
// reference files a particle leaving towards neighbour (i,j,k) under
// TransferDirection(2-i, 2-j, 2-k) of that neighbour (cell.h:1012-1048).
inline int recv_dir(int i, int j, int k) { return (2 - i) * 9 + (2 - j) * 3 + (2 - k); }

// exportParticles (cell.h:975-1159) for one cell, writing leavers into the
// receiving cells' mailboxes. Returns (migrated, removed).
void export_cell(oracle_sim* s, int64_t x, int64_t y, int64_t z, std::vector<Part>& ps, uint64_t& nmig,
                 uint64_t& nrem) {
    const ipic3d_props& P = s->props;
    const int64_t pos[3] = {x, y, z};
    const int64_t size[3] = {s->sx, s->sy, s->sz};
    const V3 w = width(s);
    const V3 center = cell_center(s, x, y, z);
    const V3 halfWidth = {w.x / 2.0, w.y / 2.0, w.z / 2.0};
    // clear the mailboxes this cell fills (cell.h:1050-1086)
    for (int d = 0; d < 27; ++d) {
        int i = d / 9, j = (d / 3) % 3, k = d % 3;
        int64_t nx = (x + (i - 1) + s->sx) % s->sx, ny = (y + (j - 1) + s->sy) % s->sy, nz = (z + (k - 1) + s->sz) % s->sz;
        s->mail[(size_t)recv_dir(i, j, k) * s->ncells + s->cidx(nx, ny, nz)].clear();
    }
    std::vector<Part> remaining;
    remaining.reserve(ps.size());
    for (Part& p : ps) {
        V3 relPos = sub(p.pos, center);
        bool invertVelocity = false, drop = false;
        V3 np = p.pos;
        for (int a = 0; a < 3; ++a) {
            if (pos[a] == 0 && relPos[a] < -halfWidth[a]) {
                if (s->cfg.bc_low[a] == IPIC3D_BC_REFLECT) {  // cell.h:1105-1107
                    invertVelocity = true;
                    np[a] = p.pos[a] + halfWidth[a];
                } else if (s->cfg.bc_low[a] == IPIC3D_BC_OPEN) {  // EXTENSION
                    drop = true;
                }
            } else if (pos[a] == size[a] - 1 && relPos[a] > halfWidth[a]) {
                if (s->cfg.bc_high[a] == IPIC3D_BC_REFLECT) {  // cell.h:1108-1110
                    invertVelocity = true;
                    np[a] = p.pos[a] - halfWidth[a];
                } else if (s->cfg.bc_high[a] == IPIC3D_BC_OPEN) {  // EXTENSION
                    drop = true;
                }
            }
        }
        p.pos = np;
        if (invertVelocity) p.vel = scale(p.vel, -1.0);  // cell.h:1119-1121
        if (drop) {
            ++nrem;
            continue;
        }
        // remove particles inside the planet (cell.h:1123-1128)
        V3 diff = sub(p.pos, {P.object_center[0], P.object_center[1], P.object_center[2]});
        double r2 = sum_sq(diff);
        if (r2 <= P.planet_radius * P.planet_radius) {
            ++nrem;
            continue;
        }
        relPos = sub(p.pos, center);
        if ((fabs(relPos.x) > halfWidth.x) || (fabs(relPos.y) > halfWidth.y) || (fabs(relPos.z) > halfWidth.z)) {
            int d3[3];
            for (int a = 0; a < 3; ++a) d3[a] = (relPos[a] < -halfWidth[a]) ? 0 : ((relPos[a] > halfWidth[a]) ? 2 : 1);
            // EXTENSION: periodic faces move the position with the cell index
            for (int a = 0; a < 3; ++a) {
                int64_t t = pos[a] + d3[a] - 1;
                if (t < 0 && s->cfg.bc_low[a] == IPIC3D_BC_PERIODIC) p.pos[a] += (double)size[a] * w[a];
                if (t >= size[a] && s->cfg.bc_high[a] == IPIC3D_BC_PERIODIC) p.pos[a] -= (double)size[a] * w[a];
            }
            int64_t nx = (x + (d3[0] - 1) + s->sx) % s->sx, ny = (y + (d3[1] - 1) + s->sy) % s->sy,
                    nz = (z + (d3[2] - 1) + s->sz) % s->sz;
            s->mail[(size_t)recv_dir(d3[0], d3[1], d3[2]) * s->ncells + s->cidx(nx, ny, nz)].push_back(p);
            ++nmig;
        } else {
            remaining.push_back(p);
        }
    }
    ps.swap(remaining);
}

// importParticles (cell.h:1195-1310): append the 26 mailboxes in the fixed
// order TransferDirection(0,0,0), (0,0,1), ..., (2,2,2), skipping (1,1,1).
void import_cell(oracle_sim* s, int64_t c, std::vector<Part>& ps) {
    size_t add_n = 0;
    for (int d = 0; d < 27; ++d)
        if (d != 13) add_n += s->mail[(size_t)d * s->ncells + c].size();
    ps.reserve(ps.size() + add_n);
    for (int d = 0; d < 27; ++d) {
        if (d == 13) continue;
        auto& box = s->mail[(size_t)d * s->ncells + c];
        ps.insert(ps.end(), box.begin(), box.end());
    }
}

// EXTENSION: drifting-Maxwellian injection into the x = 0 cell layer.
uint64_t inject(oracle_sim* s) {
    const ipic3d_config& C = s->cfg;
    const ipic3d_props& P = s->props;
    uint64_t total = 0;
    for (int64_t j = 0; j < s->sy; ++j)
        for (int64_t k = 0; k < s->sz; ++k) {
            uint64_t c = (uint64_t)s->cidx(0, j, k);
            uint64_t n = (uint64_t)floor(C.inject_per_cell + u01(inj_key(C.seed, s->step_index, c, 0)));
            auto& cell = s->cells[c];
            for (uint64_t m = 0; m < n; ++m) {
                uint64_t d = 1 + 8 * m;
                double u[7];
                for (int t = 0; t < 7; ++t) u[t] = u01(inj_key(C.seed, s->step_index, c, d + t));
                Part p;
                p.pos.x = P.origin[0] + u[0] * P.cell_width[0];
                p.pos.y = P.origin[1] + ((double)j + u[1]) * P.cell_width[1];
                p.pos.z = P.origin[2] + ((double)k + u[2]) * P.cell_width[2];
                double g1 = sqrt(-2.0 * log(1.0 - u[3])), th1 = 2.0 * M_PI * u[4];
                double g2 = sqrt(-2.0 * log(1.0 - u[5])), th2 = 2.0 * M_PI * u[6];
                p.vel.x = C.inject_drift[0] + C.inject_vth[0] * (g1 * cos(th1));
                p.vel.y = C.inject_drift[1] + C.inject_vth[1] * (g1 * sin(th1));
                p.vel.z = C.inject_drift[2] + C.inject_vth[2] * (g2 * cos(th2));
                p.q = C.inject_q;
                p.qom = C.inject_qom;
                p.id = UINT32_MAX;
                cell.push_back(p);
            }
            total += n;
        }
    return total;
}

// projectToDensityField (cell.h:787-824) for every node, plus the charge
// density from the same weights (EXTENSION).
void project(oracle_sim* s) {
    const V3 w = width(s);
    const double vol = w.x * w.y * w.z;
    const bool div8 = (s->cfg.flags & IPIC3D_F_J_DIV8) != 0;
    const int64_t size[3] = {s->sx, s->sy, s->sz};
    const int64_t nx = s->sx + 1, ny = s->sy + 1, nz = s->sz + 1;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t n = 0; n < nx * ny * nz; ++n) {
        int64_t pos[3] = {n / (ny * nz), (n / nz) % ny, n % nz};
        V3 Js = {0.0, 0.0, 0.0};
        double rs = 0.0;
        for (int i = -1; i < 1; i++)
            for (int j = -1; j < 1; j++)
                for (int k = -1; k < 1; k++) {
                    int64_t cur[3] = {pos[0] + i, pos[1] + j, pos[2] + k};
                    for (int a = 0; a < 3; ++a)  // periodic wrap of the cell index (cell.h:799-805)
                        cur[a] = (cur[a] < 0) ? size[a] - 1 : ((cur[a] >= size[a]) ? 0 : cur[a]);
                    const V3 co = cell_origin(s, cur[0], cur[1], cur[2]);
                    for (const Part& p : s->cells[s->cidx(cur[0], cur[1], cur[2])]) {
                        V3 relPos = {(p.pos.x - co.x) / w.x, (p.pos.y - co.y) / w.y, (p.pos.z - co.z) / w.z};
                        double fac = (i == 0 ? (1 - relPos.x) : relPos.x) * (j == 0 ? (1 - relPos.y) : relPos.y) *
                                     (k == 0 ? (1 - relPos.z) : relPos.z);
                        Js = add(Js, scale(scale(p.q, p.vel), fac));
                        rs += p.q * fac;
                    }
                }
        V3 J = Js / vol;
        double r = rs / vol;
        if (div8) {
            J = J / 8.0;
            r = r / 8.0;
        }
        s->density[3 * n] = J.x;
        s->density[3 * n + 1] = J.y;
        s->density[3 * n + 2] = J.z;
        s->rho[n] = r;
    }
}

// updateFieldsOnBoundaries (field.h:407-440): copy the 6 ghost faces of Field
// (whole nodes) and BcField; edges and corners keep their values.
void update_boundaries(oracle_sim* s) {
    auto run = [&](double* g, int64_t n, int per) {
        int64_t end = n - 1;
        auto at = [&](int64_t x, int64_t y, int64_t z) { return g + ((x * n + y) * n + z) * per; };
        auto cp = [&](double* dst, const double* src) { std::memcpy(dst, src, sizeof(double) * per); };
        for (int64_t a = 1; a < end; ++a)
            for (int64_t b = 1; b < end; ++b) {
                cp(at(0, a, b), at(end - 1, a, b));
                cp(at(end, a, b), at(1, a, b));
                cp(at(a, 0, b), at(a, end - 1, b));
                cp(at(a, end, b), at(a, 1, b));
                cp(at(a, b, 0), at(a, b, end - 1));
                cp(at(a, b, end), at(a, b, 1));
            }
    };
    run(s->field.data(), s->sx + 3, 9);
    run(s->bcfield.data(), s->sx + 2, 3);
}

// solveFieldLeapfrog (field.h:342-372) over [1, size+2)^3, as two phases:
// every E first (from the old Bc and J[pos-1]), then every Bc with
// pos < size+1 (from the new E). The reference updates both in one in-place
// pass whose result depends on the visiting order; the two-phase reading
// equals its reverse-row-major sweep.
void leapfrog(oracle_sim* s) {
    const ipic3d_props& P = s->props;
    const double dt = P.dt, c = P.speed_of_light;
    const double wx = P.cell_width[0], wy = P.cell_width[1], wz = P.cell_width[2];
    const int64_t end = s->sx + 2;
#pragma omp parallel for
    for (int64_t x = 1; x < end; ++x)
        for (int64_t y = 1; y < end; ++y)
            for (int64_t z = 1; z < end; ++z) {
                int64_t f = s->fidx(x, y, z);
                V3 Bc = s->Bc(s->bidx(x, y, z));
                V3 Bym = s->Bc(s->bidx(x, y - 1, z)), Bzm = s->Bc(s->bidx(x, y, z - 1)), Bxm = s->Bc(s->bidx(x - 1, y, z));
                int64_t d = s->didx(x - 1, y - 1, z - 1);
                double* E = &s->field[9 * f];
                E[0] = E[0] + dt * (c * c * ((Bc.z - Bym.z) / wy - (Bc.y - Bzm.y) / wz) - s->density[3 * d]);
                E[1] = E[1] + dt * (c * c * ((Bc.x - Bzm.x) / wz - (Bc.z - Bxm.z) / wx) - s->density[3 * d + 1]);
                E[2] = E[2] + dt * (c * c * ((Bc.y - Bxm.y) / wx - (Bc.x - Bym.x) / wy) - s->density[3 * d + 2]);
            }
#pragma omp parallel for
    for (int64_t x = 1; x < end - 1; ++x)
        for (int64_t y = 1; y < end - 1; ++y)
            for (int64_t z = 1; z < end - 1; ++z) {
                V3 E0 = s->E(s->fidx(x, y, z));
                V3 Ex = s->E(s->fidx(x + 1, y, z)), Ey = s->E(s->fidx(x, y + 1, z)), Ez = s->E(s->fidx(x, y, z + 1));
                double* Bc = &s->bcfield[3 * s->bidx(x, y, z)];
                Bc[0] = Bc[0] - dt * ((Ey.z - E0.z) / wy - (Ez.y - E0.y) / wz);
                Bc[1] = Bc[1] - dt * ((Ez.x - E0.x) / wz - (Ex.z - E0.z) / wx);
                Bc[2] = Bc[2] - dt * ((Ex.y - E0.y) / wx - (Ey.x - E0.x) / wy);
            }
}

// interpC2N (field.h:234-247): node B = 1/8 sum of the 8 surrounding Bc.
void interp_c2n(oracle_sim* s) {
    const int64_t end = s->sx + 2;
#pragma omp parallel for
    for (int64_t x = 1; x < end; ++x)
        for (int64_t y = 1; y < end; ++y)
            for (int64_t z = 1; z < end; ++z) {
                V3 acc = {0.0, 0.0, 0.0};
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++)
                        for (int k = 0; k < 2; k++) acc = add(acc, s->Bc(s->bidx(x - i, y - j, z - k)));
                double* B = &s->field[9 * s->fidx(x, y, z) + 3];
                V3 r = scale(.125, acc);
                B[0] = r.x;
                B[1] = r.y;
                B[2] = r.z;
            }
}

// solveFieldForward (field.h:294-337) as three phases over [1, size+2)^3:
// E += (c curlB - J[pos-1]) dt; Bc -= c curlE dt for pos < size+1; node B =
// interpC2N. computeCurlB / computeCurlE are field.h:162-229.
void forward(oracle_sim* s) {
    const ipic3d_props& P = s->props;
    const double dt = P.dt, c = P.speed_of_light;
    const double wx = P.cell_width[0], wy = P.cell_width[1], wz = P.cell_width[2];
    const int64_t end = s->sx + 2;
#pragma omp parallel for
    for (int64_t x = 1; x < end; ++x)
        for (int64_t y = 1; y < end; ++y)
            for (int64_t z = 1; z < end; ++z) {
                V3 Bs[2][2][2];
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++)
                        for (int k = 0; k < 2; k++) Bs[i][j][k] = s->Bc(s->bidx(x - i, y - j, z - k));
                V3 curl;
                double compZDY = .25 * (Bs[0][0][0].z - Bs[0][1][0].z + Bs[0][0][1].z - Bs[0][1][1].z + Bs[1][0][0].z - Bs[1][1][0].z + Bs[1][0][1].z - Bs[1][1][1].z) / wy;
                double compYDZ = .25 * (Bs[0][0][0].y - Bs[0][0][1].y + Bs[1][0][0].y - Bs[1][0][1].y + Bs[0][1][0].y - Bs[0][1][1].y + Bs[1][1][0].y - Bs[1][1][1].y) / wz;
                curl.x = compZDY - compYDZ;
                double compXDZ = .25 * (Bs[0][0][0].x - Bs[0][0][1].x + Bs[1][0][0].x - Bs[1][0][1].x + Bs[0][1][0].x - Bs[0][1][1].x + Bs[1][1][0].x - Bs[1][1][1].x) / wz;
                double compZDX = .25 * (Bs[0][0][0].z - Bs[1][0][0].z + Bs[0][0][1].z - Bs[1][0][1].z + Bs[0][1][0].z - Bs[1][1][0].z + Bs[0][1][1].z - Bs[1][1][1].z) / wx;
                curl.y = compXDZ - compZDX;
                double compYDX = .25 * (Bs[0][0][0].y - Bs[1][0][0].y + Bs[0][0][1].y - Bs[1][0][1].y + Bs[0][1][0].y - Bs[1][1][0].y + Bs[0][1][1].y - Bs[1][1][1].y) / wx;
                double compXDY = .25 * (Bs[0][0][0].x - Bs[0][1][0].x + Bs[0][0][1].x - Bs[0][1][1].x + Bs[1][0][0].x - Bs[1][1][0].x + Bs[1][0][1].x - Bs[1][1][1].x) / wy;
                curl.z = compYDX - compXDY;
                int64_t d = s->didx(x - 1, y - 1, z - 1);
                V3 J = {s->density[3 * d], s->density[3 * d + 1], s->density[3 * d + 2]};
                V3 inc = scale(sub(scale(c, curl), J), dt);
                double* E = &s->field[9 * s->fidx(x, y, z)];
                E[0] += inc.x;
                E[1] += inc.y;
                E[2] += inc.z;
            }
#pragma omp parallel for
    for (int64_t x = 1; x < end - 1; ++x)
        for (int64_t y = 1; y < end - 1; ++y)
            for (int64_t z = 1; z < end - 1; ++z) {
                V3 Es[2][2][2];
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++)
                        for (int k = 0; k < 2; k++) Es[i][j][k] = s->E(s->fidx(x + i, y + j, z + k));
                V3 curl;
                double compZDY = .25 * (Es[0][1][0].z - Es[0][0][0].z + Es[0][1][1].z - Es[0][0][1].z + Es[1][1][0].z - Es[1][0][0].z + Es[1][1][1].z - Es[1][0][1].z) / wy;
                double compYDZ = .25 * (Es[0][0][1].y - Es[0][0][0].y + Es[1][0][1].y - Es[1][0][0].y + Es[0][1][1].y - Es[0][1][0].y + Es[1][1][1].y - Es[1][1][0].y) / wz;
                curl.x = compZDY - compYDZ;
                double compXDZ = .25 * (Es[0][0][1].x - Es[0][0][0].x + Es[1][0][1].x - Es[1][0][0].x + Es[0][1][1].x - Es[0][1][0].x + Es[1][1][1].x - Es[1][1][0].x) / wz;
                double compZDX = .25 * (Es[1][0][0].z - Es[0][0][0].z + Es[1][0][1].z - Es[0][0][1].z + Es[1][1][0].z - Es[0][1][0].z + Es[1][1][1].z - Es[0][1][1].z) / wx;
                curl.y = compXDZ - compZDX;
                double compYDX = .25 * (Es[1][0][0].y - Es[0][0][0].y + Es[1][0][1].y - Es[0][0][1].y + Es[1][1][0].y - Es[0][1][0].y + Es[1][1][1].y - Es[0][1][1].y) / wx;
                double compXDY = .25 * (Es[0][1][0].x - Es[0][0][0].x + Es[0][1][1].x - Es[0][0][1].x + Es[1][1][0].x - Es[1][0][0].x + Es[1][1][1].x - Es[1][0][1].x) / wy;
                curl.z = compYDX - compXDY;
                V3 dec = scale(scale(c, curl), dt);
                double* Bc = &s->bcfield[3 * s->bidx(x, y, z)];
                Bc[0] -= dec.x;
                Bc[1] -= dec.y;
                Bc[2] -= dec.z;
            }
    interp_c2n(s);
}

}  // namespace

extern "C" {

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_create(const ipic3d_props* props, const ipic3d_config* cfg, oracle_sim** out) {
    if (!props || !cfg || !out) return IPIC3D_E_INVALID;
    for (int a = 0; a < 3; ++a)
        if (props->size[a] <= 0 || !(props->cell_width[a] > 0)) return IPIC3D_E_INVALID;
    // the field solvers and the ghost copy assume a cubic grid (field.h:424)
    if (cfg->solver != IPIC3D_SOLVER_STATIC && !(props->size[0] == props->size[1] && props->size[1] == props->size[2]))
        return IPIC3D_E_INVALID;
    auto* s = new (std::nothrow) oracle_sim();
    if (!s) return IPIC3D_E_NOMEM;
    s->props = *props;
    s->cfg = *cfg;
    s->sx = props->size[0];
    s->sy = props->size[1];
    s->sz = props->size[2];
    s->ncells = s->sx * s->sy * s->sz;
    s->cells.resize((size_t)s->ncells);
    s->mail.resize((size_t)s->ncells * 27);
    s->field.assign((size_t)((s->sx + 3) * (s->sy + 3) * (s->sz + 3) * 9), 0.0);
    s->bcfield.assign((size_t)((s->sx + 2) * (s->sy + 2) * (s->sz + 2) * 3), 0.0);
    s->density.assign((size_t)((s->sx + 1) * (s->sy + 1) * (s->sz + 1) * 3), 0.0);
    s->rho.assign((size_t)((s->sx + 1) * (s->sy + 1) * (s->sz + 1)), 0.0);
    *out = s;
    return IPIC3D_OK;
}

void oracle_destroy(oracle_sim* s) { delete s; }

int oracle_upload_particles(oracle_sim* s, const ipic3d_particle* p, const uint64_t* counts, const uint32_t* ids) {
    uint64_t k = 0;
    for (int64_t c = 0; c < s->ncells; ++c) {
        auto& v = s->cells[c];
        v.clear();
        v.reserve(counts[c]);
        for (uint64_t i = 0; i < counts[c]; ++i, ++k) {
            Part q;
            q.pos = {p[k].position[0], p[k].position[1], p[k].position[2]};
            q.vel = {p[k].velocity[0], p[k].velocity[1], p[k].velocity[2]};
            q.q = p[k].q;
            q.qom = p[k].qom;
            q.id = ids ? ids[k] : (uint32_t)k;
            v.push_back(q);
        }
    }
    return IPIC3D_OK;
}

int oracle_upload_fields(oracle_sim* s, const double* field, const double* bcfield, const double* density) {
    if (field) std::memcpy(s->field.data(), field, s->field.size() * sizeof(double));
    if (bcfield) std::memcpy(s->bcfield.data(), bcfield, s->bcfield.size() * sizeof(double));
    if (density) std::memcpy(s->density.data(), density, s->density.size() * sizeof(double));
    return IPIC3D_OK;
}

int oracle_download_fields(oracle_sim* s, double* field, double* bcfield, double* density, double* rho) {
    if (field) std::memcpy(field, s->field.data(), s->field.size() * sizeof(double));
    if (bcfield) std::memcpy(bcfield, s->bcfield.data(), s->bcfield.size() * sizeof(double));
    if (density) std::memcpy(density, s->density.data(), s->density.size() * sizeof(double));
    if (rho) std::memcpy(rho, s->rho.data(), s->rho.size() * sizeof(double));
    return IPIC3D_OK;
}

uint64_t oracle_particle_count(oracle_sim* s) {
    uint64_t n = 0;
    for (auto& v : s->cells) n += v.size();
    return n;
}

int oracle_download_particles(oracle_sim* s, ipic3d_particle* p, uint64_t cap, uint64_t* counts, uint32_t* ids) {
    uint64_t k = 0;
    for (int64_t c = 0; c < s->ncells; ++c) {
        if (counts) counts[c] = s->cells[c].size();
        for (const Part& q : s->cells[c]) {
            if (k >= cap) return IPIC3D_E_CAPACITY;
            if (p) {
                p[k].position[0] = q.pos.x;
                p[k].position[1] = q.pos.y;
                p[k].position[2] = q.pos.z;
                p[k].velocity[0] = q.vel.x;
                p[k].velocity[1] = q.vel.y;
                p[k].velocity[2] = q.vel.z;
                p[k].q = q.q;
                p[k].qom = q.qom;
            }
            if (ids) ids[k] = q.id;
            ++k;
        }
    }
    return IPIC3D_OK;
}

int oracle_project(oracle_sim* s) {
    project(s);
    return IPIC3D_OK;
}

int oracle_update_boundaries(oracle_sim* s) {
    update_boundaries(s);
    return IPIC3D_OK;
}

int oracle_solve_fields(oracle_sim* s) {
    if (s->cfg.solver == IPIC3D_SOLVER_LEAPFROG) {
        leapfrog(s);
        if (s->cfg.flags & IPIC3D_F_REFRESH_NODE_B) interp_c2n(s);
    } else if (s->cfg.solver == IPIC3D_SOLVER_FORWARD) {
        forward(s);
    }
    return IPIC3D_OK;
}

// mover + export over all cells, then import (simulator.h:214-223)
int oracle_move(oracle_sim* s) {
    uint64_t nmig = 0, nrem = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : nmig, nrem)
    for (int64_t c = 0; c < s->ncells; ++c) {
        int64_t x = c / (s->sy * s->sz), y = (c / s->sz) % s->sy, z = c % s->sz;
        move_cell(s, x, y, z, s->cells[c]);
        export_cell(s, x, y, z, s->cells[c], nmig, nrem);
    }
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t c = 0; c < s->ncells; ++c) import_cell(s, c, s->cells[c]);
    s->migrated = nmig;
    s->removed = nrem;
    s->injected = 0;
    if ((s->cfg.flags & IPIC3D_F_INJECT_LOW_X) && s->cfg.bc_low[0] == IPIC3D_BC_OPEN) s->injected = inject(s);
    return IPIC3D_OK;
}

int oracle_step(oracle_sim* s, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) {
        if (s->cfg.projector == IPIC3D_PROJECT_CIC) project(s);
        if (s->cfg.solver != IPIC3D_SOLVER_STATIC) {
            update_boundaries(s);
            oracle_solve_fields(s);
        }
        oracle_move(s);
        ++s->step_index;
    }
    return IPIC3D_OK;
}

int oracle_last_counts(oracle_sim* s, uint64_t* migrated, uint64_t* removed, uint64_t* injected) {
    if (migrated) *migrated = s->migrated;
    if (removed) *removed = s->removed;
    if (injected) *injected = s->injected;
    return IPIC3D_OK;
}

// writeOutputData's quantities (simulator.h:76-83): field energies over the
// interior nodes [1, size+2)^3 (field.h:443-459); particle sums per cell then
// over cells in row-major order (cell.h:1315-1355).
int oracle_conserved(oracle_sim* s, ipic3d_conserved* out) {
    const ipic3d_props& P = s->props;
    const double vol = 0.5 * P.cell_width[0] * P.cell_width[1] * P.cell_width[2];
    const double fourPI = 16.0 * atan(1.0);
    double ee = 0.0, be = 0.0;
    const int64_t end = s->sx + 2;
    for (int64_t x = 1; x < end; ++x)
        for (int64_t y = 1; y < end; ++y)
            for (int64_t z = 1; z < end; ++z) {
                int64_t f = s->fidx(x, y, z);
                ee += vol * sum_sq(s->E(f)) / (fourPI);
                be += vol * sum_sq(add(s->B(f), s->Bext(f))) / (fourPI);
            }
    double mom = 0.0, ke = 0.0, q = 0.0;
    uint64_t n = 0;
    for (const auto& cell : s->cells) {
        double cm = 0.0, ck = 0.0;
        for (const Part& p : cell) {
            cm += (p.q / p.qom) * sqrt(sum_sq(p.vel));
            ck += 0.5 * (p.q / p.qom) * sum_sq(p.vel);
            q += p.q;
        }
        mom += cm;
        ke += ck;
        n += cell.size();
    }
    out->total_momentum = mom;
    out->e_energy = ee;
    out->b_energy = be;
    out->kinetic_energy = ke;
    out->total_charge = q;
    out->particles = n;
    return IPIC3D_OK;
}

int oracle_boris(ipic3d_particle* ps, uint64_t n, const double E[3], const double B[3], double dt, uint64_t nsteps,
                 int push_pos) {
    for (uint64_t i = 0; i < n; ++i) {
        Part p;
        p.pos = {ps[i].position[0], ps[i].position[1], ps[i].position[2]};
        p.vel = {ps[i].velocity[0], ps[i].velocity[1], ps[i].velocity[2]};
        p.q = ps[i].q;
        p.qom = ps[i].qom;
        for (uint64_t t = 0; t < nsteps; ++t) {
            boris(p, {E[0], E[1], E[2]}, {B[0], B[1], B[2]}, dt);
            if (push_pos) push_position(p, dt);
        }
        ps[i].position[0] = p.pos.x;
        ps[i].position[1] = p.pos.y;
        ps[i].position[2] = p.pos.z;
        ps[i].velocity[0] = p.vel.x;
        ps[i].velocity[1] = p.vel.y;
        ps[i].velocity[2] = p.vel.z;
    }
    return IPIC3D_OK;
}

// aggregateDensityContributions (cell.h:835-855) for every node of the
// (size+1)^3 J grid from a (2 size)^3 contribution grid: J += the up to 8
// contributions at 2 pos + {-1, 0}^3 inside that grid (in i, j, k order),
// then J / vol / 8. J is updated in place.
int oracle_aggregate_contributions(const ipic3d_props* props, const double* contrib, double* J) {
    const int64_t cs[3] = {2 * props->size[0], 2 * props->size[1], 2 * props->size[2]};
    const int64_t ns[3] = {props->size[0] + 1, props->size[1] + 1, props->size[2] + 1};
    const double vol = props->cell_width[0] * props->cell_width[1] * props->cell_width[2];
    for (int64_t x = 0; x < ns[0]; ++x)
        for (int64_t y = 0; y < ns[1]; ++y)
            for (int64_t z = 0; z < ns[2]; ++z) {
                double* j = J + 3 * ((x * ns[1] + y) * ns[2] + z);
                V3 acc = {j[0], j[1], j[2]};
                for (int i = 0; i < 2; ++i)
                    for (int jj = 0; jj < 2; ++jj)
                        for (int k = 0; k < 2; ++k) {
                            const int64_t c[3] = {2 * x + i - 1, 2 * y + jj - 1, 2 * z + k - 1};
                            bool in = true;
                            for (int a = 0; a < 3; ++a) in = in && c[a] >= 0 && c[a] < cs[a];
                            if (!in) continue;
                            const double* q = contrib + 3 * ((c[0] * cs[1] + c[1]) * cs[2] + c[2]);
                            acc = add(acc, V3{q[0], q[1], q[2]});
                        }
                j[0] = acc.x / vol / 8.0;
                j[1] = acc.y / vol / 8.0;
                j[2] = acc.z / vol / 8.0;
            }
    return IPIC3D_OK;
}

double oracle_trilinear(const double corners[8], const double pos[3], double vol) {
    V3 c[2][2][2];
    for (int i = 0; i < 8; ++i) c[i / 4][(i / 2) % 2][i % 2] = {corners[i], 0.0, 0.0};
    return trilinear(c, {pos[0], pos[1], pos[2]}, vol, true).x;
}

}  // extern "C"
