// Particle initialisation of the AllScale iPIC3D reference, restated for the
// CPU oracle. TEST INFRASTRUCTURE ONLY: it produces, on any machine, the same
// initial particles the reference's host code makes, so that GPU runs on a
// box without the reference sources start from identical inputs.
//
// Follows code/app/include/ipic3d/app/:
//   initCells<Distribution>    cell.h:492-636 (two-phase: pseudo-particle
//                              binning, then per-cell reseeded generation)
//   initCells(uniform)         cell.h:638-697 (the ":U:N" benchmark)
//   vector::uniform / normal   cell.h:138-257, generic generator 262-302
//   ziggurat_normal_distribution  ziggurat_normal_distribution.h:8-127, the
//                              Marsaglia-Tsang ziggurat (J. Stat. Softw. 5(8),
//                              2000) with the reference's 64-bit SHR3 state and
//                              its use of nfix() for every draw.
// The uniform draws use std::minstd_rand and std::uniform_real_distribution
// exactly as the reference does (same standard library on both machines).
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "ipic3d_oracle.h"

namespace {

class Ziggurat {
    uint64_t jz = 0, jsr = 123456789;
    uint64_t kn[128];
    float wn[128], fn[128];

    uint64_t shr3() {
        jz = jsr;
        jsr ^= (jsr << 13);
        jsr ^= (jsr >> 17);
        jsr ^= (jsr << 5);
        return jz + jsr;
    }
    float uni() { return (float)(.5 + (int32_t)(uint32_t)shr3() * .2328306e-9); }

  public:
    explicit Ziggurat(uint64_t seed = 0) {
        const double m1 = 2147483648.0;
        double dn = 3.442619855899, tn = dn, vn = 9.91256303526217e-3, q;
        jsr ^= seed;
        q = vn / exp(-.5 * dn * dn);
        kn[0] = (uint64_t)((dn / q) * m1);
        kn[1] = 0;
        wn[0] = (float)(q / m1);
        wn[127] = (float)(dn / m1);
        fn[0] = 1.;
        fn[127] = (float)(exp(-.5 * dn * dn));
        for (int i = 126; i >= 1; i--) {
            dn = sqrt(-2. * log(vn / dn + exp(-.5 * dn * dn)));
            kn[i + 1] = (uint64_t)((dn / tn) * m1);
            tn = dn;
            fn[i] = (float)(exp(-.5 * dn * dn));
            wn[i] = (float)(dn / m1);
        }
    }

    // one normal variate (the reference's operator() calls nfix directly)
    float operator()() {
        const float r = 3.442620f;
        float value, x, y;
        int hz = (int32_t)(uint32_t)shr3();
        uint32_t iz = (uint32_t)(hz & 127);
        if (fabs((double)hz) < (double)kn[iz]) return (float)(hz)*wn[iz];
        for (;;) {
            if (iz == 0) {
                for (;;) {
                    // log of a float argument is the float overload (logf)
                    // in the reference's C++ translation unit
                    x = (float)(-0.2904764 * std::log(uni()));
                    y = -std::log(uni());
                    if (x * x <= y + y) break;
                }
                value = hz <= 0 ? -r - x : +r + x;
                break;
            }
            x = (float)(hz)*wn[iz];
            if ((double)(fn[iz] + uni() * (fn[iz - 1] - fn[iz])) < exp(-0.5 * (double)x * (double)x)) {
                value = x;
                break;
            }
            hz = (int32_t)(uint32_t)shr3();
            iz = (uint32_t)(hz & 127);
            if (fabs((double)hz) < (double)kn[iz]) {
                value = (float)(hz)*wn[iz];
                break;
            }
        }
        return value;
    }
};

struct UniformVec {  // vector::uniform (cell.h:138-174)
    double lo[3], hi[3];
    std::uniform_real_distribution<> d[3];
    std::minstd_rand g;
    UniformVec(const double* a, const double* b, uint32_t seed)
        : lo{a[0], a[1], a[2]}, hi{b[0], b[1], b[2]}, d{std::uniform_real_distribution<>(a[0], b[0]),
                                                          std::uniform_real_distribution<>(a[1], b[1]),
                                                          std::uniform_real_distribution<>(a[2], b[2])},
          g(seed) {}
    void draw(double* out) {
        out[0] = d[0](g);
        out[1] = d[1](g);
        out[2] = d[2](g);
    }
    void seed(uint32_t s) { g.seed(s); }
};

struct NormalVec {  // vector::normal (cell.h:221-257)
    double mean[3], sd[3];
    Ziggurat z;
    NormalVec(const double* m, const double* s, uint32_t seed) : mean{m[0], m[1], m[2]}, sd{s[0], s[1], s[2]}, z(seed) {}
    void draw(double* out) {
        out[0] = mean[0] + sd[0] * z();
        out[1] = mean[1] + sd[1] * z();
        out[2] = mean[2] + sd[2] * z();
    }
    void seed(uint32_t s) { z = Ziggurat(s); }
};

}  // namespace

extern "C" {

// initCells<uniform_pos_normal_speed<>>(props, numParticles, dist)
// (cell.h:492-636) for dist = uniform positions in [low, hig), normal
// velocities (mean, stddev), as src/ipic3d.cxx:76-83 builds it. Every
// particle gets q = e and qom = e/m (cell.h:624-625). Output grouped by cell
// (row-major); pass out == NULL to get the count only.
int oracle_init_uniform_pos_normal_speed(const ipic3d_props* props, uint64_t numParticles, const double low[3],
                                         const double hig[3], const double mean[3], const double stddev[3],
                                         ipic3d_particle* out, uint64_t* counts, uint64_t* n_out) {
    const int64_t sx = props->size[0], sy = props->size[1], sz = props->size[2];
    const int64_t numCells = sx * sy * sz;
    const double* o = props->origin;
    const double* w = props->cell_width;
    UniformVec pos(low, hig, 0 + 1);
    NormalVec vel(mean, stddev, 0 + 2);
    std::vector<uint64_t> dist(numCells, 0), cnt(numCells, 0);
    const int64_t numPseudo = numCells * 100;
    const uint64_t per = numParticles / (uint64_t)numPseudo;
    const double top[3] = {o[0] + sx * w[0], o[1] + sy * w[1], o[2] + sz * w[2]};
    for (int64_t i = 0; i < numPseudo; ++i) {
        double p[3], v[3];
        for (;;) {
            pos.draw(p);
            vel.draw(v);
            bool in = true;  // isInsideUniverse (cell.h:75-83)
            for (int a = 0; a < 3; ++a) in = in && (o[a] <= p[a]) && (p[a] < top[a]);
            if (in) break;
        }
        int64_t c[3];
        for (int a = 0; a < 3; ++a) c[a] = (int64_t)((p[a] - o[a]) / w[a]);  // getCellCoordinates (cell.h:64-67)
        dist[(c[0] * sy + c[1]) * sz + c[2]] += per;
    }
    uint64_t sum = 0;
    for (int64_t c = 0; c < numCells; ++c) {
        cnt[c] = dist[c];
        sum += cnt[c];
    }
    int64_t missing = (int64_t)numParticles - (int64_t)sum;
    if (missing != 0) {
        int all_correct = (int)(missing / numCells);
        int remain_correct = (int)(missing % numCells);
        for (int64_t c = 0; c < numCells; ++c) {
            cnt[c] += all_correct;
            if (c < remain_correct) cnt[c] += 1;
        }
    }
    uint64_t total = 0;
    for (int64_t c = 0; c < numCells; ++c) total += cnt[c];
    if (n_out) *n_out = total;
    if (!out) return IPIC3D_OK;
    const double e = 1.602176565e-19, m = 1.672621777e-27;
    uint64_t k = 0;
    for (int64_t x = 0; x < sx; ++x)
        for (int64_t y = 0; y < sy; ++y)
            for (int64_t z = 0; z < sz; ++z) {
                const int64_t c = (x * sy + y) * sz + z;
                double lo[3] = {w[0] * x, w[1] * y, w[2] * z};
                for (int a = 0; a < 3; ++a) lo[a] += o[a];
                double hi[3] = {lo[0] + w[0], lo[1] + w[1], lo[2] + w[2]};
                uint32_t seed = (uint32_t)(((x * 1023) + y) * 1023 + z);
                // generic_particle_generator::seed (cell.h:281-287) on a copy
                UniformVec mypos = pos;
                NormalVec myvel = vel;
                uint32_t s = seed;
                s = (1023 * s) & s;
                mypos.seed(s);
                s = (1023 * s) & s;
                myvel.seed(s);
                UniformVec next_position(lo, hi, seed);
                if (counts) counts[c] = cnt[c];
                for (uint64_t i = 0; i < cnt[c]; ++i, ++k) {
                    double p[3], v[3];
                    mypos.draw(p);
                    myvel.draw(v);
                    next_position.draw(p);
                    ipic3d_particle& q = out[k];
                    for (int a = 0; a < 3; ++a) {
                        q.position[a] = p[a];
                        q.velocity[a] = v[a];
                    }
                    q.q = e;
                    q.qom = e / m;
                }
            }
    return IPIC3D_OK;
}

// n draws of uniform_pos_normal_speed<>(low, hig, mean, stddev, seed)
// (cell.h:371-403): positions from the uniform stream seeded seed + 1,
// velocities from the ziggurat seeded seed + 2, species electron (q = -1,
// qom = -25; callers overwrite them where the reference does).
void oracle_generate_uniform_pos_normal_speed(const double low[3], const double hig[3], const double mean[3],
                                              const double stddev[3], uint32_t seed, uint64_t n,
                                              ipic3d_particle* out) {
    UniformVec pos(low, hig, seed + 1);
    NormalVec vel(mean, stddev, seed + 2);
    for (uint64_t i = 0; i < n; ++i) {
        ipic3d_particle& q = out[i];
        q.q = -1.0;
        q.qom = -25.0;
        pos.draw(q.position);
        vel.draw(q.velocity);
    }
}

// initCells(props, numParticles, uniform<>) (cell.h:638-697): the ":U:N"
// benchmark's universe. Velocities U(-0.2, 0.2) per component, electrons
// (q = -1, qom = -25, cell.h:107-118).
int oracle_init_uniform_bench(const ipic3d_props* props, uint64_t numParticles, ipic3d_particle* out,
                              uint64_t* counts) {
    const int64_t sx = props->size[0], sy = props->size[1], sz = props->size[2];
    const int64_t numCells = sx * sy * sz;
    const uint64_t ppc = numParticles / (uint64_t)numCells, remaining = numParticles % (uint64_t)numCells;
    const double* o = props->origin;
    const double* w = props->cell_width;
    const double vlo[3] = {-0.2, -0.2, -0.2}, vhi[3] = {0.2, 0.2, 0.2};
    std::vector<uint64_t> start(numCells + 1, 0);
    for (int64_t c = 0; c < numCells; ++c) start[c + 1] = start[c] + ppc + ((uint64_t)c < remaining ? 1 : 0);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t c = 0; c < numCells; ++c) {
        const int64_t x = c / (sy * sz), y = (c / sz) % sy, z = c % sz;
        double lo[3] = {w[0] * x, w[1] * y, w[2] * z};
        for (int a = 0; a < 3; ++a) lo[a] += o[a];
        double hi[3] = {lo[0] + w[0], lo[1] + w[1], lo[2] + w[2]};
        uint32_t seed = (uint32_t)(((x * 1023) + y) * 1023 + z);
        UniformVec pos(lo, hi, seed + 1);
        UniformVec vel(vlo, vhi, seed + 2);
        if (counts) counts[c] = start[c + 1] - start[c];
        for (uint64_t k = start[c]; k < start[c + 1]; ++k) {
            double p[3], v[3];
            pos.draw(p);
            vel.draw(v);
            ipic3d_particle& q = out[k];
            for (int a = 0; a < 3; ++a) {
                q.position[a] = p[a];
                q.velocity[a] = v[a];
            }
            q.q = -1.0;
            q.qom = -25.0;
        }
    }
    return IPIC3D_OK;
}

}  // extern "C"
