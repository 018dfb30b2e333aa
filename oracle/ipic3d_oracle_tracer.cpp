// The reference's standalone particle tracer (code/app/src/pic_tracer.cxx),
// restated for the CPU oracle. TEST INFRASTRUCTURE ONLY: the tests check the
// GPU tracer against it, and bench.py times it as the CPU baseline of the
// tracer workload.
//
//   oracle_tracer_config     the UniverseProperties main builds (pic_tracer.cxx:196-214)
//   oracle_tracer_particles  the map operator's particle stream (pic_tracer.cxx:225-247):
//                            uniform_pos_normal_speed<> (cell.h:371-403) over the
//                            middle 3/4 of the box, normal speeds of width v_mod,
//                            q = e, qom = e/m
//   oracle_trace             traceParticle (pic_tracer.cxx:77-148) for every particle,
//                            counting into the ParticleCount vector (pic_tracer.cxx:26-71)
// Expressions follow the reference term by term (build with
// -ffp-contract=off); pow() is the host libm's, as in the reference.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "ipic3d_oracle.h"

namespace {

constexpr double kE = 1.602176565e-19;     // elementary charge (pic_tracer.cxx:220)
constexpr double kMp = 1.672621777e-27;    // proton mass (pic_tracer.cxx:222)

struct Tracer {
    double low[3], high[3], extent[3], origin[3], w[3], center[3];
    double r2max, bz, R, dt, c;
    int64_t size[3];
};

inline double sum_sq(double a, double b, double c) {
    double r = 0.0;  // allscale::utils::sumOfSquares (utils/vector.h)
    r += a * a;
    r += b * b;
    r += c * c;
    return r;
}

// Particle::updateVelocity (particle.h:31-49) with E = 0, written as the
// reference's vector expressions evaluate
void update_velocity(double v[3], const double B[3], double qom, double dt) {
    const double E[3] = {0.0, 0.0, 0.0};
    const double k = qom * 0.5 * dt;
    const double t[3] = {k * B[0], k * B[1], k * B[2]};
    const double t_mag2 = sum_sq(t[0], t[1], t[2]);
    const double s[3] = {(2.0 * t[0]) / (1.0 + t_mag2), (2.0 * t[1]) / (1.0 + t_mag2), (2.0 * t[2]) / (1.0 + t_mag2)};
    const double kE[3] = {k * E[0], k * E[1], k * E[2]};
    const double vm[3] = {v[0] + kE[0], v[1] + kE[1], v[2] + kE[2]};
    const double vmxt[3] = {vm[1] * t[2] - vm[2] * t[1], vm[2] * t[0] - vm[0] * t[2], vm[0] * t[1] - vm[1] * t[0]};
    const double vp[3] = {vm[0] + vmxt[0], vm[1] + vmxt[1], vm[2] + vmxt[2]};
    const double vpxs[3] = {vp[1] * s[2] - vp[2] * s[1], vp[2] * s[0] - vp[0] * s[2], vp[0] * s[1] - vp[1] * s[0]};
    const double vplus[3] = {vm[0] + vpxs[0], vm[1] + vpxs[1], vm[2] + vpxs[2]};
    v[0] = vplus[0] + kE[0];
    v[1] = vplus[1] + kE[1];
    v[2] = vplus[2] + kE[2];
}

// traceParticle (pic_tracer.cxx:77-148); counts has frames x cells entries
void trace_particle(ipic3d_particle p, int T, const Tracer& g, int frame_interval, uint32_t* counts,
                    int64_t total) {
    double* P = p.position;
    for (int a = 0; a < 3; ++a) P[a] += g.center[a];
    if (sum_sq(P[0] - g.center[0], P[1] - g.center[1], P[2] - g.center[2]) < g.r2max) return;
    for (int a = 0; a < 3; ++a) {
        if (P[a] > g.high[a]) return;
        if (P[a] < g.low[a]) return;
    }
    for (int t = 0; t < T; t++) {
        int64_t pos[3];  // getCellCoordinates (cell.h:64-67)
        for (int a = 0; a < 3; ++a) pos[a] = (int64_t)((P[a] - g.origin[a]) / g.w[a]);
        const double fac1 = -g.bz * pow(g.R, 3) / pow(sum_sq(P[0], P[1], P[2]), 2.5);
        double B[3];
        B[0] = 3.0 * P[0] * P[2] * fac1;
        B[1] = 3.0 * P[1] * P[2] * fac1;
        B[2] = (2.0 * pow(P[2], 2) - pow(P[0], 2) - pow(P[1], 2)) * fac1;
        const double B_mag = sum_sq(B[0], B[1], B[2]);
        double dt_sub = M_PI * g.c / (4.0 * fabs(p.qom) * B_mag);
        int sub_cycles;
        const double ratio = g.dt / dt_sub;
        // int(dt / dt_sub): out-of-range quotients give INT_MIN on the
        // reference's x86 build (no sub-cycle runs)
        sub_cycles = (ratio >= -2147483648.0 && ratio < 2147483647.0) ? int(ratio) + 1 : INT32_MIN + 1;
        sub_cycles = sub_cycles < 100 ? sub_cycles : 100;
        dt_sub = g.dt / double(sub_cycles);
        for (int cyc = 0; cyc < sub_cycles; cyc++) {
            update_velocity(p.velocity, B, p.qom, dt_sub);
            for (int a = 0; a < 3; ++a) P[a] += p.velocity[a] * dt_sub;  // updatePosition (particle.h:24-26)
        }
        for (int a = 0; a < 3; ++a) {
            if (P[a] > g.high[a]) P[a] -= g.extent[a];
            if (P[a] < g.low[a]) P[a] += g.extent[a];
        }
        if (sum_sq(P[0] - g.center[0], P[1] - g.center[1], P[2] - g.center[2]) <= g.r2max) return;
        if (t % frame_interval == 0) {
            // ParticleCount::increment(t / frame_interval, pos): its flat
            // index with the coordinates cast to int; an index outside the
            // vector (undefined in the reference) is not counted
            const int64_t idx = (((int64_t)(t / frame_interval) * g.size[0] + (int)pos[0]) * g.size[1] + (int)pos[1]) *
                                    g.size[2] +
                                (int)pos[2];
            if (idx >= 0 && idx < total) counts[idx] += 1;
        }
    }
}

}  // namespace

extern "C" {

int oracle_tracer_config(int32_t R, ipic3d_props* out) {
    if (R <= 0 || !out) return -1;
    std::memset(out, 0, sizeof(*out));
    out->dt = 0.01;
    out->speed_of_light = 299792458;
    for (int a = 0; a < 3; ++a) out->size[a] = R;
    out->planet_radius = 6378137;
    for (int a = 0; a < 3; ++a) out->cell_width[a] = (20.0 / out->size[0]) * out->planet_radius;
    for (int a = 0; a < 3; ++a) out->object_center[a] = 0.0;
    for (int a = 0; a < 3; ++a)
        out->origin[a] = out->object_center[a] - out->size[a] * out->cell_width[a] / 2.0;
    out->external_b[2] = 3.07e-5;
    return 0;
}

int oracle_tracer_particles(const ipic3d_props* props, uint64_t n, uint32_t seed, ipic3d_particle* out) {
    if (!props || (n && !out)) return -1;
    const double e = kE, K = 1e7 * e, m = kMp, c = props->speed_of_light;
    const double v_mod = c / sqrt(1.0 + (m * c * c) / K);
    double low[3], hig[3];
    for (int a = 0; a < 3; ++a) {
        const double extent = props->cell_width[a] * (double)props->size[a];
        low[a] = props->origin[a] + extent / 8.0;
    }
    for (int a = 0; a < 3; ++a) hig[a] = low[a] + 0.75 * (props->cell_width[a] * (double)props->size[a]);
    const double mean[3] = {0.0, 0.0, 0.0}, sd[3] = {v_mod, v_mod, v_mod};
    oracle_generate_uniform_pos_normal_speed(low, hig, mean, sd, seed, n, out);
    for (uint64_t i = 0; i < n; ++i) {
        out[i].q = e;
        out[i].qom = e / m;
    }
    return 0;
}

int oracle_trace(const ipic3d_props* props, const ipic3d_particle* particles, uint64_t n, int32_t steps,
                 int32_t frame_interval, int32_t num_frames, uint32_t* counts) {
    if (!props || steps < 0 || frame_interval <= 0 || num_frames < 0) return -1;
    if (steps > 0 && (steps - 1) / frame_interval >= num_frames) return -1;
    Tracer g;
    int64_t cells = 1;
    for (int a = 0; a < 3; ++a) {
        g.extent[a] = props->cell_width[a] * (double)props->size[a];
        g.low[a] = props->origin[a];
        g.high[a] = props->origin[a] + g.extent[a];
        g.origin[a] = props->origin[a];
        g.w[a] = props->cell_width[a];
        g.center[a] = props->object_center[a];
        g.size[a] = props->size[a];
        cells *= props->size[a];
    }
    g.r2max = props->planet_radius * props->planet_radius;
    g.bz = props->external_b[2];
    g.R = props->planet_radius;
    g.dt = props->dt;
    g.c = props->speed_of_light;
    const int64_t total = cells * num_frames;
#pragma omp parallel
    {
        std::vector<uint32_t> local(total, 0);  // a ParticleCount per thread, summed after
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < (int64_t)n; ++i) trace_particle(particles[i], steps, g, frame_interval, local.data(), total);
#pragma omp critical
        for (int64_t k = 0; k < total; ++k) counts[k] += local[k];
    }
    return 0;
}

}  // extern "C"
