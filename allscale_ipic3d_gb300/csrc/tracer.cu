// The standalone particle tracer of the reference (pic_tracer.cxx): every
// particle is followed independently through the analytic Earth dipole
// (traceParticle, pic_tracer.cxx:77-148) and counted, every `frame_interval`
// steps, into a per-frame histogram over the grid cells (ParticleCount,
// pic_tracer.cxx:26-71).
//
// One thread per particle keeps its state in registers for all steps; the
// only memory traffic is the 64-byte particle record read once and one
// atomic increment per recorded frame into the histogram (L2-resident for
// the reference's 64^3 grid). The work is FP64 arithmetic, term by term in
// the reference's order (built with -fmad=false): r^2.5 correctly rounded,
// the sub-cycle rule, the Boris rotation and the periodic wrap are those of
// the reference, so trajectories and counts match its host build.
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/ipic3d_gpu.h"
#include "launch.h"
#include "particle_kernels.cuh"

namespace ipg {
namespace {

constexpr int kTraceThreads = 128;

struct TraceArgs {
    double low[3], high[3];  // universe box: origin .. origin + width * size
    double extent[3];        // width * size (the wrap distance)
    double w[3];             // cell width (getCellCoordinates)
    double center[3];        // objectCenter
    int center_zero;         // objectCenter == 0: the planet test's r^2 is the next step's field r^2
    int int_cmp;             // box and planet radius finite: comparisons on bit patterns
    long long key_low[3], key_high[3];  // order_key of low, high
    double r2max;            // planetRadius^2
    double mft;              // -Bext.z * pow(planetRadius, 3), host libm
    double dt, c;
    double inv_pic;          // 1 / (pi c), for the sub-cycle estimate
    int64_t size[3];
    int32_t steps, interval;
    int64_t total;           // entries of counts: frames * cells
    const ipic3d_particle* in;
    uint64_t n;
    uint32_t* counts;
};

// An integer that orders finite and infinite doubles as their values do
// (+0 and -0 both map to 0); NaN is tested apart. The comparisons of the
// step loop run on these keys, in the integer pipe, which the FP64-bound
// loop leaves idle.
__device__ __forceinline__ long long order_key(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : -(b & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool is_nan_bits(double x) {
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}

__device__ __forceinline__ double sum_sq(double a, double b, double c) {
    double r = a * a;  // allscale::utils::sumOfSquares: 0 + a^2 + b^2 + c^2 (0 + a^2 == a^2)
    r += b * b;
    r += c * c;
    return r;
}

__global__ void __launch_bounds__(kTraceThreads) k_trace(const TraceArgs A) {
    const uint64_t i = (uint64_t)blockIdx.x * kTraceThreads + threadIdx.x;
    if (i >= A.n) return;
    const double2* src = reinterpret_cast<const double2*>(A.in + i);
    const double2 r0 = __ldg(src), r1 = __ldg(src + 1), r2 = __ldg(src + 2), r3 = __ldg(src + 3);
    // p.position += objectCenter
    double P[3] = {r0.x + A.center[0], r0.y + A.center[1], r1.x + A.center[2]};
    double u = r1.y, v = r2.x, w = r2.y;
    const double qom = r3.y;
    // particles generated inside the planet or outside the universe are skipped
    if (sum_sq(P[0] - A.center[0], P[1] - A.center[1], P[2] - A.center[2]) < A.r2max) return;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (P[a] > A.high[a] || P[a] < A.low[a]) return;

    int64_t next_record = 0, frame = 0;
    double rf2 = sum_sq(P[0], P[1], P[2]);  // |position|^2 of the field
    for (int t = 0; t < A.steps; ++t) {
        const bool record = t == next_record;  // t % frame_interval == 0
        int64_t cx = 0, cy = 0, cz = 0;
        if (record) {  // getCellCoordinates (cell.h:64-67) before the move
            cx = (int64_t)((P[0] - A.low[0]) / A.w[0]);
            cy = (int64_t)((P[1] - A.low[1]) / A.w[1]);
            cz = (int64_t)((P[2] - A.low[2]) / A.w[2]);
        }
        // dipole B at the absolute position, E = 0 (pic_tracer.cxx:104-111)
        const double x = P[0], y = P[1], z = P[2];
        const double fac1 = A.mft / pow25_rn(rf2);
        const double bx = 3.0 * x * z * fac1;
        const double by = 3.0 * y * z * fac1;
        const double bz = (2.0 * (z * z) - (x * x) - (y * y)) * fac1;
        // adaptive sub-cycling (pic_tracer.cxx:113-118)
        double dts;
        const int ns = sub_cycles_dt(A.dt, A.c, A.inv_pic, qom, sum_sq(bx, by, bz), dts);
        for (int s = 0; s < ns; ++s) {
            boris_e0(u, v, w, bx, by, bz, qom, dts);  // updateVelocity (particle.h:31-49)
            P[0] = P[0] + u * dts;                    // updatePosition (particle.h:24-26)
            P[1] = P[1] + v * dts;
            P[2] = P[2] + w * dts;
        }
        // periodic wrap (pic_tracer.cxx:129-133)
        if (A.int_cmp) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const bool nan = is_nan_bits(P[a]);  // NaN compares false both ways
                long long k = order_key(P[a]);
                if (!nan && k > A.key_high[a]) {
                    P[a] = P[a] - A.extent[a];
                    k = order_key(P[a]);
                }
                if (!nan && k < A.key_low[a]) P[a] = P[a] + A.extent[a];
            }
        } else {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (P[a] > A.high[a]) P[a] = P[a] - A.extent[a];
                if (P[a] < A.low[a]) P[a] = P[a] + A.extent[a];
            }
        }
        // tracing stops inside the planet (pic_tracer.cxx:135-141); with the
        // object at the origin, p - center is p itself, so the test's r^2 is
        // the one the next step's field needs
        rf2 = sum_sq(P[0], P[1], P[2]);
        const double rp2 =
            A.center_zero ? rf2 : sum_sq(P[0] - A.center[0], P[1] - A.center[1], P[2] - A.center[2]);
        // rp2 is >= 0 or NaN and r2max finite >= 0: their bit patterns
        // without the sign order as the values (a NaN of either sign lies
        // above everything, so "<=" fails as in FP64)
        if (A.int_cmp ? (__double_as_longlong(rp2) & 0x7fffffffffffffffLL) <= __double_as_longlong(A.r2max)
                      : rp2 <= A.r2max)
            break;
        if (record) {
            // ParticleCount::increment(t / frame_interval, pos): the flat
            // index of its row-major vector, coordinates cast to int
            const int64_t idx = ((frame * A.size[0] + (int)cx) * A.size[1] + (int)cy) * A.size[2] + (int)cz;
            if (idx >= 0 && idx < A.total) atomicAdd(A.counts + idx, 1u);
            ++frame;
            next_record += A.interval;
        }
    }
}

int tr_fail(int status, const char* msg) { return set_last_error(status, msg); }

// Validates the arguments and fills the kernel's constants.
int trace_args(const ipic3d_props* props, uint64_t n, int32_t steps, int32_t frame_interval, int32_t num_frames,
               TraceArgs& A) {
    if (!props) return tr_fail(IPIC3D_E_INVALID, "ipic3d_gpu_trace: NULL props");
    if (steps < 0 || frame_interval <= 0 || num_frames < 0)
        return tr_fail(IPIC3D_E_INVALID, "ipic3d_gpu_trace: steps >= 0, frame_interval > 0, num_frames >= 0");
    if (steps > 0 && (steps - 1) / frame_interval >= num_frames)
        return tr_fail(IPIC3D_E_INVALID, "ipic3d_gpu_trace: num_frames must exceed (steps - 1) / frame_interval");
    int64_t cells = 1;
    for (int a = 0; a < 3; ++a) {
        if (props->size[a] <= 0 || props->size[a] > (1 << 20) || !(props->cell_width[a] > 0))
            return tr_fail(IPIC3D_E_INVALID, "ipic3d_gpu_trace: bad grid");
        cells *= props->size[a];
    }
    if (cells > ((int64_t)1 << 40) / (num_frames > 0 ? num_frames : 1))
        return tr_fail(IPIC3D_E_INVALID, "ipic3d_gpu_trace: histogram too large");
    for (int a = 0; a < 3; ++a) {
        A.extent[a] = props->cell_width[a] * (double)props->size[a];  // elementwiseProduct(cellWidth, size)
        A.low[a] = props->origin[a];
        A.high[a] = props->origin[a] + A.extent[a];
        A.w[a] = props->cell_width[a];
        A.center[a] = props->object_center[a];
        A.size[a] = props->size[a];
    }
    A.center_zero = props->object_center[0] == 0.0 && props->object_center[1] == 0.0 && props->object_center[2] == 0.0;
    A.r2max = props->planet_radius * props->planet_radius;
    A.int_cmp = std::isfinite(A.r2max) && A.r2max >= 0.0;
    for (int a = 0; a < 3; ++a) {
        A.int_cmp = A.int_cmp && std::isfinite(A.low[a]) && std::isfinite(A.high[a]);
        // order_key on the host: the same mapping
        long long bl, bh;
        std::memcpy(&bl, &A.low[a], 8);
        std::memcpy(&bh, &A.high[a], 8);
        A.key_low[a] = bl >= 0 ? bl : -(bl & 0x7fffffffffffffffLL);
        A.key_high[a] = bh >= 0 ? bh : -(bh & 0x7fffffffffffffffLL);
    }
    A.mft = -props->external_b[2] * std::pow(props->planet_radius, 3);
    A.dt = props->dt;
    A.c = props->speed_of_light;
    A.inv_pic = 1.0 / (3.14159265358979323846 * props->speed_of_light);
    A.steps = steps;
    A.interval = frame_interval;
    A.total = cells * num_frames;
    A.n = n;
    return IPIC3D_OK;
}

int launch_trace(const TraceArgs& A, cudaStream_t st) {
    if (A.n == 0 || A.steps == 0) return IPIC3D_OK;
    const uint64_t blocks = (A.n + kTraceThreads - 1) / kTraceThreads;
    if (blocks > 0x7fffffffull) return tr_fail(IPIC3D_E_INVALID, "ipic3d_gpu_trace: too many particles");
    k_trace<<<(unsigned)blocks, kTraceThreads, 0, st>>>(A);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? IPIC3D_OK : tr_fail(IPIC3D_E_CUDA, cudaGetErrorString(e));
}

// Device buffers and stream of the host-pointer entry point, grown on
// demand and kept for the next call (one set per process, calls serialised).
struct TraceBuffers {
    std::mutex mu;
    int dev = -1;
    cudaStream_t st = nullptr;
    ipic3d_particle* particles = nullptr;
    uint64_t particles_cap = 0;
    uint32_t* counts = nullptr;
    int64_t counts_cap = 0;
};
TraceBuffers g_tb;

int check_device(int& dev) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return tr_fail(IPIC3D_E_NODEVICE, "no CUDA device");
    if (cudaGetDevice(&dev) != cudaSuccess) return tr_fail(IPIC3D_E_NODEVICE, "no current CUDA device");
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (!(major == 10 && minor == 3))
        return tr_fail(IPIC3D_E_NODEVICE, "the current device is not sm_103; this library is built for sm_103a only");
    return IPIC3D_OK;
}

#define TR_CU(call)                                                                                          \
    do {                                                                                                     \
        const cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                               \
            return tr_fail(e_ == cudaErrorMemoryAllocation ? IPIC3D_E_NOMEM : IPIC3D_E_CUDA,                 \
                           cudaGetErrorString(e_));                                                          \
    } while (0)

}  // namespace
}  // namespace ipg

extern "C" {

int ipic3d_gpu_trace(const ipic3d_props* props, const ipic3d_particle* particles, uint64_t n, int32_t steps,
                     int32_t frame_interval, int32_t num_frames, uint32_t* counts) {
    using namespace ipg;
    TraceArgs A;
    int rc = trace_args(props, n, steps, frame_interval, num_frames, A);
    if (rc != IPIC3D_OK) return rc;
    if ((n && !particles) || (A.total && !counts)) return tr_fail(IPIC3D_E_INVALID, "ipic3d_gpu_trace: NULL buffer");
    if (n == 0 || steps == 0 || A.total == 0) return IPIC3D_OK;
    int dev = 0;
    if ((rc = check_device(dev)) != IPIC3D_OK) return rc;
    std::lock_guard<std::mutex> lock(g_tb.mu);
    if (g_tb.dev != dev) {  // first call, or another current device: start over
        if (g_tb.dev >= 0) {  // release the other device's buffers and stream on that device
            if (cudaSetDevice(g_tb.dev) == cudaSuccess) {
                if (g_tb.particles) cudaFree(g_tb.particles);
                if (g_tb.counts) cudaFree(g_tb.counts);
                if (g_tb.st) cudaStreamDestroy(g_tb.st);
            }
            TR_CU(cudaSetDevice(dev));
            g_tb.dev = -1;
        }
        g_tb.particles = nullptr;
        g_tb.particles_cap = 0;
        g_tb.counts = nullptr;
        g_tb.counts_cap = 0;
        g_tb.st = nullptr;
        TR_CU(cudaStreamCreateWithFlags(&g_tb.st, cudaStreamNonBlocking));
        g_tb.dev = dev;
    }
    if (g_tb.particles_cap < n) {
        if (g_tb.particles) cudaFree(g_tb.particles);
        g_tb.particles = nullptr;
        g_tb.particles_cap = 0;
        TR_CU(cudaMalloc(&g_tb.particles, n * sizeof(ipic3d_particle)));
        g_tb.particles_cap = n;
    }
    if (g_tb.counts_cap < A.total) {
        if (g_tb.counts) cudaFree(g_tb.counts);
        g_tb.counts = nullptr;
        g_tb.counts_cap = 0;
        TR_CU(cudaMalloc(&g_tb.counts, (size_t)A.total * sizeof(uint32_t)));
        g_tb.counts_cap = A.total;
    }
    cudaStream_t st = g_tb.st;
    // the histogram accumulates (res += ..., pic_tracer.cxx:282): in, add, out
    TR_CU(cudaMemcpyAsync(g_tb.counts, counts, (size_t)A.total * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    TR_CU(cudaMemcpyAsync(g_tb.particles, particles, n * sizeof(ipic3d_particle), cudaMemcpyHostToDevice, st));
    A.in = g_tb.particles;
    A.counts = g_tb.counts;
    if ((rc = launch_trace(A, st)) != IPIC3D_OK) return rc;
    TR_CU(cudaMemcpyAsync(counts, g_tb.counts, (size_t)A.total * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    TR_CU(cudaStreamSynchronize(st));
    return IPIC3D_OK;
}

int ipic3d_gpu_trace_device(const ipic3d_props* props, const ipic3d_particle* d_particles, uint64_t n,
                            int32_t steps, int32_t frame_interval, int32_t num_frames, uint32_t* d_counts,
                            void* stream) {
    using namespace ipg;
    TraceArgs A;
    int rc = trace_args(props, n, steps, frame_interval, num_frames, A);
    if (rc != IPIC3D_OK) return rc;
    if ((n && !d_particles) || (A.total && !d_counts))
        return tr_fail(IPIC3D_E_INVALID, "ipic3d_gpu_trace_device: NULL buffer");
    if ((reinterpret_cast<uintptr_t>(d_particles) & 15) != 0)
        return tr_fail(IPIC3D_E_INVALID, "ipic3d_gpu_trace_device: particles must be 16-byte aligned");
    if (n == 0 || steps == 0 || A.total == 0) return IPIC3D_OK;
    A.in = d_particles;
    A.counts = d_counts;
    return launch_trace(A, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
