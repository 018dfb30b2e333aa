// Device-side upload kernels (upload.cu): species classification, per-cell
// counts and the scatter of AoS particles into the slot layout.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ipg {

constexpr int kUploadMaxPops = 16;

struct SpeciesTable {
    int n;
    double q[kUploadMaxPops], qom[kUploadMaxPops];
};

struct UploadGeom {
    int ncells, sx, sy, sz;
    double origin[3], w[3];
};

template <typename T>
struct UploadPops {
    int npop;
    int relative;  // store cell-relative positions (FP32 layout)
    T* x[kUploadMaxPops];
    T* y[kUploadMaxPops];
    T* z[kUploadMaxPops];
    T* u[kUploadMaxPops];
    T* v[kUploadMaxPops];
    T* w[kUploadMaxPops];
    uint32_t* id[kUploadMaxPops];
    const int64_t* start[kUploadMaxPops];
    int32_t* count[kUploadMaxPops];
};

int launch_classify(const void* parts, int64_t n, const SpeciesTable& sp, uint8_t* sid, int* unknown,
                    cudaStream_t st);
int launch_count(const uint8_t* sid, const int64_t* in_off, int ncells, int npop, int32_t* counts, cudaStream_t st);
template <typename T>
int launch_scatter(const void* parts, const uint32_t* ids, const uint8_t* sid, const int64_t* in_off,
                   const UploadPops<T>& U, const UploadGeom& g, cudaStream_t st);

}  // namespace ipg
