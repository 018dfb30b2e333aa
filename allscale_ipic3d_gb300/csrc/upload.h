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

// Deposit of the uploaded particles (FP32 contexts): the node sums of J and
// rho (raw, before the periodic fold and the normalisation).
struct UploadDeposit {
    int on;
    int sx, sy, sz;  // cells per axis (nodes (s+1)^3)
    double* J;
    double* rho;
};

int launch_classify(const void* parts, int64_t n, const SpeciesTable& sp, uint8_t* sid, int* unknown,
                    cudaStream_t st);
// One pass for cells [c0, c1): classification, scatter into the existing
// slot layout, per-cell counts, and (dep.on) the cloud-in-cell deposit.
// flags[0] = a particle of an unknown species, flags[1] = a cell's slots
// were too few (the caller then re-lays out).
template <typename T>
int launch_upload_cells(const void* parts, const uint32_t* ids, const int64_t* in_off, int c0, int c1,
                        const SpeciesTable& sp, const UploadPops<T>& U, const UploadGeom& g, const UploadDeposit& dep,
                        int* flags, cudaStream_t st);
int launch_count(const uint8_t* sid, const int64_t* in_off, int ncells, int npop, int32_t* counts, cudaStream_t st);

// Download: the populations' particles as the reference's AoS records
// (Particle, particle.h:9-60), the i-th particle of cell c of population k at
// output index dst[k][c] + i; cell-relative FP32 positions are made absolute
// with the host's formula (origin + cx w) + x w in FP64.
template <typename T>
struct PackPops {
    int npop;
    int relative;
    const T* x[kUploadMaxPops];
    const T* y[kUploadMaxPops];
    const T* z[kUploadMaxPops];
    const T* u[kUploadMaxPops];
    const T* v[kUploadMaxPops];
    const T* w[kUploadMaxPops];
    const uint32_t* id[kUploadMaxPops];
    const int64_t* start[kUploadMaxPops];
    const int32_t* count[kUploadMaxPops];
    const int64_t* dst;  // [npop][ncells]
    double q[kUploadMaxPops], qom[kUploadMaxPops];
    int positions_only;  // write the three position doubles of each particle (24 bytes), not its record
};
// Cells [c0, c1): one warp per cell; `out` (records) and `out_ids` (may be
// null) are device buffers indexed by the output index.
template <typename T>
int launch_pack_cells(const PackPops<T>& P, const UploadGeom& g, int c0, int c1, void* out, uint32_t* out_ids,
                      cudaStream_t st);
template <typename T>
int launch_scatter(const void* parts, const uint32_t* ids, const uint8_t* sid, const int64_t* in_off,
                   const UploadPops<T>& U, const UploadGeom& g, cudaStream_t st);

}  // namespace ipg
