// Internal declarations shared by the CUDA translation units of the library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "mdoodz_gpu.h"

#define MDZ_THREADS 256

// Device-side copy of the grid: coordinates and tags.  All arrays are owned by
// the context (cudaMalloc'd once at mdz_create).
struct mdz_dgrid {
    int Nx, Nz, ncx, ncz;
    double dx, dz, xmin, xmax, zmin, zmax;
    double *xg, *zg, *xc, *zc, *xvz, *zvx;
    signed char *BCu, *BCv, *BCp, *BCg;
    double *BCu_val, *BCv_val;
};

// Marker store: structure of arrays, FP64 positions, int32 phases.
struct mdz_markers {
    int n = 0;
    long long cap = 0;
    double *x = nullptr, *z = nullptr, *vx = nullptr, *vz = nullptr;
    int *phase = nullptr;
};

// Cell binning of the resident markers: markers sorted by cell (stable).
struct mdz_bins {
    bool valid = false;
    int ncells = 0;
    int *cell = nullptr;        // per marker: cell index or -1 (inactive)
    int *count = nullptr;       // per cell
    int *start = nullptr;       // per cell + 1: exclusive scan of count
    int *cursor = nullptr;      // scratch for the scatter
    int *sorted = nullptr;      // marker indices grouped by cell, ascending inside a cell
    int *scan_partials = nullptr;
};

struct mdz_ctx {
    mdz_grid_desc host_desc{};
    mdz_dgrid g{};
    int n_phases = 0;
    mdz_markers m;
    mdz_bins bins;
    cudaStream_t stream = nullptr;
    long long launches = 0;
    std::string err;
    // host-call staging buffers (grown on demand)
    void *stage[8] = {nullptr};
    size_t stage_bytes[8] = {0};
};

// ---- helpers -------------------------------------------------------------
mdz_status mdz_fail(mdz_ctx *ctx, mdz_status s, const char *fmt, ...);
mdz_status mdz_cuda_check(mdz_ctx *ctx, cudaError_t e, const char *what);
// Device staging buffer slot i with at least `bytes` bytes.
void *mdz_stage(mdz_ctx *ctx, int slot, size_t bytes);

#define MDZ_CUDA(ctx, call)                                                          \
    do {                                                                              \
        cudaError_t e__ = (call);                                                     \
        if (e__ != cudaSuccess) return mdz_cuda_check((ctx), e__, #call);             \
    } while (0)

#define MDZ_LAUNCHED(ctx)                                                            \
    do {                                                                              \
        (ctx)->launches++;                                                            \
        cudaError_t e__ = cudaGetLastError();                                         \
        if (e__ != cudaSuccess) return mdz_cuda_check((ctx), e__, "kernel launch");   \
    } while (0)

static inline int mdz_blocks(long long n, int threads = MDZ_THREADS) {
    long long b = (n + threads - 1) / threads;
    return (int)(b < 1 ? 1 : b);
}

// Node-set geometry: sizes and coordinate lines of a node set.
struct mdz_nodeset {
    int nx, nz;               // nodes per direction
    const double *X, *Z;      // coordinate lines (device)
    const signed char *tag;   // tags (device)
};
mdz_nodeset mdz_get_nodeset(const mdz_ctx *ctx, int centroid);

// Binning (markers.cu)
mdz_status mdz_ensure_bins(mdz_ctx *ctx, cudaStream_t st);
