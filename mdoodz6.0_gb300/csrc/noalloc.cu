// Residual norms of the decoupled Stokes rows without any allocation: the
// norms EvaluateStokesResidualDecoupled reports (resx, resz, resp =
// sqrt(sum F^2 / count) over the x-momentum, z-momentum and continuity
// equations), computed from caller-owned device buffers with a file-scope
// static scratch array instead of context memory.
//
// Scratch: one slot of 6 doubles (three sums of squares, three counts) per row
// of the index box, i.e. Nz + 1 slots.  Pass 1 writes every slot of the call's
// rows (one CTA per row), pass 2 (one CTA) sums the slots in row order, so no
// scratch value has to start at zero and the result is bitwise reproducible.
// The scratch is shared by all calls on a device: calls that overlap in time
// (different streams, host threads) race on it and must be serialised.
#include <cmath>
#include "mdz_internal.cuh"

#define NOALLOC_MAX_ROWS 8192                    // index-box rows (Nz + 1) the scratch holds
static __device__ __align__(256) double g_noalloc_rows[NOALLOC_MAX_ROWS * 6];   // 384 KiB

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// one CTA per index-box row j in 0..Nz: Vx row j, Vz row j (j < Nz), centroid row j (j < Nz-1)
__global__ void __launch_bounds__(256) k_noalloc_rows(int Nx, int Nz, const double *__restrict__ ru,
                                                      const double *__restrict__ rv, const double *__restrict__ rp,
                                                      const signed char *__restrict__ tu,
                                                      const signed char *__restrict__ tv,
                                                      const signed char *__restrict__ tp, double *rows) {
    const int j = blockIdx.x;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i <= Nx; i += blockDim.x) {
        if (i < Nx) {
            const int c = i + j * Nx;
            if (tu[c] == -1) { acc[0] += ru[c] * ru[c]; acc[3] += 1.0; }
        }
        if (j < Nz) {
            const int c = i + j * (Nx + 1);
            if (tv[c] == -1) { acc[1] += rv[c] * rv[c]; acc[4] += 1.0; }
        }
        if (j < Nz - 1 && i < Nx - 1) {
            const int c = i + j * (Nx - 1);
            if (tp[c] == -1) { acc[2] += rp[c] * rp[c]; acc[5] += 1.0; }
        }
    }
    __shared__ double sh[6][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < 6; q++) {
        const double s = warp_sum_d(acc[q]);
        if (lane == 0) sh[q][w] = s;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[threadIdx.x][k];
        rows[(size_t)j * 6 + threadIdx.x] = s;
    }
}

// one CTA: fixed-order sum over the rows, then the norms
__global__ void __launch_bounds__(256) k_noalloc_norms(int nrows, const double *__restrict__ rows,
                                                       double *__restrict__ out3) {
    __shared__ double sh[6][256];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int r = threadIdx.x; r < nrows; r += blockDim.x)
        for (int q = 0; q < 6; q++) acc[q] += rows[(size_t)r * 6 + q];
    for (int q = 0; q < 6; q++) sh[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int q = 0; q < 6; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 3) {
        const double cnt = sh[threadIdx.x + 3][0];
        out3[threadIdx.x] = sqrt(sh[threadIdx.x][0] / (cnt > 0 ? cnt : 1.0));
    }
}

// Scratch address per device, looked up once with that device current (kept
// for the process: stale after the device's primary context is torn down).
static double *g_noalloc_ptr[64];

extern "C" mdz_status mdz_dev_residual_norms_noalloc(int Nx, int Nz, const double *ru, const double *rv,
                                                     const double *rp, const signed char *BCu,
                                                     const signed char *BCv, const signed char *BCp,
                                                     double *norms3, void *stream) {
    if (Nx < 3 || Nz < 3 || !ru || !rv || !rp || !BCu || !BCv || !BCp || !norms3) return MDZ_ERR_ARG;
    if (Nz + 1 > NOALLOC_MAX_ROWS) return MDZ_ERR_CAPACITY;   // scratch holds NOALLOC_MAX_ROWS index-box rows
    if ((long long)(Nx + 1) * (Nz + 1) > 2147483647LL) return MDZ_ERR_CAPACITY;   // the kernels' 32-bit indices
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MDZ_ERR_CUDA;
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_rows) != cudaSuccess || !p) return MDZ_ERR_CUDA;
        g_noalloc_ptr[dev] = (double *)p;
    }
    cudaStream_t st = (cudaStream_t)stream;
    k_noalloc_rows<<<Nz + 1, 256, 0, st>>>(Nx, Nz, ru, rv, rp, BCu, BCv, BCp, g_noalloc_ptr[dev]);
    if (cudaGetLastError() != cudaSuccess) return MDZ_ERR_CUDA;
    k_noalloc_norms<<<1, 256, 0, st>>>(Nz + 1, g_noalloc_ptr[dev], norms3);
    if (cudaGetLastError() != cudaSuccess) return MDZ_ERR_CUDA;
    return MDZ_OK;
}
