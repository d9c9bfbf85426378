// Deterministic grid-wide sums.
//
// Every block reduces its values in a fixed order (warp shuffles, then the
// warp sums in warp order) and writes one partial per value to a slot of its
// own; the block that arrives last (a device-scope counter) adds the partials
// up in block order and resets the counter for the next launch.  No
// floating-point atomics: the same inputs give the same bits on every run, so
// convergence tests (Krylov residuals, non-linear residual norms, pressure
// means) decide the same way run after run.
#pragma once
#include <cuda_runtime.h>

// reduction workspace of a context: partial slots and arrival counters
#define MDZ_RED_PART 131072
#define MDZ_RED_COUNTERS 128
// counter and partial-slot assignment (partial offsets in doubles)
enum {
    MDZ_RC_NORMS = 0,     // residual norms, 6 values
    MDZ_RC_PSUM = 1,      // pressure sum and count
    MDZ_RC_PRECP = 2,     // preconditioner pressure block sum and count
    MDZ_RC_DOTS = 8,      // k_dots: one counter per tile row (up to 40)
    MDZ_RC_GCR = 64,      // k_gcr_dots: [0] across tile rows, [1 + y] per tile row (up to 40)
    MDZ_RC_ENERGY = 112,  // energy-equation conjugate gradients: 3 counters
};
enum {
    MDZ_RP_NORMS = 0,         // 6 x 2048
    MDZ_RP_PSUM = 12288,      // 2 x 2048
    MDZ_RP_PRECP = 16384,     // 2 x 2048
    MDZ_RP_DOTS = 20480,      // up to 48 x 2048
    MDZ_RP_ENERGY = 118784,   // 3 x 2048 (energy-equation conjugate gradients)
};

template <typename T>
__device__ __forceinline__ T mdz_warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum of NV values over the block in a fixed order: warp sums in T (FP32
// vectors keep their sums FP32 inside a warp: FP64 instructions issue at a
// small fraction of the FP32 rate on this part), then the warp sums in FP64
// in warp order.  The result is valid in warp 0, lane 0.
// sh: 32 x NV doubles of shared memory.
template <int NV, typename T>
__device__ __forceinline__ void mdz_block_sum(const T (&v)[NV], double (&out)[NV], double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
        T s = mdz_warp_sum(v[q]);
        if (lane == 0) sh[q * 32 + wid] = (double)s;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) out[q] = mdz_warp_sum(lane < nw ? sh[q * 32 + lane] : 0.0);
    }
}

// Called by every thread of every block after its partials are written:
// true in all threads of the block that arrives last (of `total`).
__device__ __forceinline__ bool mdz_arrive_last(unsigned int *counter, unsigned int total) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        last = atomicAdd(counter, 1u) == total - 1;
        if (last) *counter = 0u;   // for the next launch (stream order)
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// In the last block: out[q] = sum over b < nb of part[q * nb + b], q < nq,
// in a fixed order (warp w takes q = w, w + nw, ...; lane l the blocks
// l, l + 32, ... in order, then a shuffle tree).  Partials are read through
// L2 (other blocks wrote them).
__device__ __forceinline__ void mdz_sum_partials(const double *part, int nb, int nq, double *out) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    for (int q = wid; q < nq; q += nw) {
        const double *p = part + (size_t)q * nb;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        int b = lane;
        for (; b + 96 < nb; b += 128) {
            a0 += __ldcg(p + b);
            a1 += __ldcg(p + b + 32);
            a2 += __ldcg(p + b + 64);
            a3 += __ldcg(p + b + 96);
        }
        for (; b < nb; b += 32) a0 += __ldcg(p + b);
        double s = mdz_warp_sum<double>((a0 + a1) + (a2 + a3));
        if (lane == 0) out[q] = s;
    }
}

// One-launch deterministic sum of NV per-thread values over the whole grid
// (1-D grid): out[q] = sum; true in the block that wrote out.  part: NV x
// gridDim.x slots.
template <int NV, typename T>
__device__ __forceinline__ bool mdz_grid_sum(const T (&v)[NV], double *part, unsigned int *counter, double *out) {
    __shared__ double sh[32 * NV];
    double b[NV];
    mdz_block_sum<NV, T>(v, b, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) part[(size_t)q * gridDim.x + blockIdx.x] = b[q];
    }
    if (!mdz_arrive_last(counter, gridDim.x)) return false;
    mdz_sum_partials(part, gridDim.x, NV, out);
    return true;
}
