// Learned initial guess for the local rheology: a 8 -> 64 -> 64 -> 2 ReLU MLP
// in BF16 with FP32 accumulation on the tensor cores: training and batch
// inference on tcgen05 with TMEM accumulators (mlp_tc.cu; engine 0), the
// warp-level mma.sync m16n8k16 kernels as engine 1 and inside the per-node
// guess of the rheology kernels.
//
// Inputs (normalised to [-1, 1] by the training ranges): log10 of the strain
// rate invariant [1/s], T [K] (as 1000 / T), P [Pa], log10 dt [s], and a
// one-hot phase index (4 phases).  Outputs: y0 = ln(eta_ve / eta_up), the
// visco-elastic viscosity the local Newton iteration solves for, relative to
// that iteration's plain start eta_up (the smallest viscosity of the active
// mechanisms, which the local solve computes anyway), and y1 = gdot / (2 Eii),
// the plastic multiplier as a fraction of the strain rate.  Predicting the
// correction to the plain start keeps the target within a few units, where the
// BF16 network is accurate to a per cent.  The plain local Newton polishes
// every guess and stays the judge (rheology.cu).
//
// Layouts shared by every kernel: weights live in shared memory as BF16 rows
// with padded strides (24 or 72 elements: conflict-free fragment loads), in
// the packed image below, which the Adam step writes directly.
#pragma once
#include <cuda_bf16.h>
#include "mdz_internal.cuh"

#define MLP_IN 8
#define MLP_H 64
#define MLP_OUT 2
// flat FP32 parameters: W1[64][8], b1[64], W2[64][64], b2[64], W3[2][64], b3[2]
#define MLP_P_W1 0
#define MLP_P_B1 512
#define MLP_P_W2 576
#define MLP_P_B2 4672
#define MLP_P_W3 4736
#define MLP_P_B3 4864
#define MLP_NPARAM 4866
// packed image (BF16 element offsets), then FP32 biases b1[64] b2[64] b3[8]
#define MLP_S1 24
#define MLP_S2 72
#define MLP_W1S 0                        // [64][24]  W1 (cols 8..23 zero)
#define MLP_W2S 1536                     // [64][72]  W2
#define MLP_W3S 6144                     // [8][72]   W3 (rows 2..7 zero)
#define MLP_W2T 6720                     // [64][72]  W2 transposed
#define MLP_W3T 11328                    // [64][24]  W3 transposed (cols 2..23 zero)
#define MLP_NBF16 12864
#define MLP_PACK_BYTES (MLP_NBF16 * 2 + 136 * 4)

struct mdz_mlp_norm {
    float lo[4], inv[4];                 // x_k = 2 (v_k - lo_k) inv_k - 1 (k = 1: v = 1000 / T)
};

// Context-resident MLP state (mlp.cu owns it).
struct mdz_mlp {
    float *params = nullptr, *adam_m = nullptr, *adam_v = nullptr;   // MLP_NPARAM each (FP32 master)
    unsigned char *packed = nullptr;                                  // MLP_PACK_BYTES
    float *partials = nullptr;                                        // blocks x (MLP_NPARAM + 1)
    float *grad = nullptr;                                            // MLP_NPARAM + 1
    int max_blocks = 0;
    uint4 *X = nullptr;                  // dataset inputs, 8 BF16 per row
    float2 *Y = nullptr;                 // dataset labels
    long long n = 0, cap = 0;
    mdz_mlp_norm norm{};
    double lo[4] = {0, 0, 0, 0}, hi[4] = {1, 1, 1, 1};
    int adam_t = 0;
    bool has_weights = false, trained = false;
    float2 *guess = nullptr;             // n_phases x (centroids + vertices)
    size_t guess_cap = 0;
    double last_loss = 0.0;
    int engine = 0;                      // inference and training: 0 tcgen05 (mlp_tc.cu), 1 warp-level mma.sync
    int *tc_err = nullptr;               // device flag: a tcgen05 commit timed out
};

bool mdz_mlp_ready(const mdz_ctx *ctx);
// tcgen05 inference of n BF16 input rows (mlp_tc.cu); d_err is raised if a
// tensor-core commit never arrived
mdz_status mdz_mlp_infer_tc(mdz_ctx *ctx, const unsigned char *packed, const uint4 *X, long long n, float2 *Y,
                            int *d_err, cudaStream_t st);
// tcgen05 training pass over nrows rows from row0: one partial gradient row (and
// the loss) per CTA in `partials`, nblk CTAs (mlp_tc.cu)
mdz_status mdz_mlp_train_tc(mdz_ctx *ctx, const unsigned char *packed, const uint4 *X, const float2 *Y,
                            long long row0, int nrows, float scale, float *partials, int nblk, int *d_err,
                            cudaStream_t st);
void mdz_mlp_free(mdz_ctx *ctx);
// guess buffer for n_phases x (nc + nv) nodes (allocated on first use)
float2 *mdz_mlp_guess_buffer(mdz_ctx *ctx, size_t n);
mdz_status mdz_dev_viscosity_learned(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm,
                                     const mdz_fields &f, int *d_counters, cudaStream_t st, int warm = 0);

// Labelled tuples by the plain local solve (rheology.cu).
mdz_status mdz_dev_mlp_samples(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm, long long n,
                               unsigned long long seed, const double lo[4], const double hi[4],
                               const mdz_mlp_norm &norm, uint4 *X, float2 *Y, cudaStream_t st);
// Per-(phase, node) guesses for the centroids and vertices of the current state (rheology.cu).
mdz_status mdz_dev_mlp_guess(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm, const mdz_fields &f,
                             float2 *guess_n, float2 *guess_s, cudaStream_t st);

// ---------------------------------------------------------------------------
// Device helpers (header-only: used by the kernels of mlp.cu and rheology.cu).
__device__ __forceinline__ uint32_t mlp_ld32(const __nv_bfloat16 *p) {
    return *reinterpret_cast<const uint32_t *>(p);
}

__device__ __forceinline__ uint32_t mlp_pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ float mlp_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float mlp_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

// D += A B, m16n8k16, BF16 operands, FP32 accumulators
__device__ __forceinline__ void mlp_mma(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct mlp_w {   // views of the packed image in shared memory
    const __nv_bfloat16 *W1, *W2, *W3, *W2T, *W3T;
    const float *b1, *b2, *b3;
};

__device__ __forceinline__ mlp_w mlp_views(const unsigned char *smem) {
    const __nv_bfloat16 *w = reinterpret_cast<const __nv_bfloat16 *>(smem);
    const float *b = reinterpret_cast<const float *>(smem + MLP_NBF16 * 2);
    return mlp_w{w + MLP_W1S, w + MLP_W2S, w + MLP_W3S, w + MLP_W2T, w + MLP_W3T, b, b + 64, b + 128};
}

// cooperative copy of the packed image (global -> shared), all threads of the CTA
__device__ __forceinline__ void mlp_load_weights(unsigned char *smem, const unsigned char *packed) {
    const uint4 *src = reinterpret_cast<const uint4 *>(packed);
    uint4 *dst = reinterpret_cast<uint4 *>(smem);
    for (int i = threadIdx.x; i < MLP_PACK_BYTES / 16; i += blockDim.x) dst[i] = src[i];
}

// Forward pass of one 16-row tile held by a warp.  X: 16 rows of the input
// staging (stride 24 BF16, columns 8..15 zero).  Fragment layouts (PTX
// m16n8k16): lane = 4 g + t; A regs {row g, cols 2t..2t+1}, {row g+8, ...},
// {row g, cols 2t+8..}, {row g+8, cols 2t+8..}; B regs {rows 2t..2t+1, col g},
// {rows 2t+8.., col g}; C {row g, cols 2t, 2t+1}, {row g+8, ...}.  The C
// fragment of n-tiles 2kt and 2kt+1 is the A fragment of k-tile kt of the next
// layer, so hidden activations never leave registers.
__device__ __forceinline__ void mlp_tile_forward(const mlp_w &W, const __nv_bfloat16 *X, uint32_t (&h1)[4][4],
                                                 uint32_t (&h2)[4][4], float (&y)[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a[4];
    a[0] = mlp_ld32(X + g * MLP_S1 + 2 * t);
    a[1] = mlp_ld32(X + (g + 8) * MLP_S1 + 2 * t);
    a[2] = mlp_ld32(X + g * MLP_S1 + 2 * t + 8);
    a[3] = mlp_ld32(X + (g + 8) * MLP_S1 + 2 * t + 8);
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        float c[2][4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int j = 2 * kt + h;
            const float b0 = W.b1[8 * j + 2 * t], b1 = W.b1[8 * j + 2 * t + 1];
            c[h][0] = b0; c[h][1] = b1; c[h][2] = b0; c[h][3] = b1;
            const __nv_bfloat16 *wr = W.W1 + (8 * j + g) * MLP_S1 + 2 * t;
            mlp_mma(c[h], a, mlp_ld32(wr), mlp_ld32(wr + 8));
        }
        h1[kt][0] = mlp_pack2(fmaxf(c[0][0], 0.f), fmaxf(c[0][1], 0.f));
        h1[kt][1] = mlp_pack2(fmaxf(c[0][2], 0.f), fmaxf(c[0][3], 0.f));
        h1[kt][2] = mlp_pack2(fmaxf(c[1][0], 0.f), fmaxf(c[1][1], 0.f));
        h1[kt][3] = mlp_pack2(fmaxf(c[1][2], 0.f), fmaxf(c[1][3], 0.f));
    }
#pragma unroll
    for (int ko = 0; ko < 4; ko++) {
        float c[2][4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int j = 2 * ko + h;
            const float b0 = W.b2[8 * j + 2 * t], b1 = W.b2[8 * j + 2 * t + 1];
            c[h][0] = b0; c[h][1] = b1; c[h][2] = b0; c[h][3] = b1;
            const __nv_bfloat16 *wr = W.W2 + (8 * j + g) * MLP_S2 + 2 * t;
#pragma unroll
            for (int kt = 0; kt < 4; kt++) mlp_mma(c[h], h1[kt], mlp_ld32(wr + 16 * kt), mlp_ld32(wr + 16 * kt + 8));
        }
        h2[ko][0] = mlp_pack2(fmaxf(c[0][0], 0.f), fmaxf(c[0][1], 0.f));
        h2[ko][1] = mlp_pack2(fmaxf(c[0][2], 0.f), fmaxf(c[0][3], 0.f));
        h2[ko][2] = mlp_pack2(fmaxf(c[1][0], 0.f), fmaxf(c[1][1], 0.f));
        h2[ko][3] = mlp_pack2(fmaxf(c[1][2], 0.f), fmaxf(c[1][3], 0.f));
    }
    {
        const float b0 = W.b3[2 * t], b1 = W.b3[2 * t + 1];
        y[0] = b0; y[1] = b1; y[2] = b0; y[3] = b1;
        const __nv_bfloat16 *wr = W.W3 + g * MLP_S2 + 2 * t;
#pragma unroll
        for (int kt = 0; kt < 4; kt++) mlp_mma(y, h2[kt], mlp_ld32(wr + 16 * kt), mlp_ld32(wr + 16 * kt + 8));
    }
}

// Warp-level inference of 32 rows: xs = the warp's [32][24] BF16 staging (rows
// filled by the caller, columns 8..23 zero), ys = [32][2] FP32 outputs.
__device__ __forceinline__ void mlp_warp_infer(const mlp_w &W, const __nv_bfloat16 *xs, float *ys) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll 1
    for (int mt = 0; mt < 2; mt++) {
        uint32_t h1[4][4], h2[4][4];
        float y[4];
        mlp_tile_forward(W, xs + 16 * mt * MLP_S1, h1, h2, y);
        if (t == 0) {
            ys[2 * (16 * mt + g)] = y[0];
            ys[2 * (16 * mt + g) + 1] = y[1];
            ys[2 * (16 * mt + g + 8)] = y[2];
            ys[2 * (16 * mt + g + 8) + 1] = y[3];
        }
    }
}

// Normalised inputs of one (node, phase): Eii, T, P, dt in the solver's scaled
// units.  Temperature enters as 1000 / T [1/K] (the creep laws are Arrhenius
// in 1/T), normalised over the reciprocal of its range.
__device__ __forceinline__ void mlp_inputs(const mdz_mlp_norm &nm, const mdz_rheo_params &prm, double Eii, double T,
                                           double P, double dt, int phase, float *x) {
    const double v[4] = {log10(Eii * prm.scale_E), 1000.0 / (T * prm.scale_T), P * prm.scale_S,
                         log10(dt / prm.scale_E)};
#pragma unroll
    for (int k = 0; k < 4; k++) x[k] = 2.0f * ((float)v[k] - nm.lo[k]) * nm.inv[k] - 1.0f;
#pragma unroll
    for (int q = 0; q < 4; q++) x[4 + q] = q == phase ? 1.0f : 0.0f;
}

// Training labels from a converged local solve: the visco-elastic viscosity
// relative to the iteration's plain start, and the plastic fraction.
__device__ __forceinline__ float2 mlp_labels(double eta_ve, double eta_up, double gdot, double Eii) {
    return make_float2((float)log(eta_ve / eta_up), (float)(gdot / (2.0 * Eii)));
}
