// Learned local-rheology guess: state, the warp-level BF16 tensor-core training
// (fused forward + backward + weight gradients per 128-row tile) and inference
// kernels (engine 1; the tcgen05 kernels of engine 0 are in mlp_tc.cu), the
// deterministic reduction with the Adam step, and the C entry points.  None of this
// has a counterpart in the reference, whose local Newton iteration
// (SOURCE/RheologyDensity.c:44-707) always starts from the smallest viscosity of
// the active creep mechanisms; the plain solve here keeps that start and remains
// the fall-back.
#include <cmath>
#include <cstring>
#include <vector>
#include "mlp.cuh"

#define MLP_RS 136            // row stride of the transposed 128-row activation tiles
#define MLP_TILE 128          // rows per CTA tile in training (4 warps x 32)

static size_t train_smem_bytes() {
    return MLP_PACK_BYTES + (size_t)(16 + 64 * 4 + 16) * MLP_RS * 2 + 4 * 32 * MLP_S1 * 2 + MLP_TILE * 2 * 4 +
           4 * 136 * 4;
}
static size_t infer_smem_bytes() { return MLP_PACK_BYTES + 8 * 32 * MLP_S1 * 2 + 8 * 64 * 4; }

// ---------------------------------------------------------------------------
// Packed image writes (one parameter)
__device__ __forceinline__ void mlp_write_packed(unsigned char *packed, int p, float w) {
    __nv_bfloat16 *pb = reinterpret_cast<__nv_bfloat16 *>(packed);
    float *bias = reinterpret_cast<float *>(packed + MLP_NBF16 * 2);
    const __nv_bfloat16 h = __float2bfloat16_rn(w);
    if (p < MLP_P_B1) {
        int o = p / 8, i = p % 8;
        pb[MLP_W1S + o * MLP_S1 + i] = h;
    } else if (p < MLP_P_W2) {
        bias[p - MLP_P_B1] = w;
    } else if (p < MLP_P_B2) {
        int q = p - MLP_P_W2, o = q / 64, i = q % 64;
        pb[MLP_W2S + o * MLP_S2 + i] = h;
        pb[MLP_W2T + i * MLP_S2 + o] = h;
    } else if (p < MLP_P_W3) {
        bias[64 + p - MLP_P_B2] = w;
    } else if (p < MLP_P_B3) {
        int q = p - MLP_P_W3, o = q / 64, i = q % 64;
        pb[MLP_W3S + o * MLP_S2 + i] = h;
        pb[MLP_W3T + i * MLP_S1 + o] = h;
    } else if (p < MLP_NPARAM) {
        bias[128 + p - MLP_P_B3] = w;
    }
}

__global__ void k_mlp_pack(const float *__restrict__ params, unsigned char *packed) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < MLP_NPARAM) mlp_write_packed(packed, p, params[p]);
}

// ---------------------------------------------------------------------------
// Training: one CTA of 4 warps per 128-row tile (grid-stride over tiles).  Each
// warp runs forward and backward for its 32 rows in registers (two m16 tiles),
// stages activations and deltas transposed in shared memory, and the CTA then
// forms the weight gradients of the tile as tensor-core products over the 128
// rows (44 output tiles of 16 x 8, 11 per warp), accumulated in registers
// across the CTA's tiles.  Each CTA writes one partial gradient; the reduction
// kernel sums the partials in a fixed order (bitwise reproducible).
__device__ __forceinline__ void mlp_store_T(__nv_bfloat16 *dst, const uint32_t (&fr)[4][4], int rbase) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        const int c0 = 16 * kt + 2 * t;
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int col = c0 + ((r & 2) ? 8 : 0), row = rbase + g + ((r & 1) ? 8 : 0);
            const uint32_t v = fr[kt][r];
            dst[col * MLP_RS + row] = __ushort_as_bfloat16((unsigned short)(v & 0xffffu));
            dst[(col + 1) * MLP_RS + row] = __ushort_as_bfloat16((unsigned short)(v >> 16));
        }
    }
}

// delta of a hidden layer: C fragment of n-tile j masked by the ReLU of the
// matching activation fragment, packed into the A fragment d, bias sums added
__device__ __forceinline__ void mlp_mask(const float (&c)[4], const uint32_t (&act)[4][4], int j,
                                         uint32_t (&d)[4][4], float (&db)[8][2]) {
    const uint32_t a0 = act[j >> 1][(j & 1) ? 2 : 0], a1 = act[j >> 1][(j & 1) ? 3 : 1];
    const float c0 = mlp_lo(a0) > 0.f ? c[0] : 0.f, c1 = mlp_hi(a0) > 0.f ? c[1] : 0.f;
    const float c2 = mlp_lo(a1) > 0.f ? c[2] : 0.f, c3 = mlp_hi(a1) > 0.f ? c[3] : 0.f;
    d[j >> 1][(j & 1) ? 2 : 0] = mlp_pack2(c0, c1);
    d[j >> 1][(j & 1) ? 3 : 1] = mlp_pack2(c2, c3);
    db[j][0] += c0 + c2;
    db[j][1] += c1 + c3;
}

__global__ void __launch_bounds__(128) k_mlp_train(const unsigned char *__restrict__ packed,
                                                   const uint4 *__restrict__ X, const float2 *__restrict__ Y,
                                                   long long row0, int nrows, float scale, float *__restrict__ partials) {
    extern __shared__ __align__(16) unsigned char sm[];
    __nv_bfloat16 *XT = reinterpret_cast<__nv_bfloat16 *>(sm + MLP_PACK_BYTES);
    __nv_bfloat16 *H1T = XT + 16 * MLP_RS, *H2T = H1T + 64 * MLP_RS, *D1T = H2T + 64 * MLP_RS;
    __nv_bfloat16 *D2T = D1T + 64 * MLP_RS, *DYT = D2T + 64 * MLP_RS, *XR = DYT + 16 * MLP_RS;
    float *LAB = reinterpret_cast<float *>(XR + 4 * 32 * MLP_S1), *BACC = LAB + 2 * MLP_TILE;
    mlp_load_weights(sm, packed);
    for (int i = threadIdx.x; i < 16 * MLP_RS; i += blockDim.x) { XT[i] = __float2bfloat16_rn(0.f); DYT[i] = XT[i]; }
    for (int i = threadIdx.x; i < 4 * 32 * MLP_S1; i += blockDim.x) XR[i] = __float2bfloat16_rn(0.f);
    for (int i = threadIdx.x; i < 4 * 136; i += blockDim.x) BACC[i] = 0.f;
    __syncthreads();
    const mlp_w W = mlp_views(sm);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc[11][4];
    float db1[8][2], db2[8][2], db3[2] = {0.f, 0.f}, loss = 0.f;
#pragma unroll
    for (int q = 0; q < 11; q++) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
#pragma unroll
    for (int j = 0; j < 8; j++) db1[j][0] = db1[j][1] = db2[j][0] = db2[j][1] = 0.f;
    const int ntiles = (nrows + MLP_TILE - 1) / MLP_TILE;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        {   // stage the warp's 32 rows
            const int rr = warp * 32 + lane, r = tile * MLP_TILE + rr;
            const bool ok = r < nrows;
            const uint4 xv = ok ? X[row0 + r] : make_uint4(0u, 0u, 0u, 0u);
            const float2 yv = ok ? Y[row0 + r] : make_float2(0.f, 0.f);
            *reinterpret_cast<uint4 *>(XR + rr * MLP_S1) = xv;
            const __nv_bfloat16 *xe = reinterpret_cast<const __nv_bfloat16 *>(&xv);
#pragma unroll
            for (int c = 0; c < 8; c++) XT[c * MLP_RS + rr] = xe[c];
            LAB[2 * rr] = yv.x;
            LAB[2 * rr + 1] = yv.y;
        }
        __syncwarp();
#pragma unroll 1
        for (int mt = 0; mt < 2; mt++) {
            const int rbase = warp * 32 + 16 * mt;
            uint32_t h1[4][4], h2[4][4], d1[4][4], d2[4][4];
            float y[4], dy[4] = {0.f, 0.f, 0.f, 0.f};
            mlp_tile_forward(W, XR + rbase * MLP_S1, h1, h2, y);
            if (t == 0) {
                const int ra = rbase + g, rb = rbase + g + 8;
                if (tile * MLP_TILE + ra < nrows) {
                    const float e0 = y[0] - LAB[2 * ra], e1 = y[1] - LAB[2 * ra + 1];
                    loss += e0 * e0 + e1 * e1;
                    dy[0] = 2.f * scale * e0; dy[1] = 2.f * scale * e1;
                }
                if (tile * MLP_TILE + rb < nrows) {
                    const float e0 = y[2] - LAB[2 * rb], e1 = y[3] - LAB[2 * rb + 1];
                    loss += e0 * e0 + e1 * e1;
                    dy[2] = 2.f * scale * e0; dy[3] = 2.f * scale * e1;
                }
            }
            db3[0] += dy[0] + dy[2];
            db3[1] += dy[1] + dy[3];
            const uint32_t ady[4] = {mlp_pack2(dy[0], dy[1]), mlp_pack2(dy[2], dy[3]), 0u, 0u};
#pragma unroll
            for (int j = 0; j < 8; j++) {   // dH2 = (dY W3) o relu'(H2)
                float c[4] = {0.f, 0.f, 0.f, 0.f};
                const __nv_bfloat16 *wr = W.W3T + (8 * j + g) * MLP_S1 + 2 * t;
                mlp_mma(c, ady, mlp_ld32(wr), mlp_ld32(wr + 8));
                mlp_mask(c, h2, j, d2, db2);
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {   // dH1 = (dH2 W2) o relu'(H1)
                float c[4] = {0.f, 0.f, 0.f, 0.f};
                const __nv_bfloat16 *wr = W.W2T + (8 * j + g) * MLP_S2 + 2 * t;
#pragma unroll
                for (int kt = 0; kt < 4; kt++) mlp_mma(c, d2[kt], mlp_ld32(wr + 16 * kt), mlp_ld32(wr + 16 * kt + 8));
                mlp_mask(c, h1, j, d1, db1);
            }
            mlp_store_T(H1T, h1, rbase);
            mlp_store_T(H2T, h2, rbase);
            mlp_store_T(D1T, d1, rbase);
            mlp_store_T(D2T, d2, rbase);
            if (t == 0) {
                DYT[0 * MLP_RS + rbase + g] = __float2bfloat16_rn(dy[0]);
                DYT[1 * MLP_RS + rbase + g] = __float2bfloat16_rn(dy[1]);
                DYT[0 * MLP_RS + rbase + g + 8] = __float2bfloat16_rn(dy[2]);
                DYT[1 * MLP_RS + rbase + g + 8] = __float2bfloat16_rn(dy[3]);
            }
        }
        __syncthreads();
        // weight gradients of the tile: K = 128 rows
#pragma unroll
        for (int q = 0; q < 11; q++) {
            const int tau = warp + 4 * q;
            const __nv_bfloat16 *A, *B;
            int mt, nt;
            if (tau < 32) { A = D2T; mt = tau >> 3; B = H1T; nt = tau & 7; }
            else if (tau < 36) { A = D1T; mt = tau - 32; B = XT; nt = 0; }
            else { A = DYT; mt = 0; B = H2T; nt = tau - 36; }
            const __nv_bfloat16 *a0 = A + (16 * mt + g) * MLP_RS + 2 * t, *a1 = a0 + 8 * MLP_RS;
            const __nv_bfloat16 *b0 = B + (8 * nt + g) * MLP_RS + 2 * t;
#pragma unroll
            for (int kk = 0; kk < 8; kk++) {
                const uint32_t a[4] = {mlp_ld32(a0 + 16 * kk), mlp_ld32(a1 + 16 * kk), mlp_ld32(a0 + 16 * kk + 8),
                                       mlp_ld32(a1 + 16 * kk + 8)};
                mlp_mma(acc[q], a, mlp_ld32(b0 + 16 * kk), mlp_ld32(b0 + 16 * kk + 8));
            }
        }
        __syncthreads();
    }
    // bias and loss sums: lanes with the same t hold the same columns; each
    // warp writes its own slot and the slots are added in warp order below
    // (no shared-memory atomics: the partials are the same bits every run)
    float *BW = BACC + 136 * warp;
#pragma unroll
    for (int j = 0; j < 8; j++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float a = db1[j][h], b = db2[j][h];
            for (int o = 4; o < 32; o <<= 1) {
                a += __shfl_xor_sync(0xffffffffu, a, o);
                b += __shfl_xor_sync(0xffffffffu, b, o);
            }
            if (g == 0) {
                BW[8 * j + 2 * t + h] = a;
                BW[64 + 8 * j + 2 * t + h] = b;
            }
        }
#pragma unroll
    for (int h = 0; h < 2; h++) {
        float a = db3[h];
        for (int o = 4; o < 32; o <<= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) BW[128 + h] = a;
    }
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if (lane == 0) BW[130] = loss;
    __syncthreads();
    for (int i = threadIdx.x; i < 131; i += blockDim.x)
        BACC[i] = ((BACC[i] + BACC[136 + i]) + BACC[272 + i]) + BACC[408 + i];
    __syncthreads();
    float *P = partials + (size_t)blockIdx.x * (MLP_NPARAM + 1);
#pragma unroll
    for (int q = 0; q < 11; q++) {
        const int tau = warp + 4 * q;
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int row = g + ((r & 2) ? 8 : 0), col = 2 * t + (r & 1);
            const float v = acc[q][r];
            if (tau < 32) {
                P[MLP_P_W2 + (16 * (tau >> 3) + row) * 64 + 8 * (tau & 7) + col] = v;
            } else if (tau < 36) {
                P[MLP_P_W1 + (16 * (tau - 32) + row) * 8 + col] = v;
            } else if (row < 2) {
                P[MLP_P_W3 + row * 64 + 8 * (tau - 36) + col] = v;
            }
        }
    }
    for (int i = threadIdx.x; i < 64; i += blockDim.x) {
        P[MLP_P_B1 + i] = BACC[i];
        P[MLP_P_B2 + i] = BACC[64 + i];
    }
    if (threadIdx.x < 2) P[MLP_P_B3 + threadIdx.x] = BACC[128 + threadIdx.x];
    if (threadIdx.x == 0) P[MLP_NPARAM] = BACC[130];
}

// Sum of the CTA partials in a fixed order (8 interleaved slices of the CTAs,
// then the slices in order); optionally one Adam step on the FP32 master
// weights, which also rewrites the packed BF16 image.  Block: 32 parameters x
// 8 slices.
__global__ void __launch_bounds__(256) k_mlp_reduce(int nblk, const float *__restrict__ partials,
                                                    float *__restrict__ grad, float *__restrict__ params,
                                                    float *__restrict__ m, float *__restrict__ v,
                                                    unsigned char *packed, float lr, float b1, float b2, float eps,
                                                    float bc1, float bc2, int adam, const int *__restrict__ tc_err) {
    __shared__ float part[8][33];
    const int lane = threadIdx.x & 31, slice = threadIdx.x >> 5, p = blockIdx.x * 32 + lane;
    if (*tc_err) return;   // a timed-out tensor-core pass leaves the weights alone
    float s = 0.f;
    if (p <= MLP_NPARAM) {
#pragma unroll 4
        for (int b = slice; b < nblk; b += 8) s += partials[(size_t)b * (MLP_NPARAM + 1) + p];
    }
    part[slice][lane] = s;
    __syncthreads();
    if (slice != 0 || p > MLP_NPARAM) return;
    s = part[0][lane];
#pragma unroll
    for (int q = 1; q < 8; q++) s += part[q][lane];
    grad[p] = s;
    if (!adam || p == MLP_NPARAM) return;
    const float mm = b1 * m[p] + (1.f - b1) * s, vv = b2 * v[p] + (1.f - b2) * s * s;
    m[p] = mm;
    v[p] = vv;
    const float w = params[p] - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
    params[p] = w;
    mlp_write_packed(packed, p, w);
}

// Inference over n rows of normalised BF16 inputs: 8 warps per CTA, 32 rows per
// warp pass, grid-stride.
__global__ void __launch_bounds__(256) k_mlp_infer(const unsigned char *__restrict__ packed,
                                                   const uint4 *__restrict__ X, long long n, float2 *__restrict__ Y) {
    extern __shared__ __align__(16) unsigned char sm[];
    __nv_bfloat16 *XS = reinterpret_cast<__nv_bfloat16 *>(sm + MLP_PACK_BYTES);
    float *YS = reinterpret_cast<float *>(XS + 8 * 32 * MLP_S1);
    mlp_load_weights(sm, packed);
    for (int i = threadIdx.x; i < 8 * 32 * MLP_S1; i += blockDim.x) XS[i] = __float2bfloat16_rn(0.f);
    __syncthreads();
    const mlp_w W = mlp_views(sm);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16 *xs = XS + warp * 32 * MLP_S1;
    float *ys = YS + warp * 64;
    for (long long base = ((long long)blockIdx.x * 8 + warp) * 32; base < n; base += (long long)gridDim.x * 8 * 32) {
        const long long r = base + lane;
        *reinterpret_cast<uint4 *>(xs + lane * MLP_S1) = r < n ? X[r] : make_uint4(0u, 0u, 0u, 0u);
        __syncwarp();
        mlp_warp_infer(W, xs, ys);
        __syncwarp();
        if (r < n) Y[r] = make_float2(ys[2 * lane], ys[2 * lane + 1]);
        __syncwarp();
    }
}

__global__ void k_mlp_rows_bf16(long long n, const float *__restrict__ x, uint4 *__restrict__ X) {
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    uint32_t w[4];
    for (int k = 0; k < 4; k++) w[k] = mlp_pack2(x[8 * r + 2 * k], x[8 * r + 2 * k + 1]);
    X[r] = make_uint4(w[0], w[1], w[2], w[3]);
}

// ---------------------------------------------------------------------------
// State
static mdz_status mlp_ensure(mdz_ctx *ctx) {
    if (ctx->mlp) return MDZ_OK;
    mdz_mlp *M = new mdz_mlp();
    ctx->mlp = M;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    M->max_blocks = (sms > 0 ? sms : 152);
    cudaError_t e = cudaMalloc((void **)&M->params, sizeof(float) * MLP_NPARAM);
    if (e == cudaSuccess) e = cudaMalloc((void **)&M->adam_m, sizeof(float) * MLP_NPARAM);
    if (e == cudaSuccess) e = cudaMalloc((void **)&M->adam_v, sizeof(float) * MLP_NPARAM);
    if (e == cudaSuccess) e = cudaMalloc((void **)&M->packed, MLP_PACK_BYTES);
    if (e == cudaSuccess) e = cudaMemset(M->packed, 0, MLP_PACK_BYTES);
    // partial gradient rows: one per CTA, two CTAs per SM for the tcgen05 pass
    if (e == cudaSuccess) e = cudaMalloc((void **)&M->partials, sizeof(float) * (MLP_NPARAM + 1) * 2 * M->max_blocks);
    if (e == cudaSuccess) e = cudaMalloc((void **)&M->grad, sizeof(float) * (MLP_NPARAM + 1));
    if (e == cudaSuccess) e = cudaMalloc((void **)&M->tc_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(M->tc_err, 0, sizeof(int));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem_bytes());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)infer_smem_bytes());
    if (e != cudaSuccess) return mdz_cuda_check(ctx, e, "MLP allocation");
    return MDZ_OK;
}

void mdz_mlp_free(mdz_ctx *ctx) {
    if (!ctx->mlp) return;
    mdz_mlp *M = ctx->mlp;
    void *p[] = {M->params, M->adam_m, M->adam_v, M->packed, M->partials, M->grad, M->X, M->Y, M->guess, M->tc_err};
    for (void *q : p)
        if (q) cudaFree(q);
    delete M;
    ctx->mlp = nullptr;
}

bool mdz_mlp_ready(const mdz_ctx *ctx) { return ctx->mlp && ctx->mlp->has_weights; }

float2 *mdz_mlp_guess_buffer(mdz_ctx *ctx, size_t n) {
    mdz_mlp *M = ctx->mlp;
    if (!M) return nullptr;
    if (M->guess_cap < n) {
        if (M->guess) cudaFree(M->guess);
        M->guess = nullptr;
        M->guess_cap = 0;
        if (cudaMalloc((void **)&M->guess, sizeof(float2) * n) != cudaSuccess) return nullptr;
        M->guess_cap = n;
    }
    return M->guess;
}

static mdz_status mlp_pack(mdz_ctx *ctx) {
    k_mlp_pack<<<mdz_blocks(MLP_NPARAM), MDZ_THREADS, 0, ctx->stream>>>(ctx->mlp->params, ctx->mlp->packed);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

static mdz_status mlp_reset_adam(mdz_ctx *ctx) {
    mdz_mlp *M = ctx->mlp;
    MDZ_CUDA(ctx, cudaMemsetAsync(M->adam_m, 0, sizeof(float) * MLP_NPARAM, ctx->stream));
    MDZ_CUDA(ctx, cudaMemsetAsync(M->adam_v, 0, sizeof(float) * MLP_NPARAM, ctx->stream));
    M->adam_t = 0;
    return MDZ_OK;
}

static uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

extern "C" mdz_status mdz_mlp_init(mdz_ctx *ctx, unsigned long long seed) {
    if (!ctx) return MDZ_ERR_ARG;
    mdz_status s = mlp_ensure(ctx);
    if (s != MDZ_OK) return s;
    // He-uniform weights, zero biases
    std::vector<float> w(MLP_NPARAM, 0.0f);
    uint64_t st = seed;
    auto fill = [&](int off, int n, int fan_in) {
        const double a = std::sqrt(6.0 / fan_in);
        for (int i = 0; i < n; i++) w[off + i] = (float)(a * (2.0 * ((splitmix(st) >> 11) * 0x1.0p-53) - 1.0));
    };
    fill(MLP_P_W1, 64 * 8, 8);
    fill(MLP_P_W2, 64 * 64, 64);
    fill(MLP_P_W3, 2 * 64, 64);
    MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->mlp->params, w.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice,
                                  ctx->stream));
    if ((s = mlp_pack(ctx)) != MDZ_OK) return s;
    if ((s = mlp_reset_adam(ctx)) != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->mlp->has_weights = true;
    ctx->mlp->trained = false;
    return MDZ_OK;
}

extern "C" mdz_status mdz_mlp_set_weights(mdz_ctx *ctx, const float *w) {
    if (!ctx || !w) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mlp_set_weights: null argument") : MDZ_ERR_ARG;
    mdz_status s = mlp_ensure(ctx);
    if (s != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->mlp->params, w, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice,
                                  ctx->stream));
    if ((s = mlp_pack(ctx)) != MDZ_OK) return s;
    if ((s = mlp_reset_adam(ctx)) != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->mlp->has_weights = true;
    return MDZ_OK;
}

extern "C" mdz_status mdz_mlp_get_weights(mdz_ctx *ctx, float *w) {
    if (!ctx || !w) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mlp_get_weights: null argument") : MDZ_ERR_ARG;
    if (!mdz_mlp_ready(ctx)) return mdz_fail(ctx, MDZ_ERR_STATE, "mlp_get_weights: no weights");
    MDZ_CUDA(ctx, cudaMemcpyAsync(w, ctx->mlp->params, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MDZ_OK;
}

extern "C" mdz_status mdz_mlp_set_ranges(mdz_ctx *ctx, const double *lo, const double *hi) {
    if (!ctx || !lo || !hi) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mlp_set_ranges: null argument") : MDZ_ERR_ARG;
    mdz_status s = mlp_ensure(ctx);
    if (s != MDZ_OK) return s;
    mdz_mlp *M = ctx->mlp;
    if (!(lo[1] > 0)) return mdz_fail(ctx, MDZ_ERR_ARG, "mlp_set_ranges: temperatures must be > 0 K");
    for (int k = 0; k < 4; k++) {
        if (!(hi[k] > lo[k])) return mdz_fail(ctx, MDZ_ERR_ARG, "mlp_set_ranges: range %d is empty", k);
        M->lo[k] = lo[k];
        M->hi[k] = hi[k];
        // temperature is fed as 1000 / T
        const double a = k == 1 ? 1000.0 / hi[k] : lo[k], b = k == 1 ? 1000.0 / lo[k] : hi[k];
        M->norm.lo[k] = (float)a;
        M->norm.inv[k] = (float)(1.0 / (b - a));
    }
    return MDZ_OK;
}

extern "C" mdz_status mdz_mlp_generate(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm,
                                       long long n, unsigned long long seed, const double *lo, const double *hi) {
    if (!ctx || !m || !prm || !lo || !hi || n <= 0)
        return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mlp_generate: bad argument") : MDZ_ERR_ARG;
    mdz_status s = mdz_check_materials(ctx, m);
    if (s != MDZ_OK) return s;
    if (m->n_phases > 4) return mdz_fail(ctx, MDZ_ERR_UNSUPPORTED, "mlp: the network encodes at most 4 phases");
    if ((s = mdz_mlp_set_ranges(ctx, lo, hi)) != MDZ_OK) return s;
    mdz_mlp *M = ctx->mlp;
    if (M->cap < n) {
        if (M->X) cudaFree(M->X);
        if (M->Y) cudaFree(M->Y);
        M->X = nullptr; M->Y = nullptr; M->cap = 0;
        MDZ_CUDA(ctx, cudaMalloc((void **)&M->X, sizeof(uint4) * n));
        MDZ_CUDA(ctx, cudaMalloc((void **)&M->Y, sizeof(float2) * n));
        M->cap = n;
    }
    M->n = n;
    if ((s = mdz_dev_mlp_samples(ctx, m, prm, n, seed, lo, hi, M->norm, M->X, M->Y, ctx->stream)) != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MDZ_OK;
}

static mdz_status mlp_tc_status(mdz_ctx *ctx);

// one pass over `rows` rows starting at row0: partial gradients + reduction (+ Adam)
static mdz_status mlp_step(mdz_ctx *ctx, const uint4 *X, const float2 *Y, long long row0, int rows, int adam,
                           float lr) {
    mdz_mlp *M = ctx->mlp;
    cudaStream_t st = ctx->stream;
    const int tiles = (rows + MLP_TILE - 1) / MLP_TILE, cap = (M->engine == 0 ? 2 : 1) * M->max_blocks;
    int nblk = tiles < cap ? tiles : cap;
    if (nblk < 1) nblk = 1;
    if (M->engine == 0) {
        mdz_status r = mdz_mlp_train_tc(ctx, M->packed, X, Y, row0, rows, 1.0f / (float)rows, M->partials, nblk,
                                        M->tc_err, st);
        if (r != MDZ_OK) return r;
    } else {
        k_mlp_train<<<nblk, 128, train_smem_bytes(), st>>>(M->packed, X, Y, row0, rows, 1.0f / (float)rows,
                                                           M->partials);
        MDZ_LAUNCHED(ctx);
    }
    float bc1 = 1.f, bc2 = 1.f;
    const float b1 = 0.9f, b2 = 0.999f;
    if (adam) {
        M->adam_t++;
        bc1 = 1.f - powf(b1, (float)M->adam_t);
        bc2 = 1.f - powf(b2, (float)M->adam_t);
    }
    k_mlp_reduce<<<(MLP_NPARAM + 1 + 31) / 32, 256, 0, st>>>(nblk, M->partials, M->grad, M->params,
                                                                     M->adam_m, M->adam_v, M->packed, lr, b1, b2,
                                                                     1e-8f, bc1, bc2, adam, M->tc_err);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

extern "C" mdz_status mdz_mlp_train(mdz_ctx *ctx, int steps, int batch, double lr, double *final_loss) {
    if (!ctx || steps < 1 || batch < 1 || !(lr > 0))
        return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mlp_train: bad argument") : MDZ_ERR_ARG;
    if (!mdz_mlp_ready(ctx)) return mdz_fail(ctx, MDZ_ERR_STATE, "mlp_train: call mdz_mlp_init first");
    mdz_mlp *M = ctx->mlp;
    if (M->n < batch) return mdz_fail(ctx, MDZ_ERR_STATE, "mlp_train: %lld samples < batch %d", M->n, batch);
    const long long nb = M->n / batch;
    double loss_acc = 0.0;
    int loss_n = 0;
    for (int s = 0; s < steps; s++) {
        // cosine decay to lr / 100
        const double c = 0.5 * (1.0 + std::cos(M_PI * (double)s / (double)steps));
        const float lrs = (float)(lr * (0.01 + 0.99 * c));
        mdz_status r = mlp_step(ctx, M->X, M->Y, (long long)(s % nb) * batch, batch, 1, lrs);
        if (r != MDZ_OK) return r;
        if (s >= steps - 8) {   // mean loss of the last steps
            float h = 0.f;
            MDZ_CUDA(ctx, cudaMemcpyAsync(&h, M->grad + MLP_NPARAM, sizeof(float), cudaMemcpyDeviceToHost,
                                          ctx->stream));
            MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            loss_acc += h / batch;
            loss_n++;
        }
    }
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    mdz_status ts = mlp_tc_status(ctx);
    if (ts != MDZ_OK) return ts;
    M->trained = true;
    M->last_loss = loss_n ? loss_acc / loss_n : 0.0;
    if (final_loss) *final_loss = M->last_loss;
    if (!std::isfinite(M->last_loss)) return mdz_fail(ctx, MDZ_ERR_NAN, "mlp_train: loss is not finite");
    return MDZ_OK;
}

extern "C" mdz_status mdz_mlp_gradients(mdz_ctx *ctx, int n, const float *x, const float *y, float *grad,
                                        double *loss) {
    if (!ctx || n < 1 || !x || !y || !grad)
        return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mlp_gradients: bad argument") : MDZ_ERR_ARG;
    if (!mdz_mlp_ready(ctx)) return mdz_fail(ctx, MDZ_ERR_STATE, "mlp_gradients: no weights");
    cudaStream_t st = ctx->stream;
    size_t bytes = sizeof(float) * 8 * n + sizeof(uint4) * n + sizeof(float2) * n;
    unsigned char *buf = (unsigned char *)mdz_stage(ctx, 6, bytes);
    if (!buf) return mdz_fail(ctx, MDZ_ERR_CUDA, "mlp_gradients: staging allocation failed");
    float *dx = (float *)buf;
    uint4 *X = (uint4 *)(buf + sizeof(float) * 8 * n);
    float2 *Y = (float2 *)(buf + sizeof(float) * 8 * n + sizeof(uint4) * n);
    MDZ_CUDA(ctx, cudaMemcpyAsync(dx, x, sizeof(float) * 8 * n, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(Y, y, sizeof(float2) * n, cudaMemcpyHostToDevice, st));
    k_mlp_rows_bf16<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, dx, X);
    MDZ_LAUNCHED(ctx);
    mdz_status s = mlp_step(ctx, X, Y, 0, n, 0, 0.f);
    if (s != MDZ_OK) return s;
    std::vector<float> h(MLP_NPARAM + 1);
    MDZ_CUDA(ctx, cudaMemcpyAsync(h.data(), ctx->mlp->grad, sizeof(float) * (MLP_NPARAM + 1), cudaMemcpyDeviceToHost,
                                  st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    if ((s = mlp_tc_status(ctx)) != MDZ_OK) return s;
    memcpy(grad, h.data(), sizeof(float) * MLP_NPARAM);
    if (loss) *loss = h[MLP_NPARAM] / (double)n;
    return MDZ_OK;
}

// The tcgen05 kernel's time-out flag (read after a synchronisation; cleared).
static mdz_status mlp_tc_status(mdz_ctx *ctx) {
    int e = 0;
    MDZ_CUDA(ctx, cudaMemcpy(&e, ctx->mlp->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (!e) return MDZ_OK;
    MDZ_CUDA(ctx, cudaMemset(ctx->mlp->tc_err, 0, sizeof(int)));
    return mdz_fail(ctx, MDZ_ERR_STATE, "mlp: a tensor-core commit did not arrive (time-out)");
}

static mdz_status mlp_infer_dev(mdz_ctx *ctx, const uint4 *X, long long n, float2 *Y, cudaStream_t st) {
    if (ctx->mlp->engine == 0) return mdz_mlp_infer_tc(ctx, ctx->mlp->packed, X, n, Y, ctx->mlp->tc_err, st);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long warps = (n + 31) / 32, blocks = (warps + 7) / 8;
    long long cap = (long long)sms * 4;
    int grid = (int)(blocks < cap ? (blocks < 1 ? 1 : blocks) : cap);
    k_mlp_infer<<<grid, 256, infer_smem_bytes(), st>>>(ctx->mlp->packed, X, n, Y);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

extern "C" mdz_status mdz_mlp_infer(mdz_ctx *ctx, long long n, const float *x, float *y) {
    if (!ctx || n < 1 || !x || !y) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mlp_infer: bad argument") : MDZ_ERR_ARG;
    if (!mdz_mlp_ready(ctx)) return mdz_fail(ctx, MDZ_ERR_STATE, "mlp_infer: no weights");
    cudaStream_t st = ctx->stream;
    size_t bytes = sizeof(float) * 8 * n + sizeof(uint4) * n + sizeof(float2) * n;
    unsigned char *buf = (unsigned char *)mdz_stage(ctx, 6, bytes);
    if (!buf) return mdz_fail(ctx, MDZ_ERR_CUDA, "mlp_infer: staging allocation failed");
    float *dx = (float *)buf;
    uint4 *X = (uint4 *)(buf + sizeof(float) * 8 * n);
    float2 *Y = (float2 *)(buf + sizeof(float) * 8 * n + sizeof(uint4) * n);
    MDZ_CUDA(ctx, cudaMemcpyAsync(dx, x, sizeof(float) * 8 * n, cudaMemcpyHostToDevice, st));
    k_mlp_rows_bf16<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, dx, X);
    MDZ_LAUNCHED(ctx);
    mdz_status s = mlp_infer_dev(ctx, X, n, Y, st);
    if (s != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaMemcpyAsync(y, Y, sizeof(float2) * n, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return mlp_tc_status(ctx);
}

extern "C" mdz_status mdz_mlp_set_engine(mdz_ctx *ctx, int engine) {
    if (!ctx || (engine != 0 && engine != 1)) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mlp_set_engine: 0 or 1") : MDZ_ERR_ARG;
    mdz_status s = mlp_ensure(ctx);
    if (s != MDZ_OK) return s;
    ctx->mlp->engine = engine;
    return MDZ_OK;
}

// Timing of the resident pieces: inference over the generated tuples and one
// training step at the given batch (CUDA events, after one warm-up each).
extern "C" mdz_status mdz_mlp_benchmark(mdz_ctx *ctx, int batch, int reps, double *ms_infer, double *ms_train_step,
                                        double *rms_error) {
    if (!ctx || batch < 1 || reps < 1) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mlp_benchmark: bad argument") : MDZ_ERR_ARG;
    if (!mdz_mlp_ready(ctx)) return mdz_fail(ctx, MDZ_ERR_STATE, "mlp_benchmark: no weights");
    mdz_mlp *M = ctx->mlp;
    if (M->n < batch) return mdz_fail(ctx, MDZ_ERR_STATE, "mlp_benchmark: generate at least one batch of tuples");
    cudaStream_t st = ctx->stream;
    float2 *Y = (float2 *)mdz_stage(ctx, 6, sizeof(float2) * M->n);
    if (!Y) return mdz_fail(ctx, MDZ_ERR_CUDA, "mlp_benchmark: staging allocation failed");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    mdz_status s = mlp_infer_dev(ctx, M->X, M->n, Y, st);
    if (s != MDZ_OK) return s;
    cudaEventRecord(a, st);
    for (int r = 0; r < reps; r++)
        if ((s = mlp_infer_dev(ctx, M->X, M->n, Y, st)) != MDZ_OK) return s;
    cudaEventRecord(b, st);
    MDZ_CUDA(ctx, cudaEventSynchronize(b));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms_infer) *ms_infer = ms / reps;
    if ((s = mlp_tc_status(ctx)) != MDZ_OK) return s;
    if (rms_error) {   // RMS of the outputs against the labels over the tuples
        std::vector<float2> h(M->n), l(M->n);
        MDZ_CUDA(ctx, cudaMemcpy(h.data(), Y, sizeof(float2) * M->n, cudaMemcpyDeviceToHost));
        MDZ_CUDA(ctx, cudaMemcpy(l.data(), M->Y, sizeof(float2) * M->n, cudaMemcpyDeviceToHost));
        double e = 0.0;
        for (long long i = 0; i < M->n; i++) {
            double d0 = h[i].x - l[i].x, d1 = h[i].y - l[i].y;
            e += d0 * d0 + d1 * d1;
        }
        *rms_error = std::sqrt(e / (2.0 * M->n));
    }
    // training step timing on a copy of the weights (restored afterwards)
    std::vector<float> keep(MLP_NPARAM);
    MDZ_CUDA(ctx, cudaMemcpy(keep.data(), M->params, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost));
    int t_keep = M->adam_t;
    if ((s = mlp_step(ctx, M->X, M->Y, 0, batch, 1, 1e-6f)) != MDZ_OK) return s;
    cudaEventRecord(a, st);
    for (int r = 0; r < reps; r++)
        if ((s = mlp_step(ctx, M->X, M->Y, 0, batch, 1, 1e-6f)) != MDZ_OK) return s;
    cudaEventRecord(b, st);
    MDZ_CUDA(ctx, cudaEventSynchronize(b));
    cudaEventElapsedTime(&ms, a, b);
    if (ms_train_step) *ms_train_step = ms / reps;
    if ((s = mlp_tc_status(ctx)) != MDZ_OK) return s;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    MDZ_CUDA(ctx, cudaMemcpy(M->params, keep.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice));
    M->adam_t = t_keep;
    if ((s = mlp_pack(ctx)) != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}

// NonNewtonianViscosityGrid with the MLP start: guesses for every (phase,
// node), then the local solves polish them (rheology.cu).
mdz_status mdz_dev_viscosity_learned(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm,
                                     const mdz_fields &f, int *d_counters, cudaStream_t st, int warm) {
    if (!mdz_mlp_ready(ctx)) return mdz_fail(ctx, MDZ_ERR_STATE, "learned guess: no MLP weights loaded");
    if (m->n_phases > 4) return mdz_fail(ctx, MDZ_ERR_UNSUPPORTED, "learned guess: at most 4 phases");
    return mdz_dev_viscosity(ctx, m, prm, f, d_counters, st, true, false, warm);
}
