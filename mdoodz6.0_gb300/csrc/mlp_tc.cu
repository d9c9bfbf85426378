// Inference of the learned-guess network on the fifth-generation tensor cores:
// tcgen05.mma with the operands in shared memory and the FP32 accumulators in
// tensor memory (TMEM), 128-row batch tiles.
//
// One CTA of 4 warps works a 128-row tile at a time (persistent over tiles):
//   layer 1  D1[128x64] = X[128x16] W1^T        1 MMA   (K = 16: 8 inputs + 8 zero columns)
//   layer 2  D2[128x64] = relu(D1 + b1) W2^T    4 MMAs  (K = 64 in steps of 16)
//   layer 3  D3[128x16] = relu(D2 + b2) W3^T    4 MMAs  (N = 16: 2 outputs + 14 zero rows of W3)
// Thread t owns row t of the tile: TMEM lane t holds that row of each
// accumulator (warp w reads lanes 32w..32w+31 with tcgen05.ld.32x32b), and the
// epilogue (bias, ReLU, BF16) writes the row back to shared memory as the next
// layer's A operand.  Operands use the canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices, adjacent along K at LBO = 128 bytes
// and along M/N at SBO = 16 K-bytes.  One elected thread issues the MMAs and
// commits them to an mbarrier that every thread then waits on (bounded: on a
// time-out the kernel raises the error flag, frees its TMEM and returns).
#include <cuda_bf16.h>
#include "mlp.cuh"

namespace {

constexpr int TC_ROWS = 128;
constexpr int TC_THREADS = 128;
constexpr int TC_TMEM_COLS = 64;           // D1, D2, D3 in turn in columns 0..63
// shared-memory image (bytes)
constexpr int SM_X = 0;                    // 128 x 16 BF16  = 4096
constexpr int SM_H = 4096;                 // 128 x 64 BF16  = 16384 (H1, then H2)
constexpr int SM_W1 = 20480;               // 64 x 16 BF16   = 2048
constexpr int SM_W2 = 22528;               // 64 x 64 BF16   = 8192
constexpr int SM_W3 = 30720;               // 16 x 64 BF16   = 2048
constexpr int SM_B = 32768;                // b1[64] b2[64] b3[16] FP32 = 576
constexpr int SM_BAR = 33344;              // mbarrier (8 bytes)
constexpr int SM_TMEM = 33352;             // TMEM base written by tcgen05.alloc
constexpr int SM_BYTES = 33408;
constexpr long long TC_WAIT_LIMIT = 1LL << 24;

// byte offset of element (r, k) of an R x K K-major operand with K / 8 core
// matrices per 8-row group
__device__ __forceinline__ uint32_t kmaj_off(int r, int k, int kgroups) {
    return (uint32_t)((r >> 3) * (kgroups * 128) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), the
// descriptor version 1 at bit 46, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        :: "r"(dtmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (long long i = 0; i < TC_WAIT_LIMIT; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive columns as two x16 loads behind one wait
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
#pragma unroll
    for (int h = 0; h < 2; h++)
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(r[16 * h + 0]), "=r"(r[16 * h + 1]), "=r"(r[16 * h + 2]), "=r"(r[16 * h + 3]),
              "=r"(r[16 * h + 4]), "=r"(r[16 * h + 5]), "=r"(r[16 * h + 6]), "=r"(r[16 * h + 7]),
              "=r"(r[16 * h + 8]), "=r"(r[16 * h + 9]), "=r"(r[16 * h + 10]), "=r"(r[16 * h + 11]),
              "=r"(r[16 * h + 12]), "=r"(r[16 * h + 13]), "=r"(r[16 * h + 14]), "=r"(r[16 * h + 15])
            : "r"(taddr + 16 * h));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float (&v)[2]) {
    uint32_t r0, r1;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r0), "=r"(r1) : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    v[0] = __uint_as_float(r0);
    v[1] = __uint_as_float(r1);
}

// epilogue of a 64-column accumulator: row `row` of relu(D + b) as BF16 into
// the K-major H operand (8 core matrices along K)
__device__ __forceinline__ void epilogue64(uint32_t taddr, const float *b, unsigned char *H, int row) {
#pragma unroll
    for (int c = 0; c < 4; c++) {
        float v[16];
        tmem_ld16(taddr + 16 * c, v);
        uint32_t w[8];
#pragma unroll
        for (int i = 0; i < 8; i++)
            w[i] = mlp_pack2(fmaxf(v[2 * i] + b[16 * c + 2 * i], 0.f), fmaxf(v[2 * i + 1] + b[16 * c + 2 * i + 1], 0.f));
        *reinterpret_cast<uint4 *>(H + kmaj_off(row, 16 * c, 8)) = make_uint4(w[0], w[1], w[2], w[3]);
        *reinterpret_cast<uint4 *>(H + kmaj_off(row, 16 * c + 8, 8)) = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

}  // namespace

__global__ void __launch_bounds__(TC_THREADS) k_mlp_infer_tc(const unsigned char *__restrict__ packed,
                                                             const uint4 *__restrict__ X, long long n,
                                                             float2 *__restrict__ Y, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights into the K-major tiles; biases
    {
        const __nv_bfloat16 *w = reinterpret_cast<const __nv_bfloat16 *>(packed);
        const float *bias = reinterpret_cast<const float *>(packed + MLP_NBF16 * 2);
        for (int e = tid; e < 64 * 16; e += TC_THREADS) {
            const int r = e >> 4, k = e & 15;
            *reinterpret_cast<__nv_bfloat16 *>(sm + SM_W1 + kmaj_off(r, k, 2)) =
                k < MLP_IN ? w[MLP_W1S + r * MLP_S1 + k] : __float2bfloat16_rn(0.f);
        }
        for (int e = tid; e < 64 * 64; e += TC_THREADS) {
            const int r = e >> 6, k = e & 63;
            *reinterpret_cast<__nv_bfloat16 *>(sm + SM_W2 + kmaj_off(r, k, 8)) = w[MLP_W2S + r * MLP_S2 + k];
        }
        for (int e = tid; e < 16 * 64; e += TC_THREADS) {
            const int r = e >> 6, k = e & 63;
            *reinterpret_cast<__nv_bfloat16 *>(sm + SM_W3 + kmaj_off(r, k, 8)) =
                r < MLP_OUT ? w[MLP_W3S + r * MLP_S2 + k] : __float2bfloat16_rn(0.f);
        }
        float *b = reinterpret_cast<float *>(sm + SM_B);
        for (int e = tid; e < 144; e += TC_THREADS) b[e] = e < 128 ? bias[e] : (e < 130 ? bias[e] : 0.f);
    }
    const uint32_t bar = smem_u32(sm + SM_BAR);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {   // TMEM columns for the three accumulators
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(sm + SM_TMEM)), "r"(TC_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_before_sync();
    }
    fence_async_smem();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(sm + SM_TMEM);
    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);   // this warp's lane quarter
    const float *b1 = reinterpret_cast<const float *>(sm + SM_B), *b2 = b1 + 64, *b3 = b1 + 128;
    const uint32_t aX = smem_u32(sm + SM_X), aH = smem_u32(sm + SM_H), aW1 = smem_u32(sm + SM_W1),
                   aW2 = smem_u32(sm + SM_W2), aW3 = smem_u32(sm + SM_W3);
    uint32_t phase = 0;
    bool ok = true;
    const long long tiles = (n + TC_ROWS - 1) / TC_ROWS;
    for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const long long row = tile * TC_ROWS + tid;
        const uint4 x = row < n ? X[row] : make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4 *>(sm + SM_X + kmaj_off(tid, 0, 2)) = x;
        *reinterpret_cast<uint4 *>(sm + SM_X + kmaj_off(tid, 8, 2)) = make_uint4(0u, 0u, 0u, 0u);
        fence_async_smem();
        tc_before_sync();
        __syncthreads();
        tc_after_sync();
        // layer 1
        if (tid == 0) {
            mma_bf16(tmem, sdesc(aX, 128, 256), sdesc(aW1, 128, 256), idesc_bf16(128, 64), 0);
            mma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait(bar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_after_sync();
        epilogue64(trow, b1, sm + SM_H, tid);
        fence_async_smem();
        tc_before_sync();
        __syncthreads();
        tc_after_sync();
        // layer 2
        if (tid == 0) {
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                mma_bf16(tmem, sdesc(aH + 256 * kk, 128, 1024), sdesc(aW2 + 256 * kk, 128, 1024),
                         idesc_bf16(128, 64), kk > 0);
            mma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait(bar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_after_sync();
        epilogue64(trow, b2, sm + SM_H, tid);
        fence_async_smem();
        tc_before_sync();
        __syncthreads();
        tc_after_sync();
        // layer 3
        if (tid == 0) {
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                mma_bf16(tmem, sdesc(aH + 256 * kk, 128, 1024), sdesc(aW3 + 256 * kk, 128, 1024),
                         idesc_bf16(128, 16), kk > 0);
            mma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait(bar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_after_sync();
        float y[2];
        tmem_ld2(trow, y);
        if (row < n) Y[row] = make_float2(y[0] + b3[0], y[1] + b3[1]);
        tc_before_sync();
        __syncthreads();
        tc_after_sync();
    }
    if (!ok) {
        // a commit that never arrived: flag it, give the tensor core one more
        // bounded wait for the work in flight, then release the TMEM
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(bar, phase ^ 1);   // the phase that timed out
    }
    tc_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TC_TMEM_COLS) : "memory");
    }
}

// Host launcher: persistent grid of up to 6 CTAs per SM (33 KB of shared
// memory and 64 TMEM columns each: six fit in both).  Each accumulator is read
// out by every thread before the next layer's MMA is issued, so the three
// layers share the CTA's 64 columns.
mdz_status mdz_mlp_infer_tc(mdz_ctx *ctx, const unsigned char *packed, const uint4 *X, long long n, float2 *Y,
                            int *d_err, cudaStream_t st) {
    static bool attr_set = false;
    if (!attr_set) {
        MDZ_CUDA(ctx, cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_BYTES));
        attr_set = true;
    }
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (n + TC_ROWS - 1) / TC_ROWS, cap = (long long)sms * 6;
    const int grid = (int)(tiles < cap ? (tiles < 1 ? 1 : tiles) : cap);
    k_mlp_infer_tc<<<grid, TC_THREADS, SM_BYTES, st>>>(packed, X, n, Y, d_err);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// Training on tcgen05: one pass of forward, backward and the weight gradients
// of the squared error over `nrows` rows, one partial gradient per CTA (the
// layout and reduction of the warp-level kernel in mlp.cu).  Thread t owns row
// t of a 128-row tile as in inference; per tile:
//   layers 1..3 as in inference
//   dH2[128x64] = dY[128x16] W3      1 MMA  (B = W3 transposed; K = 2 outputs + 14 zeros)
//   dH1[128x64] = dH2' W2            4 MMAs (B = W2 transposed), dH2' = dH2 o relu'(H2)
//   weight gradients (K = the tile's 128 rows), accumulated in TMEM over all
//   the CTA's tiles:
//     G_a[128x80] += [dH2' dH1']^T [H1 X 0]    8 MMAs: rows 0..63 x cols 0..63 = dW2,
//                                                      rows 64..127 x cols 64..71 = dW1
//     G_b[128x16] += [H2 dH2']^T [dY 0]        8 MMAs: rows 0..63 x cols 0..1 = dW3^T
// Every activation and delta is written once, row by row (16-byte stores),
// into three tiles: Q = [H1 | X | 0] (80 columns), T = [H2 | dH2' | dH1']
// (192 columns) and D = [dY | 0] (16 columns).  The forward and backward MMAs
// read column windows of them as K-major A operands; the gradient MMAs read
// them as MN-major operands (rows = K), so no transposed copy is made.  Bias
// gradients and the loss are FP32 sums of the unrounded deltas per thread,
// added over the CTA in a fixed order at the end (the partials are the same
// bits every run).
namespace {

constexpr int TR_XA = 0;          // [X | 0] 128 x 16 (A of layer 1)              4096
constexpr int TR_D = 4096;        // [dY | 0] 128 x 16                            4096
constexpr int TR_W1 = 8192;       // 64 x 16                                      2048
constexpr int TR_W2 = 10240;      // 64 x 64                                      8192
constexpr int TR_W3 = 18432;      // 16 x 64                                      2048
constexpr int TR_W3T = 20480;     // 64 x 16: W3 transposed                       2048
constexpr int TR_W2T = 22528;     // 64 x 64: W2 transposed                       8192
constexpr int TR_T = 30720;       // [H2 | dH2' | dH1'] 128 x 192                 49152
constexpr int TR_Q = 79872;       // [H1 | X | 0] 128 x 80                        20480
constexpr int TR_B = 100352;      // b1[64] b2[64] b3[16] FP32                    576
constexpr int TR_BAR = 100928;
constexpr int TR_TMEM = 100936;
constexpr int TR_BYTES = 100992;  // two CTAs per SM
constexpr int TR_TMEM_COLS = 256;  // 0..63 layers and deltas, 64..143 G_a, 160..175 G_b
constexpr int TR_GA = 64, TR_GB = 160;
constexpr int TR_SUMS = 131;       // b1, b2, b3 gradient sums and the loss per thread
constexpr int TR_TG = 24, TR_QG = 10, TR_DG = 2;   // 16-byte column groups of T, Q, D

// instruction descriptor of kind::f16 with both operands MN-major (bits 15, 16)
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int M, int N) {
    return idesc_bf16(M, N) | (1u << 15) | (1u << 16);
}

// MN-major operand without swizzle read from a row-major tile (rows = K):
// core matrices of 8 K-rows x 8 MN-columns, adjacent along MN at 128 bytes and
// along K at `kstride` (the tile's 8-row group stride); the K-direction stride
// goes in LBO and the MN-direction one in SBO
__device__ __forceinline__ uint64_t sdesc_mn(uint32_t addr, uint32_t kstride) { return sdesc(addr, kstride, 128); }

__device__ __forceinline__ void st_row16(unsigned char *tile, int groups, int row, int col, const uint32_t (&w)[8]) {
    *reinterpret_cast<uint4 *>(tile + kmaj_off(row, col, groups)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4 *>(tile + kmaj_off(row, col + 8, groups)) = make_uint4(w[4], w[5], w[6], w[7]);
}

// bit pair of a packed BF16 pair that is non-zero (the ReLU outputs are >= 0)
__device__ __forceinline__ uint64_t nz_bits(uint32_t w, int col) {
    return ((uint64_t)((w & 0x7fffu) != 0u) << col) | ((uint64_t)((w & 0x7fff0000u) != 0u) << (col + 1));
}

// every thread's shared-memory writes visible to the tensor core and every
// earlier TMEM read finished before the MMA issue
__device__ __forceinline__ void tc_handoff() {
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
}

}  // namespace

__global__ void __launch_bounds__(TC_THREADS, 2) k_mlp_train_tc(const unsigned char *__restrict__ packed,
                                                                const uint4 *__restrict__ X,
                                                                const float2 *__restrict__ Y, long long row0,
                                                                int nrows, float scale,
                                                                float *__restrict__ partials, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    {   // weights: 16-byte chunks (8 K-consecutive elements of a row; the packed
        // rows are 48 or 144 bytes long and their zero padding fills K to 16)
        const __nv_bfloat16 *w = reinterpret_cast<const __nv_bfloat16 *>(packed);
        const float *bias = reinterpret_cast<const float *>(packed + MLP_NBF16 * 2);
        const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
        for (int e = tid; e < 64 * 2; e += TC_THREADS) {
            const int r = e >> 1, q = 8 * (e & 1);
            *reinterpret_cast<uint4 *>(sm + TR_W1 + kmaj_off(r, q, 2)) =
                *reinterpret_cast<const uint4 *>(w + MLP_W1S + r * MLP_S1 + q);
            *reinterpret_cast<uint4 *>(sm + TR_W3T + kmaj_off(r, q, 2)) =
                *reinterpret_cast<const uint4 *>(w + MLP_W3T + r * MLP_S1 + q);
        }
        for (int e = tid; e < 64 * 8; e += TC_THREADS) {
            const int r = e >> 3, q = 8 * (e & 7);
            *reinterpret_cast<uint4 *>(sm + TR_W2 + kmaj_off(r, q, 8)) =
                *reinterpret_cast<const uint4 *>(w + MLP_W2S + r * MLP_S2 + q);
            *reinterpret_cast<uint4 *>(sm + TR_W2T + kmaj_off(r, q, 8)) =
                *reinterpret_cast<const uint4 *>(w + MLP_W2T + r * MLP_S2 + q);
        }
        for (int e = tid; e < 16 * 8; e += TC_THREADS) {
            const int r = e >> 3, q = 8 * (e & 7);
            *reinterpret_cast<uint4 *>(sm + TR_W3 + kmaj_off(r, q, 8)) =
                r < MLP_OUT ? *reinterpret_cast<const uint4 *>(w + MLP_W3S + r * MLP_S2 + q) : z4;
        }
        // the zero columns of every tile (only the others are rewritten)
        for (int e = tid; e < TR_W1 / 16; e += TC_THREADS) reinterpret_cast<uint4 *>(sm)[e] = make_uint4(0u, 0u, 0u, 0u);
        for (int e = tid; e < (TR_B - TR_Q) / 16; e += TC_THREADS)
            reinterpret_cast<uint4 *>(sm + TR_Q)[e] = make_uint4(0u, 0u, 0u, 0u);
        float *b = reinterpret_cast<float *>(sm + TR_B);
        for (int e = tid; e < 144; e += TC_THREADS) b[e] = e < 130 ? bias[e] : 0.f;
    }
    const uint32_t bar = smem_u32(sm + TR_BAR);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(sm + TR_TMEM)), "r"(TR_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_before_sync();
    }
    fence_async_smem();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(sm + TR_TMEM);
    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
    const float *b1 = reinterpret_cast<const float *>(sm + TR_B), *b2 = b1 + 64, *b3 = b1 + 128;
    unsigned char *sT = sm + TR_T, *sQ = sm + TR_Q;
    const uint32_t aXA = smem_u32(sm + TR_XA), aD = smem_u32(sm + TR_D), aW1 = smem_u32(sm + TR_W1),
                   aW2 = smem_u32(sm + TR_W2), aW3 = smem_u32(sm + TR_W3), aW3T = smem_u32(sm + TR_W3T),
                   aW2T = smem_u32(sm + TR_W2T), aT = smem_u32(sT), aQ = smem_u32(sQ);
    constexpr uint32_t SBO_T = TR_TG * 128, SBO_Q = TR_QG * 128, SBO_D = TR_DG * 128;
    float db1[64], db2[64], db3[2] = {0.f, 0.f}, loss = 0.f;
#pragma unroll
    for (int j = 0; j < 64; j++) db1[j] = db2[j] = 0.f;
    uint32_t phase = 0;
    bool ok = true;
    int started = 0;
    const int ntiles = (nrows + TC_ROWS - 1) / TC_ROWS;
    // the rows of the next tile are loaded while the current one is worked
    uint4 xn = make_uint4(0u, 0u, 0u, 0u);
    float2 ln = make_float2(0.f, 0.f);
    if (blockIdx.x * TC_ROWS + tid < nrows) {
        xn = X[row0 + blockIdx.x * TC_ROWS + tid];
        ln = Y[row0 + blockIdx.x * TC_ROWS + tid];
    }
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int rl = tile * TC_ROWS + tid;
        const bool valid = rl < nrows;
        const uint4 xv = xn;
        const float2 lab = ln;
        {
            const int rn = rl + gridDim.x * TC_ROWS;
            if (tile + (int)gridDim.x < ntiles && rn < nrows) {
                xn = X[row0 + rn];
                ln = Y[row0 + rn];
            }
        }
        *reinterpret_cast<uint4 *>(sm + TR_XA + kmaj_off(tid, 0, 2)) = xv;   // read by layer 1 only
        tc_handoff();
        // layer 1; its commit also covers the previous tile's gradient MMAs,
        // whose operand tiles the epilogues below overwrite
        if (tid == 0) {
            mma_bf16(tmem, sdesc(aXA, 128, SBO_D), sdesc(aW1, 128, 256), idesc_bf16(128, 64), 0);
            mma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait(bar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_after_sync();
        uint64_t m1 = 0, m2 = 0;
#pragma unroll
        for (int cc = 0; cc < 2; cc++) {   // H1 = relu(D + b1) into Q, and its mask
            float v32[32];
            tmem_ld32(trow + 32 * cc, v32);
#pragma unroll
            for (int c = 2 * cc; c < 2 * cc + 2; c++) {
                const float *v = v32 + 16 * (c - 2 * cc);
                uint32_t w[8];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    w[i] = mlp_pack2(fmaxf(v[2 * i] + b1[16 * c + 2 * i], 0.f),
                                     fmaxf(v[2 * i + 1] + b1[16 * c + 2 * i + 1], 0.f));
                    m1 |= nz_bits(w[i], 16 * c + 2 * i);
                }
                st_row16(sQ, TR_QG, tid, 16 * c, w);
            }
        }
        *reinterpret_cast<uint4 *>(sQ + kmaj_off(tid, 64, TR_QG)) = xv;
        tc_handoff();
        if (tid == 0) {   // layer 2: A = Q columns 0..63
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                mma_bf16(tmem, sdesc(aQ + 256 * kk, 128, SBO_Q), sdesc(aW2 + 256 * kk, 128, 1024),
                         idesc_bf16(128, 64), kk > 0);
            mma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait(bar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_after_sync();
#pragma unroll
        for (int cc = 0; cc < 2; cc++) {   // H2 = relu(D + b2) into T columns 0..63
            float v32[32];
            tmem_ld32(trow + 32 * cc, v32);
#pragma unroll
            for (int c = 2 * cc; c < 2 * cc + 2; c++) {
                const float *v = v32 + 16 * (c - 2 * cc);
                uint32_t w[8];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    w[i] = mlp_pack2(fmaxf(v[2 * i] + b2[16 * c + 2 * i], 0.f),
                                     fmaxf(v[2 * i + 1] + b2[16 * c + 2 * i + 1], 0.f));
                    m2 |= nz_bits(w[i], 16 * c + 2 * i);
                }
                st_row16(sT, TR_TG, tid, 16 * c, w);
            }
        }
        tc_handoff();
        if (tid == 0) {   // layer 3: A = T columns 0..63
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                mma_bf16(tmem, sdesc(aT + 256 * kk, 128, SBO_T), sdesc(aW3 + 256 * kk, 128, 1024),
                         idesc_bf16(128, 16), kk > 0);
            mma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait(bar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_after_sync();
        {   // output, error, dY (the mean's 1 / rows folded in) into D
            float y[2];
            tmem_ld2(trow, y);
            float dy0 = 0.f, dy1 = 0.f;
            if (valid) {
                const float e0 = (y[0] + b3[0]) - lab.x, e1 = (y[1] + b3[1]) - lab.y;
                loss += e0 * e0 + e1 * e1;
                dy0 = 2.f * scale * e0;
                dy1 = 2.f * scale * e1;
            }
            db3[0] += dy0;
            db3[1] += dy1;
            *reinterpret_cast<uint4 *>(sm + TR_D + kmaj_off(tid, 0, TR_DG)) = make_uint4(mlp_pack2(dy0, dy1), 0u, 0u, 0u);
        }
        tc_handoff();
        if (tid == 0) {   // dH2 = dY W3
            mma_bf16(tmem, sdesc(aD, 128, SBO_D), sdesc(aW3T, 128, 256), idesc_bf16(128, 64), 0);
            mma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait(bar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_after_sync();
#pragma unroll
        for (int cc = 0; cc < 2; cc++) {   // dH2' = dH2 o relu'(H2) into T columns 64..127
            float v32[32];
            tmem_ld32(trow + 32 * cc, v32);
#pragma unroll
            for (int c = 2 * cc; c < 2 * cc + 2; c++) {
                const float *v = v32 + 16 * (c - 2 * cc);
                uint32_t w[8];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const int col = 16 * c + 2 * i;
                    const float d0 = ((m2 >> col) & 1ull) ? v[2 * i] : 0.f;
                    const float d1 = ((m2 >> (col + 1)) & 1ull) ? v[2 * i + 1] : 0.f;
                    db2[col] += d0;
                    db2[col + 1] += d1;
                    w[i] = mlp_pack2(d0, d1);
                }
                st_row16(sT, TR_TG, tid, 64 + 16 * c, w);
            }
        }
        tc_handoff();
        if (tid == 0) {   // dH1 = dH2' W2: A = T columns 64..127
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                mma_bf16(tmem, sdesc(aT + 1024 + 256 * kk, 128, SBO_T), sdesc(aW2T + 256 * kk, 128, 1024),
                         idesc_bf16(128, 64), kk > 0);
            mma_commit(bar);
        }
        ok = __syncthreads_and(mbar_wait(bar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_after_sync();
#pragma unroll
        for (int cc = 0; cc < 2; cc++) {   // dH1' = dH1 o relu'(H1) into T columns 128..191
            float v32[32];
            tmem_ld32(trow + 32 * cc, v32);
#pragma unroll
            for (int c = 2 * cc; c < 2 * cc + 2; c++) {
                const float *v = v32 + 16 * (c - 2 * cc);
                uint32_t w[8];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const int col = 16 * c + 2 * i;
                    const float d0 = ((m1 >> col) & 1ull) ? v[2 * i] : 0.f;
                    const float d1 = ((m1 >> (col + 1)) & 1ull) ? v[2 * i + 1] : 0.f;
                    db1[col] += d0;
                    db1[col + 1] += d1;
                    w[i] = mlp_pack2(d0, d1);
                }
                st_row16(sT, TR_TG, tid, 128 + 16 * c, w);
            }
        }
        tc_handoff();
        if (tid == 0) {   // weight gradients of the tile, K = its rows in steps of 16 (two 8-row groups)
#pragma unroll
            for (int kk = 0; kk < 8; kk++)
                mma_bf16(tmem + TR_GA, sdesc_mn(aT + 1024 + 2 * SBO_T * kk, SBO_T),
                         sdesc_mn(aQ + 2 * SBO_Q * kk, SBO_Q), idesc_bf16_mn(128, 80), started | kk);
#pragma unroll
            for (int kk = 0; kk < 8; kk++)
                mma_bf16(tmem + TR_GB, sdesc_mn(aT + 2 * SBO_T * kk, SBO_T), sdesc_mn(aD + 2 * SBO_D * kk, SBO_D),
                         idesc_bf16_mn(128, 16), started | kk);
        }
        started = 1;
    }
    if (ok && started) {
        if (tid == 0) mma_commit(bar);
        ok = __syncthreads_and(mbar_wait(bar, phase));
        phase ^= 1;
    }
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(bar, phase ^ 1);   // the phase that timed out
    } else {
        tc_after_sync();
        float *P = partials + (size_t)blockIdx.x * (MLP_NPARAM + 1);
        if (warp < 2) {   // rows 0..63 of G_a: dW2[tid][:]; of G_b: dW3[:][tid]
#pragma unroll
            for (int c = 0; c < 4; c++) {
                float v[16];
                tmem_ld16(trow + TR_GA + 16 * c, v);
#pragma unroll
                for (int j = 0; j < 16; j++) P[MLP_P_W2 + tid * 64 + 16 * c + j] = started ? v[j] : 0.f;
            }
            float v3[2];
            tmem_ld2(trow + TR_GB, v3);
            P[MLP_P_W3 + tid] = started ? v3[0] : 0.f;
            P[MLP_P_W3 + 64 + tid] = started ? v3[1] : 0.f;
        } else {          // rows 64..127 of G_a, columns 64..71: dW1[tid - 64][:]
            float v[16];
            tmem_ld16(trow + TR_GA + 64, v);
#pragma unroll
            for (int j = 0; j < MLP_IN; j++) P[MLP_P_W1 + (tid - 64) * MLP_IN + j] = started ? v[j] : 0.f;
        }
        // bias gradients and the loss: per-thread sums, then added over the
        // threads in row order (T and Q are free now)
        float *S = reinterpret_cast<float *>(sT);
#pragma unroll
        for (int j = 0; j < 64; j++) {
            S[tid * TR_SUMS + j] = db1[j];
            S[tid * TR_SUMS + 64 + j] = db2[j];
        }
        S[tid * TR_SUMS + 128] = db3[0];
        S[tid * TR_SUMS + 129] = db3[1];
        S[tid * TR_SUMS + 130] = loss;
        __syncthreads();
        for (int p = tid; p < TR_SUMS; p += TC_THREADS) {
            float s = 0.f;
#pragma unroll 16
            for (int r = 0; r < TC_ROWS; r++) s += S[r * TR_SUMS + p];
            const int dst = p < 64 ? MLP_P_B1 + p : (p < 128 ? MLP_P_B2 + p - 64 : (p < 130 ? MLP_P_B3 + p - 128 : MLP_NPARAM));
            P[dst] = s;
        }
    }
    tc_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TR_TMEM_COLS) : "memory");
    }
}

// Host launcher: `nblk` CTAs (two per SM at most: 99 KB of shared memory and
// 256 TMEM columns each) over the batch's tiles; each writes its partial
// gradient row of `partials`.
mdz_status mdz_mlp_train_tc(mdz_ctx *ctx, const unsigned char *packed, const uint4 *X, const float2 *Y,
                            long long row0, int nrows, float scale, float *partials, int nblk, int *d_err,
                            cudaStream_t st) {
    static bool attr_set = false;
    if (!attr_set) {
        MDZ_CUDA(ctx, cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TR_BYTES));
        attr_set = true;
    }
    k_mlp_train_tc<<<nblk, TC_THREADS, TR_BYTES, st>>>(packed, X, Y, row0, nrows, scale, partials, d_err);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}
