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
        mbar_wait(bar, phase);
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
