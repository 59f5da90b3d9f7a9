// Forward GEMMs of the learned surrogate on the 5th-generation tensor cores (tcgen05).
//
// C[M x N] = act(A[M x K] * B[N x K]^T + bias): A the bf16 activations (K contiguous), B a
// bf16 weight matrix in its [out x in] layout (K contiguous), FP32 accumulation in tensor
// memory (TMEM), epilogue + bias, GELU (tanh form, mlp_common.cuh) or identity, bf16 or
// FP32 output.
//
// One CTA of 128 threads computes a 128 x BN tile.  K is consumed 32 at a time through a
// 4-stage ring in shared memory: every thread copies 16-byte chunks two k-blocks ahead with
// cp.async into the canonical no-swizzle K-major layout (8 x 16-byte core matrices, the
// two core matrices of a 16-wide K slice adjacent: LBO = 128 B, 8-row groups 512 B apart:
// SBO), then one thread issues two tcgen05.mma (M = 128, N = BN, K = 16 each) and commits
// them to the stage's mbarrier, which releases the stage for refilling.  After the last
// commit, each warp reads its 32 TMEM lanes (rows) with tcgen05.ld and runs the epilogue.
//
// Every mbarrier wait is bounded: on a timeout the block agrees (a barrier reduction),
// stops issuing, drains its copies, frees its TMEM and records the failure in a device
// error word that the host reads (rbf_mlp_tc_status).
#include <cuda_bf16.h>

#include <algorithm>

#include "mlp_common.cuh"
#include "rbf_internal.cuh"

namespace {

constexpr int TC_M = 128, TC_KB = 32, TC_STAGES = 4, TC_THREADS = 128;
constexpr unsigned kWaitLimit = 1u << 26;  // try_wait polls before a wait is declared failed

__device__ unsigned int g_tc_error;  // set to 1 when a wait ran out

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: canonical layout without swizzle (version 1)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: D FP32, A and B bf16, both K-major, M x N
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, bool valid) {
    const int n = valid ? 16 : 0;  // 0: zero-fill, nothing read
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned it = 0; it < kWaitLimit; it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <int BN>
__global__ void __launch_bounds__(TC_THREADS) gemm_tc_kernel(int M, int N, int K, const __nv_bfloat16 *__restrict__ A,
                                                             int lda, const __nv_bfloat16 *__restrict__ B, int ldb,
                                                             const float *__restrict__ bias, int gelu_on,
                                                             float *__restrict__ Cf, __nv_bfloat16 *__restrict__ Cb,
                                                             int ldc) {
    constexpr int A_BYTES = TC_M * TC_KB * 2, B_BYTES = BN * TC_KB * 2, STAGE = A_BYTES + B_BYTES;
    extern __shared__ __align__(128) char smem[];
    __shared__ __align__(8) unsigned long long bars[TC_STAGES];
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * TC_M, n0 = blockIdx.x * BN;
    const int nkb = K / TC_KB;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        for (int s = 0; s < TC_STAGES; s++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bars[s])));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_slot;

    // copies of k-block kb into its stage: A rows (128 x 4 chunks) then B rows (BN x 4 chunks)
    auto load_stage = [&](int kb) {
        const int s = kb % TC_STAGES;
        const uint32_t base = smem_u32(smem + s * STAGE);
        const int k0 = kb * TC_KB;
        for (int c = tid; c < (TC_M + BN) * 4; c += TC_THREADS) {
            const int row = c >> 2, kc = c & 3;
            if (row < TC_M) {
                const int gr = m0 + row;
                const bool ok = gr < M;
                cp_async16(base + (uint32_t)(((row & 7) * 16) + (kc * 128) + ((row >> 3) * 512)),
                           A + (size_t)(ok ? gr : 0) * lda + k0 + kc * 8, ok);
            } else {
                const int br = row - TC_M, gn = n0 + br;
                const bool ok = gn < N;
                cp_async16(base + A_BYTES + (uint32_t)(((br & 7) * 16) + (kc * 128) + ((br >> 3) * 512)),
                           B + (size_t)(ok ? gn : 0) * ldb + k0 + kc * 8, ok);
            }
        }
    };

    // copies run TC_AHEAD k-blocks ahead of the MMAs; a refilled stage was last read by the
    // MMAs of k-block next - STAGES, two blocks before the one being issued, so one block of
    // MMAs stays in flight while the next is issued
    constexpr int TC_AHEAD = 2;
    int failed = 0;
    for (int kb = 0; kb < TC_AHEAD; kb++) {
        if (kb < nkb) load_stage(kb);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    for (int kb = 0; kb < nkb; kb++) {
        const int next = kb + TC_AHEAD;
        bool to = false;
        if (next < nkb) {
            // use number next / STAGES of the stage: wait for the completion of use - 1
            if (next >= TC_STAGES) to = !mbar_wait(smem_u32(&bars[next % TC_STAGES]), ((next / TC_STAGES) - 1) & 1);
            if (!to) load_stage(next);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group %0;\n" ::"n"(TC_AHEAD) : "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        if (__syncthreads_or(to)) {
            failed = 1;
            break;
        }
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int s = kb % TC_STAGES;
            const uint32_t a0 = smem_u32(smem + s * STAGE), b0 = a0 + A_BYTES;
#pragma unroll
            for (int j = 0; j < TC_KB / 16; j++) {
                const uint64_t ad = smem_desc(a0 + j * 256, 128, 512), bd = smem_desc(b0 + j * 256, 128, 512);
                const uint32_t acc = (kb > 0 || j > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(instr_desc(TC_M, BN)), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&bars[s]))
                         : "memory");
        }
    }
    if (!failed && nkb > 0) {
        const int last = nkb - 1;
        const bool to = !mbar_wait(smem_u32(&bars[last % TC_STAGES]), (last / TC_STAGES) & 1);
        if (__syncthreads_or(to)) failed = 1;
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (!failed) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t v[16];
            const uint32_t addr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(addr));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            const int col = n0 + c0;
            if (row < M && col < N) {
                float o[16];
                if (bias && col + 16 <= N) {
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const float4 bv = __ldg(reinterpret_cast<const float4 *>(bias + col) + j);
                        o[4 * j] = __uint_as_float(v[4 * j]) + bv.x;
                        o[4 * j + 1] = __uint_as_float(v[4 * j + 1]) + bv.y;
                        o[4 * j + 2] = __uint_as_float(v[4 * j + 2]) + bv.z;
                        o[4 * j + 3] = __uint_as_float(v[4 * j + 3]) + bv.w;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        o[j] = __uint_as_float(v[j]) + (bias && col + j < N ? bias[col + j] : 0.0f);
                }
                if (gelu_on)
#pragma unroll
                    for (int j = 0; j < 16; j++) o[j] = gelu(o[j]);
                if (Cb) {
                    __nv_bfloat16 *dst = Cb + (size_t)row * ldc + col;
                    if (col + 16 <= N) {
                        uint4 w[2];
                        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(w);
#pragma unroll
                        for (int j = 0; j < 8; j++) h[j] = __floats2bfloat162_rn(o[2 * j], o[2 * j + 1]);
                        reinterpret_cast<uint4 *>(dst)[0] = w[0];
                        reinterpret_cast<uint4 *>(dst)[1] = w[1];
                    } else {
                        for (int j = 0; j < 16 && col + j < N; j++) dst[j] = __float2bfloat16_rn(o[j]);
                    }
                } else {
                    float *dst = Cf + (size_t)row * ldc + col;
                    if (col + 16 <= N) {
#pragma unroll
                        for (int j = 0; j < 4; j++)
                            reinterpret_cast<float4 *>(dst)[j] =
                                make_float4(o[4 * j], o[4 * j + 1], o[4 * j + 2], o[4 * j + 3]);
                    } else {
                        for (int j = 0; j < 16 && col + j < N; j++) dst[j] = o[j];
                    }
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(&g_tc_error, 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN));
}

template <int BN>
int launch_tc(rbf_ctx *ctx, int M, int N, int K, const void *A, int lda, const void *B, int ldb, const float *bias,
              int gelu_on, float *Cf, void *Cb, int ldc) {
    constexpr size_t smem = (size_t)TC_STAGES * (TC_M * TC_KB * 2 + BN * TC_KB * 2);
    RBF_CUDA(ctx, cudaFuncSetAttribute(gemm_tc_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((N + BN - 1) / BN, (M + TC_M - 1) / TC_M);
    gemm_tc_kernel<BN><<<grid, TC_THREADS, smem, ctx->stream>>>(M, N, K, (const __nv_bfloat16 *)A, lda,
                                                                (const __nv_bfloat16 *)B, ldb, bias, gelu_on, Cf,
                                                                (__nv_bfloat16 *)Cb, ldc);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

}  // namespace

extern "C" {

int rbf_mlp_gemm_tc(rbf_ctx *ctx, int32_t M, int32_t N, int32_t K, const void *A, int32_t lda, const void *B,
                    int32_t ldb, const float *bias, int32_t gelu_on, float *Cf, void *Cb, int32_t ldc) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    if (M < 0 || N < 1 || K < TC_KB || K % TC_KB != 0)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "gemm_tc: K must be a positive multiple of %d", TC_KB);
    if (lda % 8 || ldb % 8 || lda < K || ldb < K || ((uintptr_t)A & 15) || ((uintptr_t)B & 15))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "gemm_tc: operands need 16-byte aligned rows (ld multiple of 8, >= K)");
    if ((Cf == nullptr) == (Cb == nullptr)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "gemm_tc: give exactly one output");
    if (bias && ((uintptr_t)bias & 15)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "gemm_tc: bias must be 16-byte aligned");
    if (ldc < N || (Cb && ((ldc % 8) || ((uintptr_t)Cb & 15))) || (Cf && ((ldc % 4) || ((uintptr_t)Cf & 15))))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "gemm_tc: output rows must be 16-byte aligned");
    if (M == 0) return RBF_OK;
    if (N <= 32) return launch_tc<32>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
    if (N <= 64) return launch_tc<64>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
    if (N <= 128) return launch_tc<128>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
    return launch_tc<256>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
}

// 0: every tensor-core GEMM since the last call completed; 1: one gave up waiting (its
// output is incomplete).  Synchronises the context's stream; clears the flag.
int rbf_mlp_tc_status(rbf_ctx *ctx, int32_t *failed) {
    if (!ctx || !failed) return RBF_ERR_ARGUMENT;
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    unsigned int h = 0, z = 0;
    RBF_CUDA(ctx, cudaMemcpyFromSymbol(&h, g_tc_error, sizeof h));
    RBF_CUDA(ctx, cudaMemcpyToSymbol(g_tc_error, &z, sizeof z));
    *failed = (int32_t)h;
    return RBF_OK;
}

}  // extern "C"
