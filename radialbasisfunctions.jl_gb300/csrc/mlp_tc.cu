// Forward GEMMs of the learned surrogate on the 5th-generation tensor cores (tcgen05).
//
// C[M x N] = act(A[M x K] * B[N x K]^T + bias): A the bf16 activations (K contiguous), B a
// bf16 weight matrix in its [out x in] layout (K contiguous), FP32 accumulation in tensor
// memory (TMEM), epilogue + bias, GELU (tanh form, mlp_common.cuh) or identity, bf16 or
// FP32 output.
//
// One CTA of 128 threads computes a 128 x BN tile.  K is consumed 32 at a time through a
// 4-stage ring in shared memory filled by TMA: a stage holds, for A and for B, four boxes of
// 8 K-elements (16 bytes) x all tile rows, which is the canonical no-swizzle K-major layout
// of tcgen05 directly (8 x 16-byte core matrices; core matrices along K one box apart:
// LBO; 8-row groups 128 bytes apart: SBO).  One thread runs the pipeline: it arms a stage's
// "full" mbarrier with the expected bytes and issues its 8 box loads, waits for a stage to
// land, issues two tcgen05.mma (M = 128, N = BN, K = 16 each) and commits them to the
// stage's "empty" mbarrier, which it waits on before refilling the stage.  Rows past M
// (and past N) are zero-filled by TMA.  After the last commit, each warp reads its 32 TMEM
// lanes (rows) with tcgen05.ld, runs the epilogue into a shared tile, and the block writes
// the tile out row by row (coalesced).
//
// Every mbarrier wait is bounded: on a timeout the block agrees (a barrier reduction),
// stops issuing, frees its TMEM and records the failure in a device error word that the
// host reads (rbf_mlp_tc_status).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

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

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void mbar_expect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
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
__global__ void __launch_bounds__(TC_THREADS) gemm_tc_kernel(const __grid_constant__ CUtensorMap mapA,
                                                             const __grid_constant__ CUtensorMap mapB, int M, int N,
                                                             int K, const float *__restrict__ bias, int gelu_on,
                                                             float *__restrict__ Cf, __nv_bfloat16 *__restrict__ Cb,
                                                             int ldc) {
    constexpr int A_BYTES = TC_M * TC_KB * 2, B_BYTES = BN * TC_KB * 2, STAGE = A_BYTES + B_BYTES;
    extern __shared__ __align__(1024) char smem[];
    __shared__ __align__(8) unsigned long long full[TC_STAGES], empty[TC_STAGES];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * TC_M, n0 = blockIdx.x * BN;
    const int nkb = K / TC_KB;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        for (int s = 0; s < TC_STAGES; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        // TMA writes need 128-byte aligned destinations (the stage offsets are multiples of 2 KB)
        s_fail = (smem_u32(smem) & 1023u) ? 1 : 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_slot;

    if (tid == 0 && !s_fail) {
        auto issue = [&](int kb) {
            const int s = kb % TC_STAGES;
            const uint32_t a0 = smem_u32(smem + s * STAGE), b0 = a0 + A_BYTES, bar = smem_u32(&full[s]);
            mbar_expect(bar, STAGE);
#pragma unroll
            for (int kc = 0; kc < TC_KB / 8; kc++) {
                const int x = kb * TC_KB + kc * 8;  // 8 bf16 = 16 bytes: TMA x stays 16-byte aligned
                tma_load_2d(a0 + kc * (TC_M * 16), &mapA, x, m0, bar);
                tma_load_2d(b0 + kc * (BN * 16), &mapB, x, n0, bar);
            }
        };
        int fail = 0;
        for (int kb = 0; kb < nkb && kb < TC_STAGES; kb++) issue(kb);
        for (int kb = 0; kb < nkb && !fail; kb++) {
            const int s = kb % TC_STAGES;
            if (!mbar_wait(smem_u32(&full[s]), (kb / TC_STAGES) & 1)) {
                fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t a0 = smem_u32(smem + s * STAGE), b0 = a0 + A_BYTES;
#pragma unroll
            for (int j = 0; j < TC_KB / 16; j++) {
                // K slice 16j..16j+15 = boxes 2j, 2j+1: core matrices along K one box apart (LBO),
                // 8-row groups 128 bytes apart (SBO)
                const uint64_t ad = smem_desc(a0 + 2 * j * (TC_M * 16), TC_M * 16, 128);
                const uint64_t bd = smem_desc(b0 + 2 * j * (BN * 16), BN * 16, 128);
                const uint32_t acc = (kb > 0 || j > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(instr_desc(TC_M, BN)), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&empty[s]))
                         : "memory");
            // refill the stage of the previous k-block once its MMAs have read it
            if (kb >= 1) {
                const int prev = kb - 1, next = prev + TC_STAGES;
                if (next < nkb) {
                    if (!mbar_wait(smem_u32(&empty[prev % TC_STAGES]), (prev / TC_STAGES) & 1)) {
                        fail = 1;
                        break;
                    }
                    issue(next);
                }
            }
        }
        s_fail = fail;
    }
    __syncthreads();
    int failed = s_fail;
    if (!failed && nkb > 0) {
        const int last = nkb - 1;
        const bool to = !mbar_wait(smem_u32(&empty[last % TC_STAGES]), (last / TC_STAGES) & 1);
        if (__syncthreads_or(to)) failed = 1;
    }
    if (!failed) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // Epilogue, two passes through the (now idle) stage memory: each thread finishes its
        // TMEM row into a padded shared tile (row stride an odd number of 16-byte units, so
        // the 16-byte writes of a quarter-warp hit distinct banks), then each warp writes
        // whole rows to global memory, contiguous 16-byte pieces across its lanes.
        const int r_loc = warp * 32 + lane;
        constexpr int LDB = BN + 8;  // bf16 tile row stride (elements)
        constexpr int LDF = BN + 4;  // fp32 tile row stride (elements)
        __nv_bfloat16 *tb = reinterpret_cast<__nv_bfloat16 *>(smem);
        float *tf = reinterpret_cast<float *>(smem);
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
                uint4 w[2];
                __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(w);
#pragma unroll
                for (int j = 0; j < 8; j++) h[j] = __floats2bfloat162_rn(o[2 * j], o[2 * j + 1]);
                uint4 *dst = reinterpret_cast<uint4 *>(tb + r_loc * LDB + c0);
                dst[0] = w[0];
                dst[1] = w[1];
            } else {
                float4 *dst = reinterpret_cast<float4 *>(tf + r_loc * LDF + c0);
#pragma unroll
                for (int j = 0; j < 4; j++) dst[j] = make_float4(o[4 * j], o[4 * j + 1], o[4 * j + 2], o[4 * j + 3]);
            }
        }
        __syncthreads();
        const int ncol = min(BN, N - n0);
#pragma unroll 1
        for (int r = warp; r < TC_M; r += TC_THREADS / 32) {
            const int grow = m0 + r;
            if (grow >= M) break;
            if (Cb) {
                __nv_bfloat16 *g = Cb + (size_t)grow * ldc + n0;
                const __nv_bfloat16 *t = tb + r * LDB;
                for (int u = lane; u < BN / 8; u += 32) {
                    if (u * 8 + 8 <= ncol)
                        reinterpret_cast<uint4 *>(g)[u] = reinterpret_cast<const uint4 *>(t)[u];
                    else
                        for (int j = u * 8; j < ncol; j++) g[j] = t[j];
                }
            } else {
                float *g = Cf + (size_t)grow * ldc + n0;
                const float *t = tf + r * LDF;
                for (int u = lane; u < BN / 4; u += 32) {
                    if (u * 4 + 4 <= ncol)
                        reinterpret_cast<float4 *>(g)[u] = reinterpret_cast<const float4 *>(t)[u];
                    else
                        for (int j = u * 4; j < ncol; j++) g[j] = t[j];
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

// ---------------------------------------------------------------------------------------
// Persistent, warp-specialised variant for K <= 256 and N <= 256 (the surrogate's layers):
// the whole weight matrix B stays in shared memory (loaded once per CTA), only the
// activations stream through a TMA ring, and two TMEM accumulators let the epilogue of one
// 128-row tile overlap the MMAs of the next.  Operands use the 128-byte swizzled K-major
// layout: one TMA box of 64 K-elements (128 bytes) x all rows per stage instead of 16-byte
// boxes (the canonical swizzled layout: 8-row groups 1024 bytes apart, K steps of 16 = 32
// bytes inside the swizzle atom); K beyond the operand's width is zero-filled by TMA.  One CTA per SM; warp 0 issues the TMA loads,
// warp 1 the MMAs (and owns the TMEM allocation), the other 8 or 16 run the epilogue: warp w reads
// TMEM lane quadrant w % 4 (the quadrant a warp may access) and a part of the columns, and
// stores straight to global memory (each row's 16-column pieces are 32- or 64-byte runs).
// Barriers: full/empty per ring stage (TMA <-> MMA), bfull (B resident), accf/acce per
// accumulator (MMA <-> epilogue).  Waits are bounded; a wait that runs out raises a shared
// abort flag that every role polls, the producer then drains its copies still in flight,
// and the failure is recorded in g_tc_error.
// ---------------------------------------------------------------------------------------
constexpr int TP_STAGES = 3, TP_KB = 64;
// per epilogue warp: 32 rows x 64 bytes of output staged (row stride 80 bytes) so that the
// global writes go out as full 64-byte row pieces, four lanes per row
constexpr int TP_STG_ROW = 80, TP_STG_WARP = 32 * TP_STG_ROW;
// epilogue warps: four per TMEM lane quadrant for wide tiles (each a quarter of the columns),
// two for narrow ones
__host__ __device__ constexpr int tp_epi_warps(int bn) { return bn >= 128 ? 16 : 8; }
__host__ __device__ constexpr int tp_threads(int bn) { return (2 + tp_epi_warps(bn)) * 32; }

// shared-memory matrix descriptor, 128-byte swizzle, K-major (LBO unused, SBO = 8 rows x 128 B)
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3fffu) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}

__device__ __forceinline__ bool mbar_wait_abort(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                                unsigned limit = kWaitLimit) {
    for (unsigned it = 0; it < limit; it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255u) == 255u && *abort_flag) return false;
    }
    *abort_flag = 1;
    return false;
}

template <int BN>
__global__ void __launch_bounds__(tp_threads(BN), 1)
    gemm_tc_persistent_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int M,
                              int N, int K, const float *__restrict__ bias, int gelu_on, float *__restrict__ Cf,
                              __nv_bfloat16 *__restrict__ Cb, int ldc, unsigned wait_limit, int issue_loads) {
    // issue_loads == 0 (self-test only): the producer issues no copy at all, so every wait of
    // the other roles runs out after wait_limit polls with nothing in flight
    constexpr int A_BYTES = TC_M * TP_KB * 2, B_BOX = BN * TP_KB * 2;
    constexpr uint32_t TMEM_COLS = 2 * BN;  // two accumulators; BN in {32, 64, 128, 256}
    constexpr int EPI = tp_epi_warps(BN), PARTS = EPI / 4, PCOLS = BN / PARTS;
    static_assert(PCOLS >= 16 && PCOLS % 16 == 0, "16-column pieces per epilogue warp");
    extern __shared__ __align__(1024) char smem[];
    __shared__ __align__(8) unsigned long long full[TP_STAGES], empty[TP_STAGES], bfull, accf[2], acce[2];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    __shared__ int consumed;  // ring k-blocks the MMA warp has taken (for the producer's drain)
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nkb = (K + TP_KB - 1) / TP_KB;
    const int ntiles = (M + TC_M - 1) / TC_M;
    char *bsm = smem;                             // B: nkb swizzled boxes of BN rows x 128 bytes
    char *asm_ring = smem + (size_t)nkb * B_BOX;  // A ring (boxes are multiples of 4 KB)
    char *stg_all = asm_ring + TP_STAGES * A_BYTES;  // epilogue staging, TP_STG_WARP per warp

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        for (int s = 0; s < TP_STAGES; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bfull)));
        for (int b = 0; b < 2; b++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&accf[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&acce[b])), "r"(EPI * 32));
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        abort_flag = (smem_u32(smem) & 1023u) ? 1 : 0;  // TMA destinations need 128-byte alignment
        consumed = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_slot;
    int issued = 0;

    if (warp == 0) {
        if (lane == 0 && !abort_flag && issue_loads) {
            // B once: nkb boxes of 64 K-elements x BN rows (zero-filled past K)
            const uint32_t bb = smem_u32(&bfull);
            mbar_expect(bb, (uint32_t)nkb * B_BOX);
            for (int kb = 0; kb < nkb; kb++) tma_load_2d(smem_u32(bsm) + kb * B_BOX, &mapB, kb * TP_KB, 0, bb);
            int it = 0;
            for (int t = blockIdx.x; t < ntiles && !abort_flag; t += gridDim.x) {
                const int m0 = t * TC_M;
                for (int kb = 0; kb < nkb; kb++, it++) {
                    const int s = it % TP_STAGES;
                    if (it >= TP_STAGES &&
                        !mbar_wait_abort(smem_u32(&empty[s]), ((it / TP_STAGES) - 1) & 1, &abort_flag, wait_limit))
                        break;
                    const uint32_t a0 = smem_u32(asm_ring + s * A_BYTES), bar = smem_u32(&full[s]);
                    mbar_expect(bar, A_BYTES);
                    tma_load_2d(a0, &mapA, kb * TP_KB, m0, bar);
                    issued = it + 1;
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && !abort_flag && mbar_wait_abort(smem_u32(&bfull), 0, &abort_flag, wait_limit)) {
            int it = 0, tc = 0;
            for (int t = blockIdx.x; t < ntiles && !abort_flag; t += gridDim.x, tc++) {
                const int buf = tc & 1;
                if (tc >= 2 && !mbar_wait_abort(smem_u32(&acce[buf]), ((tc >> 1) - 1) & 1, &abort_flag, wait_limit)) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d = tmem + (uint32_t)(buf * BN);
                bool ok = true;
                for (int kb = 0; kb < nkb; kb++, it++) {
                    const int s = it % TP_STAGES;
                    if (!mbar_wait_abort(smem_u32(&full[s]), (it / TP_STAGES) & 1, &abort_flag, wait_limit)) {
                        ok = false;
                        break;
                    }
                    consumed = it + 1;
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t a0 = smem_u32(asm_ring + s * A_BYTES), b0 = smem_u32(bsm + kb * B_BOX);
#pragma unroll
                    for (int j = 0; j < TP_KB / 16; j++) {  // K slice 16j..16j+15: 32 bytes into the atom
                        const uint64_t ad = smem_desc_sw128(a0 + 32 * j);
                        const uint64_t bd = smem_desc_sw128(b0 + 32 * j);
                        const uint32_t acc = (kb > 0 || j > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                            "l"(ad), "l"(bd), "r"(instr_desc(TC_M, BN)), "r"(acc)
                            : "memory");
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                     smem_u32(&empty[s]))
                                 : "memory");
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 smem_u32(&accf[buf]))
                             : "memory");
            }
        }
    } else {
        // epilogue: TMEM lane quadrant q, columns [part * PCOLS, (part + 1) * PCOLS)
        const int q = warp & 3, part = (warp - 2) >> 2;
        const int c_begin = part * PCOLS, c_end = c_begin + PCOLS;
        int tc = 0;
        for (int t = blockIdx.x; t < ntiles && !abort_flag; t += gridDim.x, tc++) {
            const int buf = tc & 1;
            if (!mbar_wait_abort(smem_u32(&accf[buf]), (tc >> 1) & 1, &abort_flag, wait_limit)) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            char *stg = stg_all + (warp - 2) * TP_STG_WARP;
            const int esz = Cb ? 2 : 4, seg_cols = 64 / esz;  // 32 bf16 or 16 FP32 columns per piece
            for (int s0 = c_begin; s0 < c_end; s0 += seg_cols) {
                for (int c0 = s0; c0 < s0 + seg_cols; c0 += 16) {
                    uint32_t v[16];
                    const uint32_t addr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * BN + c0);
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                        "[%16];\n"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                          "=r"(v[15])
                        : "r"(addr));
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    float o[16];
                    if (bias && c0 + 16 <= N) {
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const float4 bv = __ldg(reinterpret_cast<const float4 *>(bias + c0) + j);
                            o[4 * j] = __uint_as_float(v[4 * j]) + bv.x;
                            o[4 * j + 1] = __uint_as_float(v[4 * j + 1]) + bv.y;
                            o[4 * j + 2] = __uint_as_float(v[4 * j + 2]) + bv.z;
                            o[4 * j + 3] = __uint_as_float(v[4 * j + 3]) + bv.w;
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < 16; j++)
                            o[j] = __uint_as_float(v[j]) + (bias && c0 + j < N ? bias[c0 + j] : 0.0f);
                    }
                    if (gelu_on)
#pragma unroll
                        for (int j = 0; j < 16; j++) o[j] = gelu(o[j]);
                    char *dst = stg + lane * TP_STG_ROW + (c0 - s0) * esz;
                    if (Cb) {
                        uint4 w[2];
                        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(w);
#pragma unroll
                        for (int j = 0; j < 8; j++) h[j] = __floats2bfloat162_rn(o[2 * j], o[2 * j + 1]);
                        reinterpret_cast<uint4 *>(dst)[0] = w[0];
                        reinterpret_cast<uint4 *>(dst)[1] = w[1];
                    } else {
#pragma unroll
                        for (int j = 0; j < 4; j++)
                            reinterpret_cast<float4 *>(dst)[j] = make_float4(o[4 * j], o[4 * j + 1], o[4 * j + 2], o[4 * j + 3]);
                    }
                }
                __syncwarp();
                // 8 rows per instruction, each row's 64 bytes by four consecutive lanes
#pragma unroll
                for (int r8 = 0; r8 < 4; r8++) {
                    const int rr = r8 * 8 + (lane >> 2), piece = lane & 3;
                    const int grow = t * TC_M + q * 32 + rr;
                    const int col = s0 + piece * (16 / esz);
                    const uint4 val = *reinterpret_cast<const uint4 *>(stg + rr * TP_STG_ROW + piece * 16);
                    if (grow < M) {
                        if (Cb) {
                            __nv_bfloat16 *g = Cb + (size_t)grow * ldc + col;
                            if (col + 8 <= N) {
                                *reinterpret_cast<uint4 *>(g) = val;
                            } else {
                                const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&val);
                                for (int j = 0; j < 8 && col + j < N; j++) g[j] = e[j];
                            }
                        } else {
                            float *g = Cf + (size_t)grow * ldc + col;
                            if (col + 4 <= N) {
                                *reinterpret_cast<uint4 *>(g) = val;
                            } else {
                                const float *e = reinterpret_cast<const float *>(&val);
                                for (int j = 0; j < 4 && col + j < N; j++) g[j] = e[j];
                            }
                        }
                    }
                }
                __syncwarp();
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(&acce[buf])) : "memory");
        }
    }
    __syncthreads();
    if (abort_flag) {
        // drain: wait (bounded) for the copies the producer issued but the MMA warp never took
        if (warp == 0 && lane == 0) {
            for (int it = consumed; it < issued; it++) {
                const int s = it % TP_STAGES;
                volatile int never = 0;
                mbar_wait_abort(smem_u32(&full[s]), (it / TP_STAGES) & 1, &never);  // full limit
            }
            atomicExch(&g_tc_error, 1u);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS));
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder(rbf_ctx *ctx) {
    static void *fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            fn = nullptr;
    }
    if (!fn) rbf_fail(ctx, RBF_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
}

// 2-D bf16 tensor map over a row-major [rows x cols] matrix with row stride ld, boxes of
// 8 columns (16 bytes) x box_rows rows, no swizzle, zero fill outside
int make_map(rbf_ctx *ctx, CUtensorMap *map, const void *base, int rows, int cols, int ld, int box_rows,
             bool sw128 = false) {
    auto enc = tensor_map_encoder(ctx);
    if (!enc) return RBF_ERR_CUDA;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {sw128 ? 64u : 8u, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, sw128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return rbf_fail(ctx, RBF_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return RBF_OK;
}

template <int BN>
int launch_tc(rbf_ctx *ctx, int M, int N, int K, const void *A, int lda, const void *B, int ldb, const float *bias,
              int gelu_on, float *Cf, void *Cb, int ldc) {
    // the stage ring, and afterwards the output tile of the epilogue (row strides BN + 8
    // bf16 or BN + 4 FP32): the larger of the two
    constexpr size_t ring = (size_t)TC_STAGES * (TC_M * TC_KB * 2 + BN * TC_KB * 2);
    const size_t tile = Cb ? (size_t)TC_M * (BN + 8) * 2 : (size_t)TC_M * (BN + 4) * 4;
    const size_t smem = std::max(ring, tile);
    CUtensorMap ma, mb;
    RBF_TRY(make_map(ctx, &ma, A, M, K, lda, TC_M));
    RBF_TRY(make_map(ctx, &mb, B, N, K, ldb, BN));
    RBF_CUDA(ctx, cudaFuncSetAttribute(gemm_tc_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((N + BN - 1) / BN, (M + TC_M - 1) / TC_M);
    gemm_tc_kernel<BN><<<grid, TC_THREADS, smem, ctx->stream>>>(ma, mb, M, N, K, bias, gelu_on, Cf,
                                                                (__nv_bfloat16 *)Cb, ldc);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

template <int BN>
int launch_tc_persistent(rbf_ctx *ctx, int M, int N, int K, const void *A, int lda, const void *B, int ldb,
                         const float *bias, int gelu_on, float *Cf, void *Cb, int ldc, unsigned wait_limit = kWaitLimit,
                         int issue_loads = 1) {
    const int nkb = (K + TP_KB - 1) / TP_KB;
    const size_t smem = (size_t)nkb * BN * TP_KB * 2 + (size_t)TP_STAGES * TC_M * TP_KB * 2 +
                        (size_t)tp_epi_warps(BN) * TP_STG_WARP;
    CUtensorMap ma, mb;
    RBF_TRY(make_map(ctx, &ma, A, M, K, lda, TC_M, true));
    RBF_TRY(make_map(ctx, &mb, B, N, K, ldb, BN, true));
    RBF_CUDA(ctx, cudaFuncSetAttribute(gemm_tc_persistent_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    const int ntiles = (M + TC_M - 1) / TC_M;
    const int grid = std::max(1, std::min(ntiles, ctx->num_sms));
    gemm_tc_persistent_kernel<BN><<<grid, tp_threads(BN), smem, ctx->stream>>>(ma, mb, M, N, K, bias, gelu_on, Cf,
                                                                           (__nv_bfloat16 *)Cb, ldc, wait_limit,
                                                                           issue_loads);
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
    if (K <= 256) {  // the weights fit in shared memory: the persistent kernel
        if (N <= 32) return launch_tc_persistent<32>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
        if (N <= 64) return launch_tc_persistent<64>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
        if (N <= 128) return launch_tc_persistent<128>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
        if (N <= 256) return launch_tc_persistent<256>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
    }
    if (N <= 32) return launch_tc<32>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
    if (N <= 64) return launch_tc<64>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
    if (N <= 128) return launch_tc<128>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
    return launch_tc<256>(ctx, M, N, K, A, lda, B, ldb, bias, gelu_on, Cf, Cb, ldc);
}

// Self-test of the bounded waits: one persistent GEMM (M = 256, N = 32, K = 64) whose
// producer issues no copy, with a wait limit of 4096 polls.  The MMA warp's wait for the
// resident weights runs out, it raises the abort flag, the epilogue warps give up their
// waits, and the block frees its tensor memory and returns: no copy and no MMA was ever in
// flight.  *failed receives the error flag that launch left (1 when the timeout path works).
int rbf_mlp_tc_selftest_timeout(rbf_ctx *ctx, int32_t *failed) {
    if (!ctx || !failed) return RBF_ERR_ARGUMENT;
    RBF_CUDA(ctx, cudaSetDevice(ctx->device));
    int32_t before = 0;
    RBF_TRY(rbf_mlp_tc_status(ctx, &before));  // clear what earlier launches left
    constexpr int M = 256, N = 32, K = 64;
    DevBuf a, b, c;
    RBF_TRY(a.alloc(ctx, sizeof(__nv_bfloat16) * M * K));
    RBF_TRY(b.alloc(ctx, sizeof(__nv_bfloat16) * N * K));
    RBF_TRY(c.alloc(ctx, sizeof(float) * M * N));
    RBF_CUDA(ctx, cudaMemsetAsync(a.ptr, 0, sizeof(__nv_bfloat16) * M * K, ctx->stream));
    RBF_CUDA(ctx, cudaMemsetAsync(b.ptr, 0, sizeof(__nv_bfloat16) * N * K, ctx->stream));
    RBF_TRY(launch_tc_persistent<32>(ctx, M, N, K, a.ptr, K, b.ptr, K, nullptr, 0, c.as<float>(), nullptr, N, 4096u, 0));
    RBF_TRY(rbf_mlp_tc_status(ctx, failed));
    if (before) {  // keep an earlier failure visible to the next status call
        unsigned int one = 1;
        RBF_CUDA(ctx, cudaMemcpyToSymbol(g_tc_error, &one, sizeof one));
    }
    return RBF_OK;
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
