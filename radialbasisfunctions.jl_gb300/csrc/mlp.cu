// Kernels of the learned stencil surrogate: a small MLP (e.g. 96 -> 256 -> 256 -> 256 -> 32,
// GELU) whose training (forward, backward, Adam) and inference run on these kernels.
//
// GEMM: C[M x N] = A[M x K] * B[N x K]^T with A and B bf16, K contiguous in both (the
// [out x in] layout of a weight matrix), FP32 accumulation on the tensor cores through
// mma.sync m16n8k16.  One 64x64 tile per block of 4 warps (each warp 32x32 = 2 x 4
// fragments), K staged through shared memory 32 at a time.  Epilogues: + bias, GELU (tanh form, mlp_common.cuh),
// or multiplication by GELU'(aux) for the backward pass; outputs FP32 and/or bf16.
// K must be a multiple of 32 and leading dimensions multiples of 8 (inputs are padded).  A
// GEMM with few output tiles and a long K (the weight gradients, K = batch) splits K over the
// blocks and sums the slices' tiles in a second, deterministic pass.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "mlp_common.cuh"
#include "rbf_internal.cuh"

namespace {

constexpr int BM = 64, BN = 64, BK = 32, SPAD = 8;  // smem rows of 40 bf16 = 80 B

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

enum { EPI_NONE = 0, EPI_GELU = 1, EPI_GELU_GRAD = 2 };

__global__ void __launch_bounds__(128) gemm_bf16_kernel(int M, int N, int K, const __nv_bfloat16 *__restrict__ A,
                                                        int lda, const __nv_bfloat16 *__restrict__ B, int ldb,
                                                        const float *__restrict__ bias, int epi,
                                                        const float *__restrict__ aux, int ldaux,
                                                        float *__restrict__ Cf, int ldcf, __nv_bfloat16 *__restrict__ Cb,
                                                        int ldcb, float *__restrict__ Zf, int ldz, int kchunk,
                                                        float *__restrict__ part) {
    // split K (gridDim.z > 1): this block sums K slice blockIdx.z (kchunk elements) and writes
    // its raw tile to part[blockIdx.z][M][N]; splitk_reduce_kernel applies the epilogue
    __shared__ __align__(16) __nv_bfloat16 As[BM][BK + SPAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + SPAD];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1;
    const int g = lane >> 2, tig = lane & 3;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int t = 0; t < 4; t++) acc[i][j][t] = 0.0f;

    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    for (int k0 = kb; k0 < ke; k0 += BK) {
        // 64 rows x 32 bf16 = 256 chunks of 16 B per operand; 2 per thread
#pragma unroll
        for (int it = 0; it < 2; it++) {
            const int c = tid + it * 128;
            const int r = c >> 2, cc = (c & 3) * 8;
            uint4 va = make_uint4(0, 0, 0, 0), vb = make_uint4(0, 0, 0, 0);
            if (m0 + r < M) va = *reinterpret_cast<const uint4 *>(A + (size_t)(m0 + r) * lda + k0 + cc);
            if (n0 + r < N) vb = *reinterpret_cast<const uint4 *>(B + (size_t)(n0 + r) * ldb + k0 + cc);
            *reinterpret_cast<uint4 *>(&As[r][cc]) = va;
            *reinterpret_cast<uint4 *>(&Bs[r][cc]) = vb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int mi = 0; mi < 2; mi++) {
                const int r = wm * 32 + mi * 16 + g;
                af[mi][0] = *reinterpret_cast<const uint32_t *>(&As[r][kk + 2 * tig]);
                af[mi][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + 2 * tig]);
                af[mi][2] = *reinterpret_cast<const uint32_t *>(&As[r][kk + 8 + 2 * tig]);
                af[mi][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + 8 + 2 * tig]);
            }
#pragma unroll
            for (int ni = 0; ni < 4; ni++) {
                const int r = wn * 32 + ni * 8 + g;
                bf[ni][0] = *reinterpret_cast<const uint32_t *>(&Bs[r][kk + 2 * tig]);
                bf[ni][1] = *reinterpret_cast<const uint32_t *>(&Bs[r][kk + 8 + 2 * tig]);
            }
#pragma unroll
            for (int mi = 0; mi < 2; mi++)
#pragma unroll
                for (int ni = 0; ni < 4; ni++) mma_bf16(acc[mi][ni], af[mi], bf[ni]);
        }
        __syncthreads();
    }
    // epilogue: fragment (mi, ni) element t sits at row g (+8 for t >= 2), col 2*tig + (t & 1)
#pragma unroll
    for (int mi = 0; mi < 2; mi++)
#pragma unroll
        for (int ni = 0; ni < 4; ni++)
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const int row = m0 + wm * 32 + mi * 16 + g + (t >= 2 ? 8 : 0);
                const int col = n0 + wn * 32 + ni * 8 + 2 * tig + (t & 1);
                if (row >= M || col >= N) continue;
                float z = acc[mi][ni][t];
                if (part) {
                    part[((size_t)blockIdx.z * M + row) * N + col] = z;
                    continue;
                }
                if (bias) z += bias[col];
                if (Zf) Zf[(size_t)row * ldz + col] = z;
                float o = z;
                if (epi == EPI_GELU) o = gelu(z);
                else if (epi == EPI_GELU_GRAD) o = z * gelu_grad(aux[(size_t)row * ldaux + col]);
                if (Cf) Cf[(size_t)row * ldcf + col] = o;
                if (Cb) Cb[(size_t)row * ldcb + col] = __float2bfloat16_rn(o);
            }
}

// Sum of the split-K partial tiles in slice order (deterministic), then the epilogue of
// gemm_bf16_kernel.
__global__ void splitk_reduce_kernel(int M, int N, int nsplit, const float *__restrict__ part,
                                     const float *__restrict__ bias, int epi, const float *__restrict__ aux, int ldaux,
                                     float *__restrict__ Cf, int ldcf, __nv_bfloat16 *__restrict__ Cb, int ldcb,
                                     float *__restrict__ Zf, int ldz) {
    const int64_t total = (int64_t)M * N;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int row = (int)(t / N), col = (int)(t % N);
        float z = 0.0f;
        for (int sp = 0; sp < nsplit; sp++) z += part[(size_t)sp * total + t];
        if (bias) z += bias[col];
        if (Zf) Zf[(size_t)row * ldz + col] = z;
        float o = z;
        if (epi == EPI_GELU) o = gelu(z);
        else if (epi == EPI_GELU_GRAD) o = z * gelu_grad(aux[(size_t)row * ldaux + col]);
        if (Cf) Cf[(size_t)row * ldcf + col] = o;
        if (Cb) Cb[(size_t)row * ldcb + col] = __float2bfloat16_rn(o);
    }
}

__global__ void transpose_bf16_kernel(int rows, int cols, const __nv_bfloat16 *__restrict__ in, int ldi,
                                      __nv_bfloat16 *__restrict__ out, int ldo) {
    __shared__ __nv_bfloat16 tile[32][34];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, c = c0 + threadIdx.x;
        tile[y][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * ldi + c] : __float2bfloat16_rn(0.0f);
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int c = c0 + y, r = r0 + threadIdx.x;
        if (c < cols && r < rows) out[(size_t)c * ldo + r] = tile[threadIdx.x][y];
    }
}

// float (rows x cols, ldi) -> bf16 (ldo), zero padding beyond cols up to pad_cols
__global__ void f32_to_bf16_kernel(int rows, int cols, int pad_cols, const float *__restrict__ in, int ldi,
                                   __nv_bfloat16 *__restrict__ out, int ldo) {
    const int64_t total = (int64_t)rows * pad_cols;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / pad_cols), c = (int)(t % pad_cols);
        out[(size_t)r * ldo + c] = __float2bfloat16_rn(c < cols ? in[(size_t)r * ldi + c] : 0.0f);
    }
}

// loss = sum (Y - T)^2 / (rows * cols); dY = 2 (Y - T) / (rows * cols), in bf16 (ld ldd)
__global__ void mse_kernel(int rows, int cols, const float *__restrict__ Y, int ldy, const float *__restrict__ T,
                           int ldt, __nv_bfloat16 *__restrict__ dY, int ldd, int pad_cols, float *__restrict__ loss) {
    const int64_t total = (int64_t)rows * pad_cols;
    const float sc = 1.0f / ((float)rows * (float)cols);
    float local = 0.0f;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / pad_cols), c = (int)(t % pad_cols);
        float gv = 0.0f;
        if (c < cols) {
            const float d = Y[(size_t)r * ldy + c] - T[(size_t)r * ldt + c];
            local += d * d;
            gv = 2.0f * d * sc;
        }
        dY[(size_t)r * ldd + c] = __float2bfloat16_rn(gv);
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, local * sc);
}

// column sums of a bf16 matrix (bias gradients): one thread per column
__global__ void colsum_bf16_kernel(int rows, int cols, const __nv_bfloat16 *__restrict__ in, int ldi,
                                   float *__restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.0f;
    for (int r = 0; r < rows; r++) s += __bfloat162float(in[(size_t)r * ldi + c]);
    out[c] = s;
}

// Adam on FP32 master parameters, refreshing their bf16 copy
__global__ void adam_kernel(int64_t n, float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                            float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                            __nv_bfloat16 *__restrict__ pb) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float g = gr[i];
        const float mi = b1 * m[i] + (1.0f - b1) * g;
        const float vi = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        p[i] = pi;
        if (pb) pb[i] = __float2bfloat16_rn(pi);
    }
}

int grid1d(rbf_ctx *ctx, int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)ctx->num_sms * 8));
}

}  // namespace

extern "C" {

int rbf_mlp_gemm(rbf_ctx *ctx, int32_t M, int32_t N, int32_t K, const void *A, int32_t lda, const void *B, int32_t ldb,
                 const float *bias, int32_t epi, const float *aux, int32_t ldaux, float *Cf, int32_t ldcf, void *Cb,
                 int32_t ldcb, float *Zf, int32_t ldz) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    if (M < 0 || N < 0 || K <= 0 || K % BK != 0) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "gemm: K must be a positive multiple of 32");
    if (lda % 8 || ldb % 8 || ((uintptr_t)A & 15) || ((uintptr_t)B & 15) || lda < K || ldb < K)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "gemm: operands need 16-byte aligned rows (ld multiple of 8, >= K)");
    if (epi == EPI_GELU_GRAD && !aux) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "gemm: GELU-gradient epilogue needs aux");
    if (M == 0 || N == 0) return RBF_OK;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
    // few output tiles over a long K (the weight gradients: K = batch): split K so that the
    // GEMM fills the GPU (about two blocks per SM), slices of at least 128
    const int tiles = (int)(grid.x * grid.y);
    int nsplit = 1, kchunk = K;
    if (2 * tiles < ctx->num_sms && K >= 256) {
        nsplit = std::min(K / 128, (2 * ctx->num_sms + tiles - 1) / tiles);
        kchunk = ((K + nsplit - 1) / nsplit + BK - 1) / BK * BK;
        nsplit = (K + kchunk - 1) / kchunk;
    }
    if (nsplit <= 1) {
        gemm_bf16_kernel<<<grid, 128, 0, ctx->stream>>>(M, N, K, (const __nv_bfloat16 *)A, lda, (const __nv_bfloat16 *)B,
                                                         ldb, bias, epi, aux, ldaux, Cf, ldcf, (__nv_bfloat16 *)Cb, ldcb,
                                                         Zf, ldz, K, nullptr);
        RBF_CHECK_LAUNCH(ctx);
        return RBF_OK;
    }
    DevBuf part;
    RBF_TRY(part.alloc(ctx, sizeof(float) * (size_t)nsplit * M * N));
    grid.z = nsplit;
    gemm_bf16_kernel<<<grid, 128, 0, ctx->stream>>>(M, N, K, (const __nv_bfloat16 *)A, lda, (const __nv_bfloat16 *)B, ldb,
                                                     nullptr, 0, nullptr, 0, nullptr, 0, nullptr, 0, nullptr, 0, kchunk,
                                                     part.as<float>());
    RBF_CHECK_LAUNCH(ctx);
    splitk_reduce_kernel<<<grid1d(ctx, (int64_t)M * N), 256, 0, ctx->stream>>>(
        M, N, nsplit, part.as<float>(), bias, epi, aux, ldaux, Cf, ldcf, (__nv_bfloat16 *)Cb, ldcb, Zf, ldz);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_mlp_transpose(rbf_ctx *ctx, int32_t rows, int32_t cols, const void *in, int32_t ldi, void *out, int32_t ldo) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    if (rows <= 0 || cols <= 0) return RBF_OK;
    transpose_bf16_kernel<<<dim3((cols + 31) / 32, (rows + 31) / 32), dim3(32, 8), 0, ctx->stream>>>(
        rows, cols, (const __nv_bfloat16 *)in, ldi, (__nv_bfloat16 *)out, ldo);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_mlp_to_bf16(rbf_ctx *ctx, int32_t rows, int32_t cols, int32_t pad_cols, const float *in, int32_t ldi, void *out,
                    int32_t ldo) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    if (pad_cols < cols || ldo < pad_cols) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "to_bf16: pad_cols < cols or ldo < pad_cols");
    f32_to_bf16_kernel<<<grid1d(ctx, (int64_t)rows * pad_cols), 256, 0, ctx->stream>>>(rows, cols, pad_cols, in, ldi,
                                                                                      (__nv_bfloat16 *)out, ldo);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_mlp_mse(rbf_ctx *ctx, int32_t rows, int32_t cols, const float *Y, int32_t ldy, const float *T, int32_t ldt,
                void *dY, int32_t ldd, int32_t pad_cols, float *loss) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    RBF_CUDA(ctx, cudaMemsetAsync(loss, 0, sizeof(float), ctx->stream));
    mse_kernel<<<grid1d(ctx, (int64_t)rows * pad_cols), 256, 0, ctx->stream>>>(rows, cols, Y, ldy, T, ldt,
                                                                              (__nv_bfloat16 *)dY, ldd, pad_cols, loss);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_mlp_colsum(rbf_ctx *ctx, int32_t rows, int32_t cols, const void *in, int32_t ldi, float *out) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    colsum_bf16_kernel<<<(cols + 127) / 128, 128, 0, ctx->stream>>>(rows, cols, (const __nv_bfloat16 *)in, ldi, out);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_mlp_adam(rbf_ctx *ctx, int64_t n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2,
                 float eps, int32_t step, void *p_bf16) {
    if (!ctx || step < 1) return RBF_ERR_ARGUMENT;
    const float c1 = 1.0f / (1.0f - powf(b1, (float)step)), c2 = 1.0f / (1.0f - powf(b2, (float)step));
    adam_kernel<<<grid1d(ctx, n), 256, 0, ctx->stream>>>(n, p, g, m, v, lr, b1, b2, eps, c1, c2, (__nv_bfloat16 *)p_bf16);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

}  // extern "C"

namespace {
// double -> float on the integer pipe (mantissa truncated; bf16 inputs need far less)
__device__ __forceinline__ float trunc_to_float(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7ffu) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}

// Network inputs of one stencil: the offsets x_i - x0 of its k points (stencil order, i.e.
// sorted by distance) in the local units of the solver (divided by the power of two s >=
// the stencil radius), as bf16, padded with zeros to ldo.  One warp per stencil.  Only the
// subtraction runs in FP64 (cancellation); the rest is FP32, which is far more accurate than
// the bf16 result (the FP64 pipe of this part is ~70x slower than FP32).
__global__ void features_kernel(const double *__restrict__ data, const double *__restrict__ eval, int dim,
                                const int32_t *__restrict__ adjl, int64_t ne, int k, __nv_bfloat16 *__restrict__ out,
                                int ldo, int ldo_pad, int vec) {
    // each warp assembles its stencil's row in shared memory and writes it with 16-byte
    // stores (the per-lane offsets are 2-6 bytes wide and would scatter into many pieces)
    extern __shared__ __align__(16) __nv_bfloat16 fbuf[];
    __nv_bfloat16 *buf = fbuf + (size_t)(threadIdx.x >> 5) * ldo_pad;
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; e < ne; e += nw) {
        float dv[2][3];
        float r2max = 0.0f;
#pragma unroll
        for (int s = 0; s < 2; s++) {
            const int i = lane + 32 * s;
#pragma unroll
            for (int d = 0; d < 3; d++) dv[s][d] = 0.0f;
            if (i < k) {
                const int32_t g = __ldg(&adjl[e * k + i]);
                float r2 = 0.0f;
                for (int d = 0; d < dim; d++) {
                    dv[s][d] = trunc_to_float(__ldg(&data[(int64_t)g * dim + d]) - __ldg(&eval[e * dim + d]));
                    r2 = fmaf(dv[s][d], dv[s][d], r2);
                }
                r2max = fmaxf(r2max, r2);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r2max = fmaxf(r2max, __shfl_xor_sync(0xffffffffu, r2max, o));
        int es = 0;
        if (r2max > 0.0f) frexpf(sqrtf(r2max), &es);
        // 2^-es as an exact float (es within the normal range; otherwise ldexpf)
        const bool pow_ok = es > -126 && es < 127;
        const float sc = pow_ok ? __int_as_float((127 - es) << 23) : 1.0f;
#pragma unroll
        for (int s = 0; s < 2; s++) {
            const int i = lane + 32 * s;
            if (i < k)
                for (int d = 0; d < dim; d++)
                    buf[i * dim + d] = __float2bfloat16_rn(pow_ok ? dv[s][d] * sc : ldexpf(dv[s][d], -es));
        }
        for (int c = k * dim + lane; c < ldo; c += 32) buf[c] = __float2bfloat16_rn(0.0f);
        __syncwarp();
        __nv_bfloat16 *row = out + (size_t)e * ldo;
        if (vec) {
            for (int u = lane; u < ldo / 8; u += 32)
                reinterpret_cast<uint4 *>(row)[u] = reinterpret_cast<const uint4 *>(buf)[u];
        } else {
            for (int c = lane; c < ldo; c += 32) row[c] = buf[c];
        }
        __syncwarp();
    }
}
}  // namespace

extern "C" int rbf_mlp_features(rbf_ctx *ctx, const double *data, int64_t n_data, const double *eval, int32_t dim,
                                const int32_t *adjl, int64_t ne, int32_t k, void *out, int32_t ldo) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    if (dim < 1 || dim > 3 || k < 1 || k > 64 || ldo < k * dim || ldo > 4096 || ne < 0 || n_data < 1 ||
        n_data > INT32_MAX)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT,
                        "features: need 1 <= dim <= 3, 1 <= k <= 64, k*dim <= ldo <= 4096, n_data >= 1");
    if (ne == 0) return RBF_OK;
    bool idx_ok = false;
    RBF_TRY(rbf_check_indices(ctx, adjl, ne * (int64_t)k, (int32_t)n_data, &idx_ok));
    if (!idx_ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "features: a neighbour index is outside [0, n_data)");
    const int64_t blocks = std::min<int64_t>((ne + 7) / 8, (int64_t)ctx->num_sms * 32);
    const int ldo_pad = (ldo + 7) & ~7;
    const int vec = (ldo % 8 == 0 && ((uintptr_t)out & 15) == 0) ? 1 : 0;
    const size_t smem = sizeof(__nv_bfloat16) * 8 * (size_t)ldo_pad;
    if (smem > 48 * 1024) RBF_CUDA(ctx, cudaFuncSetAttribute(features_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    features_kernel<<<(unsigned)blocks, 256, smem, ctx->stream>>>(data, eval, dim, adjl, ne, k, (__nv_bfloat16 *)out, ldo,
                                                                  ldo_pad, vec);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}
