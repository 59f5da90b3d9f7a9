// Diagnostics: kernel-launch accounting and pipe-throughput probes used to state the
// roofline of the build kernels (FP64 / FP32 FMA rate of the device, measured, since the
// generated peaks cover only HBM bandwidth and bf16 tensor throughput).
#include "rbf_internal.cuh"

namespace {

template <class T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T *out, int iters, T seed) {
    T a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
      a7 = a0 + 7;
    const T m = (T)0.999999, c = (T)1e-7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
            a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
            a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
        }
    }
    T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == (T)-12345.0) out[threadIdx.x] = s;  // keeps the chain alive
}

template <class T>
int probe(rbf_ctx *ctx, double *tflops) {
    DevBuf o;
    RBF_TRY(o.alloc(ctx, sizeof(T) * 256));
    const int blocks = ctx->num_sms * 8, iters = 2048;
    fma_probe_kernel<T><<<blocks, 256, 0, ctx->stream>>>(o.as<T>(), 16, (T)1);  // warm-up
    RBF_CHECK_LAUNCH(ctx);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    fma_probe_kernel<T><<<blocks, 256, 0, ctx->stream>>>(o.as<T>(), iters, (T)1);
    cudaEventRecord(e1, ctx->stream);
    RBF_CUDA(ctx, cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    double flops = 2.0 * 64.0 * iters * (double)blocks * 256.0;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return RBF_OK;
}

}  // namespace

extern "C" int64_t rbf_ctx_kernel_launches(const rbf_ctx *ctx) { return ctx ? ctx->launches : -1; }

extern "C" int rbf_diag_fma_peak(rbf_ctx *ctx, int32_t fp64, double *tflops) {
    if (!ctx || !tflops) return RBF_ERR_ARGUMENT;
    cudaSetDevice(ctx->device);
    return fp64 ? probe<double>(ctx, tflops) : probe<float>(ctx, tflops);
}
