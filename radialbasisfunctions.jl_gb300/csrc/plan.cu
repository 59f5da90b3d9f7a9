// Build -> apply captured in one CUDA graph (rbf_plan_*).
//
// A time loop over moving points re-builds the weights on fixed stencils and applies the
// operator every step (update_weights! then the operator call, src/operators/
// operators.jl:589-602 and 217-218).  Through the plain entry points every step pays the
// host-side argument checks, the staging decisions, a stream synchronisation and the
// launch latency of each kernel.  A plan records the counter reset, the build kernel and
// the SpMV once, on device buffers fixed at creation, and replays them as one graph
// launch; new coordinates or a new field are written into the same buffers in between.
#include <cstring>

#include "rbf_internal.cuh"
#include "stencil_common.cuh"

int rbf_build_fp64_launch(rbf_ctx *ctx, const StencilParams &P);
int rbf_build_fp32_launch(rbf_ctx *ctx, const StencilParams &P);
int rbf_plan_params(rbf_ctx *ctx, const rbf_build_cfg *cfg, StencilParams &P);

struct rbf_plan {
    rbf_ctx *ctx = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *counters = nullptr;  // the build's counters (device), reset inside the graph
    void *defer = nullptr;     // room for the stencils the FP32 path hands to its second kernel
    cudaStream_t capture = nullptr;
};

namespace {

int plan_capture(rbf_plan *pl, const StencilParams &P, int precision, const int64_t *row_ptr, const int32_t *col,
                 const double *val_op, int64_t ne, int64_t ns, const double *x, double *y) {
    rbf_ctx *ctx = pl->ctx;
    auto enqueue = [&]() -> int {
        RBF_CUDA(ctx, cudaMemsetAsync(pl->counters, 0, sizeof(unsigned long long) * 8 + sizeof(double), ctx->stream));
        RBF_TRY(precision == RBF_PREC_FP64 ? rbf_build_fp64_launch(ctx, P) : rbf_build_fp32_launch(ctx, P));
        RBF_TRY(rbf_spmm_device(ctx, ne, ns, row_ptr, col, val_op, 1, 1, x, 1, 1.0, 0.0, y, 1));
        return RBF_OK;
    };
    cudaStream_t user = ctx->stream;
    ctx->stream = pl->capture;
    // one plain run first: loads the kernels and sets their attributes outside the capture
    int st = enqueue();
    if (st == RBF_OK) {
        cudaError_t e = cudaStreamSynchronize(pl->capture);
        if (e != cudaSuccess) st = rbf_fail(ctx, RBF_ERR_CUDA, "plan warm-up failed: %s", cudaGetErrorString(e));
    }
    if (st == RBF_OK) {
        cudaError_t e = cudaStreamBeginCapture(pl->capture, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            st = rbf_fail(ctx, RBF_ERR_CUDA, "cudaStreamBeginCapture failed: %s", cudaGetErrorString(e));
        } else {
            st = enqueue();
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(pl->capture, &g);
            if (st == RBF_OK && e != cudaSuccess)
                st = rbf_fail(ctx, RBF_ERR_CUDA, "cudaStreamEndCapture failed: %s", cudaGetErrorString(e));
            if (st == RBF_OK) {
                pl->graph = g;
                e = cudaGraphInstantiate(&pl->exec, g, 0);
                if (e != cudaSuccess) st = rbf_fail(ctx, RBF_ERR_CUDA, "cudaGraphInstantiate failed: %s", cudaGetErrorString(e));
            } else if (g) {
                cudaGraphDestroy(g);
            }
        }
    }
    ctx->stream = user;
    return st;
}

}  // namespace

extern "C" {

int rbf_plan_create(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns, const double *eval,
                    int64_t ne, const int32_t *adjl, int32_t k, const int64_t *row_ptr, int32_t *col, double *val,
                    int32_t op_index, const double *x, double *y, rbf_plan **out) {
    if (!ctx || !out) return RBF_ERR_ARGUMENT;
    *out = nullptr;
    if (!cfg) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null configuration");
    if (cfg->precision != RBF_PREC_FP64 && cfg->precision != RBF_PREC_FP32_REFINED)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "a plan builds in plain FP64 or FP32-refined precision");
    const void *ptrs[] = {data, eval, adjl, row_ptr, col, val, x, y};
    for (const void *p : ptrs)
        if (!p || !rbf_is_device_ptr(p)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "a plan takes device pointers only");
    if (k < 1 || k > RBF_MAX_STENCIL) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "k must be in 1..%d", RBF_MAX_STENCIL);
    if (ns < k || ns >= INT32_MAX || ne < 1 || ne >= INT32_MAX) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid sizes");
    StencilParams P;
    memset(&P, 0, sizeof P);
    P.k = k;
    RBF_TRY(rbf_plan_params(ctx, cfg, P));
    if (op_index < 0 || op_index >= cfg->nops) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "op_index out of range");
    bool idx_ok = true;
    RBF_TRY(rbf_check_indices(ctx, adjl, ne * (int64_t)k, (int32_t)ns, &idx_ok));
    if (!idx_ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "adjl holds indices outside [0, %lld)", (long long)ns);
    int64_t nnz = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&nnz, row_ptr + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nnz != ne * (int64_t)k) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "row_ptr is not the layout of k entries per row");
    rbf_plan *pl = new rbf_plan();
    pl->ctx = ctx;
    cudaError_t e = cudaStreamCreateWithFlags(&pl->capture, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&pl->counters, sizeof(unsigned long long) * 8 + sizeof(double));
    if (e == cudaSuccess && cfg->precision != RBF_PREC_FP64) e = cudaMalloc(&pl->defer, sizeof(int32_t) * (size_t)ne);
    if (e != cudaSuccess) {
        if (pl->counters) cudaFree(pl->counters);
        if (pl->capture) cudaStreamDestroy(pl->capture);
        delete pl;
        return rbf_fail(ctx, RBF_ERR_CUDA, "plan allocation failed: %s", cudaGetErrorString(e));
    }
    P.ne = ne;
    P.ns = ns;
    P.nnz = nnz;
    P.data = data;
    P.eval = eval;
    P.adjl = adjl;
    P.row_ptr = row_ptr;
    P.col = col;
    P.val = val;
    P.counters = static_cast<unsigned long long *>(pl->counters);
    P.max_resid = reinterpret_cast<double *>(static_cast<unsigned long long *>(pl->counters) + 8);
    P.defer = static_cast<int32_t *>(pl->defer);
    const int st = plan_capture(pl, P, cfg->precision, row_ptr, col, val + (size_t)op_index * nnz, ne, ns, x, y);
    if (st != RBF_OK) {
        rbf_plan_destroy(pl);
        return st;
    }
    *out = pl;
    return RBF_OK;
}

int rbf_plan_launch(rbf_plan *pl) {
    if (!pl || !pl->exec) return RBF_ERR_ARGUMENT;
    rbf_ctx *ctx = pl->ctx;
    RBF_CUDA(ctx, cudaGraphLaunch(pl->exec, ctx->stream));
    return RBF_OK;
}

int rbf_plan_counters(rbf_plan *pl, int64_t *singular, int64_t *fallback, int64_t *residuals) {
    if (!pl) return RBF_ERR_ARGUMENT;
    rbf_ctx *ctx = pl->ctx;
    unsigned long long hc[8];
    RBF_CUDA(ctx, cudaMemcpyAsync(hc, pl->counters, sizeof hc, cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (singular) *singular = (int64_t)hc[0];
    if (fallback) *fallback = (int64_t)hc[2];
    if (residuals) *residuals = (int64_t)hc[4];
    return RBF_OK;
}

int rbf_plan_destroy(rbf_plan *pl) {
    if (!pl) return RBF_OK;
    if (pl->capture) cudaStreamSynchronize(pl->capture);
    if (pl->ctx) cudaStreamSynchronize(pl->ctx->stream);
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    if (pl->counters) cudaFree(pl->counters);
    if (pl->defer) cudaFree(pl->defer);
    if (pl->capture) cudaStreamDestroy(pl->capture);
    delete pl;
    return RBF_OK;
}

}  // extern "C"
