// Internal declarations shared by the translation units of librbffd_gb300.so.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <map>
#include <string>

#include "rbffd.h"

// Round-to-nearest-even double -> float on the integer pipe (on GB300 the conversion
// instruction runs on the FP64 pipe); values outside the FP32 normal range take it anyway.
__device__ __forceinline__ float d2f_rn_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    if (e <= 0 || e >= 255) return (float)x;
    const unsigned long long m = b & 0xfffffffffffffull;
    const unsigned long long rem = m & 0x1fffffffull, half = 1ull << 28;
    unsigned r = ((unsigned)e << 23) | (unsigned)(m >> 29);
    if (rem > half || (rem == half && (r & 1u))) r += 1u;  // a carry into the exponent is the right result
    return __uint_as_float(((unsigned)(b >> 32) & 0x80000000u) | r);
}

// Size-class keys of the batched build: (m * 65 + k) * 8 + (polynomial degree + 1), k <= 64
// the stencil length, m <= 64 the normal-derivative unknowns (RBF_FLAG_NORMAL_DOF).
constexpr int kRbfBatchKeys = 65 * 65 * 8;

// One tuned size class of the batched build: the tile shape chosen and the trial timings.
// tile 2 of a batched class: the split-row register kernel on the class's stencils (its own launch)
constexpr int kTileSplit = 2;

struct rbf_tune_entry {
    int tile = 0;  // 0: one warp per stencil, 1: the whole block on one stencil, 2: split-row kernel
    float ms_warp = 0.f, ms_block = 0.f, ms_split = 0.f;
    long long sample = 0;
};

struct rbf_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string last_error;
    long long launches = 0;      // kernels launched through this context
    long long knn_fallback = 0;  // queries re-run by the exact FP64 neighbour search
    std::map<unsigned long long, rbf_tune_entry> tune;  // batched build: size class -> tile
    bool timing = false;  // record CUDA events around the device work of knn / spmm
    float last_ms = 0.f;  // duration of the last timed device work
};

int rbf_fail(rbf_ctx *ctx, int code, const char *fmt, ...);

#define RBF_CUDA(ctx, expr)                                                                  \
    do {                                                                                     \
        cudaError_t e_ = (expr);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return rbf_fail((ctx), RBF_ERR_CUDA, "%s failed: %s", #expr, cudaGetErrorString(e_)); \
    } while (0)

#define RBF_CHECK_LAUNCH(ctx)                                                                \
    do {                                                                                     \
        (ctx)->launches++;                                                                   \
        RBF_CUDA(ctx, cudaGetLastError());                                                   \
    } while (0)

#define RBF_TRY(expr)             \
    do {                          \
        int s_ = (expr);          \
        if (s_ != RBF_OK) return s_; \
    } while (0)

// Stream-ordered device buffer owned by a host scope.
struct DevBuf {
    void *ptr = nullptr;
    cudaStream_t stream = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() {
        if (ptr) cudaFreeAsync(ptr, stream);
    }
    int alloc(rbf_ctx *ctx, size_t bytes) {
        stream = ctx->stream;
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMallocAsync(&ptr, bytes, stream);
        if (e != cudaSuccess) {
            ptr = nullptr;
            return rbf_fail(ctx, RBF_ERR_CUDA, "device allocation of %zu bytes failed: %s", bytes,
                            cudaGetErrorString(e));
        }
        return RBF_OK;
    }
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

// An input array that may live on the host or the device; host data is staged to the
// device on the context stream.
struct InArray {
    const void *dptr = nullptr;
    DevBuf staged;
    int bind(rbf_ctx *ctx, const void *p, size_t bytes);
    template <class T> const T *as() const { return static_cast<const T *>(dptr); }
};

// An output array that may live on the host or the device; host outputs are written
// through a device staging buffer and copied back by finish().
struct OutArray {
    void *user = nullptr;
    void *dptr = nullptr;
    size_t bytes = 0;
    bool host = false;
    DevBuf staged;
    int bind(rbf_ctx *ctx, void *p, size_t bytes_);
    int finish(rbf_ctx *ctx);
    template <class T> T *as() const { return static_cast<T *>(dptr); }
};

bool rbf_is_device_ptr(const void *p);

// ---- kernels (launch wrappers), one per translation unit --------------------------
struct KnnGrid;  // opaque grid description (knn.cu)

int rbf_knn_device(rbf_ctx *ctx, const double *d_data, int64_t ns, const double *d_eval, int64_t ne,
                   int dim, int k, int32_t *d_idx);

struct StencilParams;  // stencil.cuh

int rbf_count_rows_device(rbf_ctx *ctx, int64_t ne, int k, const uint8_t *d_isb,
                          const int32_t *d_g2b, const double *d_alpha, const double *d_beta,
                          int64_t *d_row_ptr, int64_t *nnz, const int64_t *d_adj_ptr = nullptr,
                          const int32_t *d_adj_idx = nullptr);

int rbf_boundary_map_device(rbf_ctx *ctx, int64_t n, const uint8_t *d_isb, int32_t *d_g2b,
                            int64_t *n_boundary);

int rbf_check_indices(rbf_ctx *ctx, const int32_t *d_idx, int64_t n, int32_t hi, bool *ok);
int rbf_backward_launch(rbf_ctx *ctx, const StencilParams &P, bool refined, const double *dW, double *ddata,
                        double *deval);
int rbf_sytrf_rook_device(rbf_ctx *ctx, int nt, double *dA, int64_t lda, int32_t *dipiv, int32_t *dperm,
                          int64_t *info);
int rbf_check_ipiv_device(rbf_ctx *ctx, int nt, const int32_t *dipiv, bool *ok);
int rbf_sytrs_rook_device(rbf_ctx *ctx, int nt, const double *dA, int64_t lda, const int32_t *dipiv,
                          const int32_t *dperm, const double *db, double *dx);
int rbf_interp_assemble_device(rbf_ctx *ctx, int dim, int phs, int nmon, const int8_t (*exps)[3], const double *dx,
                               int n, double *dA, int64_t lda);
int rbf_interp_eval_device(rbf_ctx *ctx, int dim, int phs, int nmon, const int8_t (*exps)[3], const double *dx, int n,
                           const double *dcoef, const double *dxe, int64_t m, double *dout);
int rbf_exclusive_scan_i64(rbf_ctx *ctx, const int64_t *d_in, int64_t *d_out, int64_t n,
                           int64_t *total);
// operator algebra on built weights (algebra.cu)
int rbf_weights_axpby_device(rbf_ctx *ctx, int64_t nnz, double alpha, const double *a, double beta, const double *b,
                             double *out);
int rbf_weights_directional_device(rbf_ctx *ctx, int64_t ne, const int64_t *rp, int nd, const double *val,
                                   int64_t nnz, const double *v, int per_row, double *out);
// sliced-ELL copy of an operator (sell.cu)
int rbf_sell_offsets_device(rbf_ctx *ctx, int64_t ne, const int64_t *d_rp, int64_t *d_off, int64_t *sell_nnz);
int rbf_sell_fill_device(rbf_ctx *ctx, int64_t ne, const int64_t *d_rp, const int32_t *d_col, const double *d_val,
                         const int64_t *d_off, int32_t *d_scol, double *d_sval);
int rbf_spmv_sell_device(rbf_ctx *ctx, int64_t ne, const int64_t *d_off, const int32_t *d_scol, const double *d_sval,
                         const double *d_x, double alpha, double beta, double *d_y);
int rbf_sell_offsets_perm_device(rbf_ctx *ctx, int64_t ne, const int64_t *d_rp, const int32_t *d_row_at,
                                 int64_t *d_off, int64_t *sell_nnz);
int rbf_sell_fill_perm_device(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *d_rp, const int32_t *d_col,
                              const double *d_val, const int32_t *d_row_at, const int32_t *d_col_at,
                              const int64_t *d_off, int32_t *d_scol, double *d_sval);
int rbf_spmv_sell_perm_device(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *d_off, const int32_t *d_scol,
                              const double *d_sval, const int32_t *d_row_at, const int32_t *d_col_at,
                              const double *d_x, double *d_xwork, double alpha, double beta, double *d_y);
int rbf_exclusive_scan_i32(rbf_ctx *ctx, const int32_t *d_in, int32_t *d_out, int64_t n,
                           int64_t *total);

int rbf_spmm_device(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *d_row_ptr,
                    const int32_t *d_col, const double *d_val, int nf, int layout,
                    const double *d_X, int64_t ldx, double alpha, double beta, double *d_Y,
                    int64_t ldy);

int rbf_csr_to_csc_device(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *d_row_ptr,
                          const int32_t *d_col, const double *d_val, int64_t *d_col_ptr,
                          int32_t *d_row, double *d_valc);
