// Sliced-ELL copy of an operator and its single-field apply.
//
// Why: on GB300 the FP64 pipe retires 2 lanes per cycle per SM, about one DFMA per 13
// bytes of HBM traffic at the copy rate, and a CSR apply of a 30-entry row spends ~41 FP64
// operations on it (30 DFMAs, padding of the paired loads, the cross-lane reduction, the
// scaling): on a locality-ordered cloud the CSR kernel is FP64-bound before it is
// HBM-bound.  In the sliced layout (slices of 32 rows; inside a slice, entry j of the 32
// rows is contiguous) one thread owns one row: 4-byte columns and 8-byte values are read
// fully coalesced, the row is summed in registers (no reduction), so the FP64 work is one
// DFMA per entry plus the scaling.
//   slice s = rows 32s .. 32s+31, width w_s = longest row of the slice;
//   entry j of row r at slice_off[s] + 32 j + (r - 32 s), j < w_s;
//   entries past a row's end: column 0, value 0 (padding only in slices of uneven rows).
// slice_off has ceil(ne/32) + 1 entries; slice_off[last] is the sliced entry count.
#include <algorithm>

#include "rbf_internal.cuh"

namespace {

__global__ void sell_width_kernel(int64_t ne, const int64_t *__restrict__ rp, int64_t *__restrict__ w) {
    const int64_t nsl = (ne + 31) / 32;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nsl; s += (int64_t)gridDim.x * blockDim.x) {
        int64_t m = 0;
        const int64_t r1 = min(ne, 32 * s + 32);
        for (int64_t r = 32 * s; r < r1; r++) m = max(m, rp[r + 1] - rp[r]);
        w[s] = 32 * m;
    }
}

__global__ void sell_fill_kernel(int64_t ne, const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                                 const double *__restrict__ val, const int64_t *__restrict__ off,
                                 int32_t *__restrict__ scol, double *__restrict__ sval) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ne; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = r >> 5, lane = r & 31;
        const int64_t w = (off[s + 1] - off[s]) >> 5;
        const int64_t a = rp[r], len = rp[r + 1] - a;
        int32_t *c = scol + off[s] + lane;
        double *v = sval + off[s] + lane;
        for (int64_t j = 0; j < w; j++) {
            c[32 * j] = j < len ? col[a + j] : 0;
            v[32 * j] = j < len ? val[a + j] : 0.0;
        }
    }
}

// One thread per row; U entries in flight per thread, two accumulators.
template <int U>
__global__ void __launch_bounds__(256) spmv_sell_kernel(int64_t ne, const int64_t *__restrict__ off,
                                                        const int32_t *__restrict__ scol,
                                                        const double *__restrict__ sval,
                                                        const double *__restrict__ x, double alpha, double beta,
                                                        double *__restrict__ y) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ne; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = r >> 5;
        const int64_t o = off[s] + (r & 31);
        const int w = (int)((off[s + 1] - off[s]) >> 5);
        double s0 = 0.0, s1 = 0.0;
        int j = 0;
        for (; j + U <= w; j += U) {
            int32_t c[U];
            double v[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                c[u] = __ldcs(&scol[o + 32 * (int64_t)(j + u)]);
                v[u] = __ldcs(&sval[o + 32 * (int64_t)(j + u)]);
            }
#pragma unroll
            for (int u = 0; u < U; u += 2) {
                s0 = fma(v[u], __ldg(&x[c[u]]), s0);
                if (u + 1 < U) s1 = fma(v[u + 1], __ldg(&x[c[u + 1]]), s1);
            }
        }
        for (; j < w; j++) s0 = fma(__ldcs(&sval[o + 32 * (int64_t)j]), __ldg(&x[__ldcs(&scol[o + 32 * (int64_t)j])]), s0);
        const double sm = s0 + s1;
        y[r] = (beta == 0.0) ? alpha * sm : fma(alpha, sm, beta * y[r]);
    }
}

// ---- the copy in a locality order of rows and columns (a Morton order from
// rbf_reorder_points): slice s holds the rows row_at[32 s .. 32 s + 31]; a row's entries keep
// their CSR order with each column j replaced by its position pos_col[j] in the column order.
__global__ void sell_width_perm_kernel(int64_t ne, const int64_t *__restrict__ rp, const int32_t *__restrict__ row_at,
                                       int64_t *__restrict__ w) {
    const int64_t nsl = (ne + 31) / 32;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nsl; s += (int64_t)gridDim.x * blockDim.x) {
        int64_t m = 0;
        const int64_t r1 = min(ne, 32 * s + 32);
        for (int64_t r = 32 * s; r < r1; r++) {
            const int64_t u = row_at[r];
            m = max(m, rp[u + 1] - rp[u]);
        }
        w[s] = 32 * m;
    }
}

__global__ void invert_perm_kernel(int64_t n, const int32_t *__restrict__ at, int32_t *__restrict__ pos) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        pos[at[i]] = (int32_t)i;
}

__global__ void sell_fill_perm_kernel(int64_t ne, const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                                      const double *__restrict__ val, const int32_t *__restrict__ row_at,
                                      const int32_t *__restrict__ pos_col, const int64_t *__restrict__ off,
                                      int32_t *__restrict__ scol, double *__restrict__ sval) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ne; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = r >> 5, lane = r & 31;
        const int64_t w = (off[s + 1] - off[s]) >> 5;
        const int64_t u = row_at[r];
        const int64_t a = rp[u], len = rp[u + 1] - a;
        int32_t *c = scol + off[s] + lane;
        double *v = sval + off[s] + lane;
        for (int64_t j = 0; j < w; j++) {
            c[32 * j] = j < len ? pos_col[col[a + j]] : 0;
            v[32 * j] = j < len ? val[a + j] : 0.0;
        }
    }
}

// x in the column order: xo[i] = x[col_at[i]] (the field read once, scattered within L2)
__global__ void gather_perm_kernel(int64_t n, const int32_t *__restrict__ col_at, const double *__restrict__ x,
                                   double *__restrict__ xo) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        xo[i] = __ldg(&x[__ldcs(&col_at[i])]);
}

// spmv_sell_kernel on the ordered copy: row r of the copy is the operator's row row_at[r],
// whose result goes straight to y[row_at[r]]
template <int U>
__global__ void __launch_bounds__(256) spmv_sell_perm_kernel(int64_t ne, const int64_t *__restrict__ off,
                                                             const int32_t *__restrict__ scol,
                                                             const double *__restrict__ sval,
                                                             const int32_t *__restrict__ row_at,
                                                             const double *__restrict__ xo, double alpha, double beta,
                                                             double *__restrict__ y) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ne; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = r >> 5;
        const int64_t o = off[s] + (r & 31);
        const int w = (int)((off[s + 1] - off[s]) >> 5);
        const int64_t u = __ldcs(&row_at[r]);
        double s0 = 0.0, s1 = 0.0;
        int j = 0;
        for (; j + U <= w; j += U) {
            int32_t c[U];
            double v[U];
#pragma unroll
            for (int q = 0; q < U; q++) {
                c[q] = __ldcs(&scol[o + 32 * (int64_t)(j + q)]);
                v[q] = __ldcs(&sval[o + 32 * (int64_t)(j + q)]);
            }
#pragma unroll
            for (int q = 0; q < U; q += 2) {
                s0 = fma(v[q], __ldg(&xo[c[q]]), s0);
                if (q + 1 < U) s1 = fma(v[q + 1], __ldg(&xo[c[q + 1]]), s1);
            }
        }
        for (; j < w; j++) s0 = fma(__ldcs(&sval[o + 32 * (int64_t)j]), __ldg(&xo[__ldcs(&scol[o + 32 * (int64_t)j])]), s0);
        const double sm = s0 + s1;
        y[u] = (beta == 0.0) ? alpha * sm : fma(alpha, sm, beta * y[u]);
    }
}

int sell_blocks(rbf_ctx *ctx, int64_t work, int threads, int per_sm) {
    int64_t b = (work + threads - 1) / threads;
    b = std::min<int64_t>(b, (int64_t)ctx->num_sms * per_sm);
    return (int)std::max<int64_t>(b, 1);
}

}  // namespace

int rbf_sell_offsets_device(rbf_ctx *ctx, int64_t ne, const int64_t *d_rp, int64_t *d_off, int64_t *sell_nnz) {
    const int64_t nsl = (ne + 31) / 32;
    DevBuf w;
    RBF_TRY(w.alloc(ctx, sizeof(int64_t) * (nsl + 1)));
    RBF_CUDA(ctx, cudaMemsetAsync(w.ptr, 0, sizeof(int64_t) * (nsl + 1), ctx->stream));
    if (nsl > 0) {
        sell_width_kernel<<<sell_blocks(ctx, nsl, 256, 8), 256, 0, ctx->stream>>>(ne, d_rp, w.as<int64_t>());
        RBF_CHECK_LAUNCH(ctx);
    }
    return rbf_exclusive_scan_i64(ctx, w.as<int64_t>(), d_off, nsl + 1, sell_nnz);
}

int rbf_sell_fill_device(rbf_ctx *ctx, int64_t ne, const int64_t *d_rp, const int32_t *d_col, const double *d_val,
                         const int64_t *d_off, int32_t *d_scol, double *d_sval) {
    if (ne == 0) return RBF_OK;
    sell_fill_kernel<<<sell_blocks(ctx, ne, 256, 8), 256, 0, ctx->stream>>>(ne, d_rp, d_col, d_val, d_off, d_scol,
                                                                           d_sval);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_spmv_sell_device(rbf_ctx *ctx, int64_t ne, const int64_t *d_off, const int32_t *d_scol, const double *d_sval,
                         const double *d_x, double alpha, double beta, double *d_y) {
    if (ne == 0) return RBF_OK;
    spmv_sell_kernel<6><<<sell_blocks(ctx, ne, 256, 8), 256, 0, ctx->stream>>>(ne, d_off, d_scol, d_sval, d_x, alpha,
                                                                               beta, d_y);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_sell_offsets_perm_device(rbf_ctx *ctx, int64_t ne, const int64_t *d_rp, const int32_t *d_row_at,
                                 int64_t *d_off, int64_t *sell_nnz) {
    const int64_t nsl = (ne + 31) / 32;
    DevBuf w;
    RBF_TRY(w.alloc(ctx, sizeof(int64_t) * (nsl + 1)));
    RBF_CUDA(ctx, cudaMemsetAsync(w.ptr, 0, sizeof(int64_t) * (nsl + 1), ctx->stream));
    if (nsl > 0) {
        sell_width_perm_kernel<<<sell_blocks(ctx, nsl, 256, 8), 256, 0, ctx->stream>>>(ne, d_rp, d_row_at,
                                                                                       w.as<int64_t>());
        RBF_CHECK_LAUNCH(ctx);
    }
    return rbf_exclusive_scan_i64(ctx, w.as<int64_t>(), d_off, nsl + 1, sell_nnz);
}

int rbf_sell_fill_perm_device(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *d_rp, const int32_t *d_col,
                              const double *d_val, const int32_t *d_row_at, const int32_t *d_col_at,
                              const int64_t *d_off, int32_t *d_scol, double *d_sval) {
    if (ne == 0) return RBF_OK;
    DevBuf pos;
    RBF_TRY(pos.alloc(ctx, sizeof(int32_t) * (size_t)std::max<int64_t>(ns, 1)));
    if (ns > 0) {
        invert_perm_kernel<<<sell_blocks(ctx, ns, 256, 8), 256, 0, ctx->stream>>>(ns, d_col_at, pos.as<int32_t>());
        RBF_CHECK_LAUNCH(ctx);
    }
    sell_fill_perm_kernel<<<sell_blocks(ctx, ne, 256, 8), 256, 0, ctx->stream>>>(ne, d_rp, d_col, d_val, d_row_at,
                                                                                pos.as<int32_t>(), d_off, d_scol,
                                                                                d_sval);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_spmv_sell_perm_device(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *d_off, const int32_t *d_scol,
                              const double *d_sval, const int32_t *d_row_at, const int32_t *d_col_at,
                              const double *d_x, double *d_xwork, double alpha, double beta, double *d_y) {
    if (ne == 0) return RBF_OK;
    if (ns > 0) {
        gather_perm_kernel<<<sell_blocks(ctx, ns, 256, 8), 256, 0, ctx->stream>>>(ns, d_col_at, d_x, d_xwork);
        RBF_CHECK_LAUNCH(ctx);
    }
    spmv_sell_perm_kernel<6><<<sell_blocks(ctx, ne, 256, 8), 256, 0, ctx->stream>>>(ne, d_off, d_scol, d_sval,
                                                                                    d_row_at, d_xwork, alpha, beta,
                                                                                    d_y);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}
