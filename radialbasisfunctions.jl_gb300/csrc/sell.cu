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
