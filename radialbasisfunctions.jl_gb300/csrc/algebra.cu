// Operator algebra on built weights, on the device (replaces the host-side sparse-matrix
// arithmetic of src/operators/operator_algebra.jl:245-295 and the weight combination of
// src/operators/directional.jl:69-82).
//
// Operators built on the same stencils share their CSR structure (row_ptr, col), so a sum,
// a difference or a scaling is an entry-wise combination of the value arrays:
//   out = alpha * a + beta * b          (rbf_weights_axpby; beta = 0 scales a)
// and the directional derivative sum_i v_i d/dx_i combines the D gradient value arrays of
// one Jacobian build:
//   out[p] = sum_i v_i(row(p)) * val_i[p]   (v constant: one vector; else one per row)
// The products and sums are rounded separately (no fused multiply-add), in the order the
// reference's broadcasts evaluate them, so the results equal the host arithmetic bit for
// bit (scalings by powers of two, +-1 included, are exact and move the exponent on the
// integer pipe).  Roofline: HBM; bytes (inputs + output) * 8 per entry.
#include <algorithm>
#include <cmath>

#include "rbf_internal.cuh"

namespace {

// s * x for s = +-2^sh, exactly as __dmul_rn(s, x) rounds it: when x and the product are
// normal numbers the product is x with its exponent moved (and the sign flipped for s < 0),
// done on the integer pipe; zeros, subnormals, infinities, NaNs and products leaving the
// normal range take the FP64 multiply.  On GB300 the FP64 pipe, not HBM, would otherwise
// bound this pass (2 multiplies + 1 add per entry against 24 bytes).
__device__ __forceinline__ double mul_pow2(double x, int sh, bool neg, double s) {
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    const int ee = e + sh;
    if (e != 0 && e != 0x7ff && ee > 0 && ee < 0x7ff)
        return __longlong_as_double((b + ((long long)sh << 52)) ^ (neg ? (long long)0x8000000000000000ull : 0ll));
    return __dmul_rn(s, x);
}

struct Scale {
    double s;
    int sh;     // s = +-2^sh when pow2
    bool neg, pow2;
};

template <bool APOW2, bool BPOW2>
__global__ void axpby_kernel(int64_t n, Scale A, const double *__restrict__ a, Scale B,
                             const double *__restrict__ b, double *__restrict__ out) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const double t = APOW2 ? mul_pow2(a[p], A.sh, A.neg, A.s) : __dmul_rn(A.s, a[p]);
        if (b) {
            const double u = BPOW2 ? mul_pow2(b[p], B.sh, B.neg, B.s) : __dmul_rn(B.s, b[p]);
            out[p] = __dadd_rn(t, u);
        } else {
            out[p] = t;
        }
    }
}

Scale make_scale(double s) {
    Scale c{s, 0, s < 0.0, false};
    int ex = 0;
    const double m = std::frexp(std::fabs(s), &ex);  // |s| = m 2^ex, m in [0.5, 1)
    if (std::isfinite(s) && s != 0.0 && m == 0.5 && ex - 1 > -1022 && ex - 1 < 1023) {
        c.pow2 = true;
        c.sh = ex - 1;
    }
    return c;
}

// one warp per row: the row's entries are contiguous, the direction of the row is read once
__global__ void directional_kernel(int64_t ne, const int64_t *__restrict__ rp, int nd, const double *__restrict__ val,
                                   int64_t nnz, const double *__restrict__ v, int per_row, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < ne; r += nwarps) {
        const double *vr = v + (per_row ? r * nd : 0);
        const int64_t a = rp[r], b = rp[r + 1];
        for (int64_t p = a + lane; p < b; p += 32) {
            double s = __dmul_rn(vr[0], val[p]);
            for (int i = 1; i < nd; i++) s = __dadd_rn(s, __dmul_rn(vr[i], val[(int64_t)i * nnz + p]));
            out[p] = s;
        }
    }
}

int algebra_blocks(rbf_ctx *ctx, int64_t work) {
    int64_t b = (work + 255) / 256;
    b = std::min<int64_t>(b, (int64_t)ctx->num_sms * 8);
    return (int)std::max<int64_t>(b, 1);
}

}  // namespace

int rbf_weights_axpby_device(rbf_ctx *ctx, int64_t nnz, double alpha, const double *a, double beta, const double *b,
                             double *out) {
    if (nnz == 0) return RBF_OK;
    const Scale A = make_scale(alpha), B = make_scale(beta);
    const int g = algebra_blocks(ctx, nnz);
    if (A.pow2 && (B.pow2 || !b))
        axpby_kernel<true, true><<<g, 256, 0, ctx->stream>>>(nnz, A, a, B, b, out);
    else if (A.pow2)
        axpby_kernel<true, false><<<g, 256, 0, ctx->stream>>>(nnz, A, a, B, b, out);
    else if (B.pow2 || !b)
        axpby_kernel<false, true><<<g, 256, 0, ctx->stream>>>(nnz, A, a, B, b, out);
    else
        axpby_kernel<false, false><<<g, 256, 0, ctx->stream>>>(nnz, A, a, B, b, out);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_weights_directional_device(rbf_ctx *ctx, int64_t ne, const int64_t *rp, int nd, const double *val,
                                   int64_t nnz, const double *v, int per_row, double *out) {
    if (ne == 0) return RBF_OK;
    directional_kernel<<<algebra_blocks(ctx, ne * 32), 256, 0, ctx->stream>>>(ne, rp, nd, val, nnz, v, per_row, out);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}
