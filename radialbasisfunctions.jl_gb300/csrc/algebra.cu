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
// bit.  Roofline: HBM; bytes (inputs + output) * 8 per entry.
#include <algorithm>

#include "rbf_internal.cuh"

namespace {

__global__ void axpby_kernel(int64_t n, double alpha, const double *__restrict__ a, double beta,
                             const double *__restrict__ b, double *__restrict__ out) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const double t = __dmul_rn(alpha, a[p]);
        out[p] = b ? __dadd_rn(t, __dmul_rn(beta, b[p])) : t;
    }
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
    axpby_kernel<<<algebra_blocks(ctx, nnz), 256, 0, ctx->stream>>>(nnz, alpha, a, beta, b, out);
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
