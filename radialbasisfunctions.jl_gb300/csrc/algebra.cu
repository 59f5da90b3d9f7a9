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
__device__ __forceinline__ double axpby_one(double av, double bv, bool has_b, const Scale &A, const Scale &B) {
    const double t = APOW2 ? mul_pow2(av, A.sh, A.neg, A.s) : __dmul_rn(A.s, av);
    if (!has_b) return t;
    const double u = BPOW2 ? mul_pow2(bv, B.sh, B.neg, B.s) : __dmul_rn(B.s, bv);
    return __dadd_rn(t, u);
}

// VEC: every pointer 16-byte aligned; a thread then moves four entries per step as two
// 16-byte loads per input and two stores (more bytes in flight per thread: the pass is a
// stream), the scalar tail after the last whole group of four
template <bool APOW2, bool BPOW2, bool VEC>
__global__ void axpby_kernel(int64_t n, Scale A, const double *__restrict__ a, Scale B,
                             const double *__restrict__ b, double *__restrict__ out) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
    const bool hb = b != nullptr;
    int64_t done = 0;
    if (VEC) {
        const int64_t n4 = n >> 2;
        for (int64_t g = tid; g < n4; g += nt) {
            const double2 a0 = __ldcs(reinterpret_cast<const double2 *>(a) + 2 * g);
            const double2 a1 = __ldcs(reinterpret_cast<const double2 *>(a) + 2 * g + 1);
            double2 b0 = make_double2(0.0, 0.0), b1 = b0;
            if (hb) {
                b0 = __ldcs(reinterpret_cast<const double2 *>(b) + 2 * g);
                b1 = __ldcs(reinterpret_cast<const double2 *>(b) + 2 * g + 1);
            }
            const double2 o0 = make_double2(axpby_one<APOW2, BPOW2>(a0.x, b0.x, hb, A, B),
                                            axpby_one<APOW2, BPOW2>(a0.y, b0.y, hb, A, B));
            const double2 o1 = make_double2(axpby_one<APOW2, BPOW2>(a1.x, b1.x, hb, A, B),
                                            axpby_one<APOW2, BPOW2>(a1.y, b1.y, hb, A, B));
            __stcs(reinterpret_cast<double2 *>(out) + 2 * g, o0);
            __stcs(reinterpret_cast<double2 *>(out) + 2 * g + 1, o1);
        }
        done = n4 << 2;
    }
    for (int64_t p = done + tid; p < n; p += nt) out[p] = axpby_one<APOW2, BPOW2>(a[p], hb ? b[p] : 0.0, hb, A, B);
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
    const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(out)) &
                      15u) == 0;
    const int g = algebra_blocks(ctx, vec ? (nnz + 3) / 4 : nnz);
    const bool ap = A.pow2, bp = B.pow2 || !b;
#define RBF_AXPBY(AP, BP)                                                                       \
    do {                                                                                        \
        if (vec)                                                                                \
            axpby_kernel<AP, BP, true><<<g, 256, 0, ctx->stream>>>(nnz, A, a, B, b, out);       \
        else                                                                                    \
            axpby_kernel<AP, BP, false><<<g, 256, 0, ctx->stream>>>(nnz, A, a, B, b, out);      \
    } while (0)
    if (ap && bp)
        RBF_AXPBY(true, true);
    else if (ap)
        RBF_AXPBY(true, false);
    else if (bp)
        RBF_AXPBY(false, true);
    else
        RBF_AXPBY(false, false);
#undef RBF_AXPBY
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
