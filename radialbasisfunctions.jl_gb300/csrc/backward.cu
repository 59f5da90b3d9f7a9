// Reverse-mode sensitivities of the built weights with respect to the point positions
// (replaces the backward rules of _build_weights: src/solve/backward.jl:31-522 with
// src/solve/ad_shared.jl:63-157).  Given the cotangent dW of the weights (CSR order), the
// gradients Δdata (ns x dim) and Δeval (ne x dim) of L = <dW, W>.
//
// Per stencil, one warp.  The forward system is assembled in the stencil's local coordinates
// X_i = (x_i - x0) s, s = 2^-es (as the forward build) and solved once for the weights λ
// (A λ = b) and the adjoint η (A η = [dW_i s^q; 0]: A is symmetric, and the global weights are
// λ s^q for an operator of order q): by an FP64 LU, or by the forward's FP32 factorisation
// refined with FP64 residuals (FP64 fallback).  With the implicit-function
// rule ΔA = -η λᵀ, Δb = η (backward.jl:31-58) and b_i = ℒφ(x0 - x_i):
//   ∂L/∂X_i = Σ_ops [ Σ_{j≠i} -(η_i λ_j + η_j λ_i) ∇φ(X_i - X_j)            (backward.jl:85-120)
//                     + Σ_m -(η_i λ_{k+m} + η_{k+m} λ_i) ∇p_m(X_i)        (backward.jl:122-145)
//                     - η_i ∇ℒφ(-X_i) ]                                   (backward.jl:160-200)
// Lane i owns point i; for k <= 32 each pair term is evaluated once and its odd partner share
// passed by a shuffle (otherwise lane i sums over all j).  The weights depend on the positions
// only through X, so Δdata[x_i] += s ∂L/∂X_i (atomics: a
// point belongs to many stencils) and Δeval[e] = -s Σ_i ∂L/∂X_i.  The polynomial
// right-hand side ℒp_m(x0) is constant in local coordinates.
// Supported: PHS 1/3/5/7, the identity (regrid), the Laplacian and first partials, interior
// stencils (no Hermite rows).  The gradients of the applied operators follow
// src/solve/operator_second_derivatives.jl, PHS1's rows vanishing below r = 1e-12.
#include <algorithm>

#include "stencil_solve.cuh"

namespace {

// ∇φ(D) for φ = r^p: p r^(p-2) D (PHS1: D / (r + guard))
__device__ __forceinline__ void grad_phi(int p, const double *D, int dim, double r, double a1, double *g) {
    const double c = p == 1 ? 1.0 / (r + a1)
                            : (p == 3 ? 3.0 * r : (p == 5 ? 5.0 * r * r * r : 7.0 * r * r * r * r * r));
    for (int d = 0; d < dim; d++) g[d] = c * D[d];
}

// ∇_D of the operator applied to φ at D (the right-hand-side entry); a1 the avoid-inf guard
// of an r denominator and r0 the radius below which PHS1's rows are zero, both in local units
__device__ __forceinline__ void grad_lphi(int p, int op, int od, const double *D, int dim, double r, double a1,
                                          double r0, double *g) {
    if (op == RBF_OP_IDENTITY) {
        grad_phi(p, D, dim, r, a1, g);
        return;
    }
    if (p == 1 && r < r0) {
        for (int d = 0; d < dim; d++) g[d] = 0.0;
        return;
    }
    if (op == RBF_OP_LAPLACIAN) {  // 2/r, 12 r, 30 r^3, 56 r^5
        const double c = p == 1 ? -2.0 / (r * r * r)
                                : (p == 3 ? 12.0 / (r + a1) : (p == 5 ? 90.0 * r : 280.0 * r * r * r));
        for (int d = 0; d < dim; d++) g[d] = c * D[d];
        return;
    }
    // first partial along od (D_od / r, 3 r D_od, 5 r^3 D_od, 7 r^5 D_od): row od of the Hessian
    const double dd = D[od];
    double a, b;  // gradient = a D_od D + b e_od
    if (p == 1) {
        a = -1.0 / (r * r * r);
        b = 1.0 / r;
    } else if (p == 3) {
        a = 3.0 / (r + a1);
        b = 3.0 * r;
    } else if (p == 5) {
        a = 15.0 * r;
        b = 5.0 * r * r * r;
    } else {
        a = 35.0 * r * r * r;
        b = 7.0 * r * r * r * r * r;
    }
    for (int d = 0; d < dim; d++) g[d] = a * dd * D[d] + (d == od ? b : 0.0);
}

// The kernels see the build's parameters with the operator list doubled (P2.nops = 2 nops):
// columns n .. n+nops-1 of the stencil system hold the forward right-hand sides, columns
// n+nops .. n+2nops-1 are assembled as a copy and overwritten with the adjoint's.

// The adjoint right-hand sides of stencil e: dW in the weights' CSR order, in local units,
// zero on the polynomial rows; scaled by a power of two that brings their largest entry to
// the forward right-hand sides' (so the refinement's relative acceptance weighs the weights
// and the adjoint alike; exact, undone on the solution).  Returns the inverse scale.
__device__ double adjoint_rhs(const StencilParams &P2, int nops, double *M, const int *cols, const double *dW,
                              int64_t e, int es, int lane) {
    const int k = P2.k, n = P2.n, ld = mat_ld(n, P2.nops);
    const int64_t rp = P2.row_ptr[e];
    const bool sorted = !(P2.flags & RBF_FLAG_STENCIL_ORDER);
    const bool local = (P2.flags & RBF_FLAG_LOCAL_UNITS) != 0;
    double amax = 0.0, bmax = 0.0;
    for (int i = lane; i < n; i += 32) {
        int rank = i;
        if (i < k && sorted) {
            rank = 0;
            const int ci = cols[i];
            for (int j = 0; j < k; j++) {
                const int cj = cols[j];
                rank += (cj < ci) || (cj == ci && j < i);
            }
        }
        for (int q = 0; q < nops; q++) {
            const double g = i < k ? dW[(int64_t)q * P2.nnz + rp + rank] : 0.0;
            const double v = local ? g : ldexp(g, -es * P2.op_order[q]);
            M[i * ld + n + nops + q] = v;
            amax = fmax(amax, fabs(v));
            bmax = fmax(bmax, fabs(M[i * ld + n + q]));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
        bmax = fmax(bmax, __shfl_xor_sync(0xffffffffu, bmax, o));
    }
    int ea = 0, eb = 0;
    if (amax > 0.0 && bmax > 0.0 && isfinite(amax) && isfinite(bmax)) {
        frexp(amax, &ea);
        frexp(bmax, &eb);
    }
    const int sh = eb - ea;
    __syncwarp();
    if (sh != 0)
        for (int i = lane; i < n; i += 32)
            for (int q = 0; q < nops; q++) M[i * ld + n + nops + q] = ldexp(M[i * ld + n + nops + q], sh);
    __syncwarp();
    return ldexp(1.0, -sh);
}

// ∂L/∂X_i for lane i from the weights λ (sol[i * rs + q]) and the scaled adjoint η
// (sol[i * rs + nops + q] * inv), then Δdata += s ∂L/∂X_i (atomics) and Δeval = -s Σ_i ∂L/∂X_i.
// The pair term -(η_i λ_j + η_j λ_i) ∇φ(X_i - X_j) is odd in (i, j): for k <= 32 each pair is
// evaluated once, in cyclic rounds (round d: lane i takes the pair (i, i + d mod k)), and the
// partner's share reaches its lane by a shuffle.
__device__ void accumulate_gradients(const StencilParams &P2, int nops, const double *X, const int *cols,
                                     const double *sol, int rs, double inv, int es, int64_t e, double *ddata,
                                     double *deval, int lane) {
    const int k = P2.k, dim = P2.dim, nmon = P2.nmon;
    const AvoidInf<double> AI = avoid_inf_scaled<double>(es);
    const double r0 = ldexp(1e-12, -es);  // PHS1's zero radius, local units
    const double s = ldexp(1.0, -es);
    double G[3] = {0.0, 0.0, 0.0};
    for (int i = lane; i < k; i += 32) {
        double gi[3] = {0.0, 0.0, 0.0};
        const double *xi = &X[i * 3];
        for (int q = 0; q < nops; q++) {
            const double lam_i = sol[i * rs + q], eta_i = sol[i * rs + nops + q] * inv;
            if (k > 32) {
                for (int j = 0; j < k; j++) {
                    if (j == i) continue;
                    const double sc = -(eta_i * sol[j * rs + q] + (sol[j * rs + nops + q] * inv) * lam_i);
                    double D[3], g[3];
                    for (int d = 0; d < dim; d++) D[d] = xi[d] - X[j * 3 + d];
                    grad_phi(P2.phs, D, dim, sqrt(sq_norm(D, dim)), AI.a1, g);
                    for (int d = 0; d < dim; d++) gi[d] += sc * g[d];
                }
            }
            for (int m = 0; m < nmon; m++) {
                const double sc = -(eta_i * sol[(k + m) * rs + q] + (sol[(k + m) * rs + nops + q] * inv) * lam_i);
                for (int d = 0; d < dim; d++) gi[d] += sc * mono_d1<double>(P2, m, d, xi);
            }
            double D[3], g[3];
            for (int d = 0; d < dim; d++) D[d] = -xi[d];
            grad_lphi(P2.phs, P2.op_code[q], P2.op_dim[q], D, dim, sqrt(sq_norm(D, dim)), AI.a1, r0, g);
            for (int d = 0; d < dim; d++) gi[d] -= eta_i * g[d];
        }
        for (int d = 0; d < dim; d++) G[d] += gi[d];
        if (k > 32)
            for (int d = 0; d < dim; d++) atomicAdd(&ddata[(int64_t)cols[i] * dim + d], s * gi[d]);
        else
            for (int d = 0; d < 3; d++) G[d] = gi[d];  // pair terms follow; G is lane i's point here
    }
    if (k <= 32) {
        // pair terms, each pair once; G holds lane i's sum so far (lanes >= k hold zeros)
        const bool act = lane < k;
        const double *xi = &X[(act ? lane : 0) * 3];
        for (int q = 0; q < nops; q++) {
            const double lam_i = act ? sol[lane * rs + q] : 0.0;
            const double eta_i = act ? sol[lane * rs + nops + q] * inv : 0.0;
            for (int dd = 1; dd <= k / 2; dd++) {
                int j = lane + dd;
                if (j >= k) j -= k;
                // round k/2 of an even k meets every pair twice: the lower lane takes it
                const bool use = act && (2 * dd != k || lane < dd);
                double c[3] = {0.0, 0.0, 0.0};
                if (use) {
                    const double sc = -(eta_i * sol[j * rs + q] + (sol[j * rs + nops + q] * inv) * lam_i);
                    double D[3], g[3];
                    for (int d = 0; d < dim; d++) D[d] = xi[d] - X[j * 3 + d];
                    grad_phi(P2.phs, D, dim, sqrt(sq_norm(D, dim)), AI.a1, g);
                    for (int d = 0; d < dim; d++) {
                        G[d] += sc * g[d];
                        c[d] = -sc * g[d];
                    }
                }
                int src = lane - dd;  // the lane whose pair ends at this lane's point
                if (src < 0) src += k;
                if (!act) src = lane;
                for (int d = 0; d < 3; d++) {
                    const double recv = __shfl_sync(0xffffffffu, c[d], src);
                    if (act) G[d] += recv;
                }
            }
        }
        if (act)
            for (int d = 0; d < dim; d++) atomicAdd(&ddata[(int64_t)cols[lane] * dim + d], s * G[d]);
    }
    for (int d = 0; d < 3; d++)
        for (int o = 16; o > 0; o >>= 1) G[d] += __shfl_xor_sync(0xffffffffu, G[d], o);
    if (lane < dim) deval[e * dim + lane] = -s * (lane == 0 ? G[0] : (lane == 1 ? G[1] : G[2]));
    __syncwarp();
}

// FP64: re-assemble, LU with both right-hand-side blocks, gradients
__global__ void build_backward_kernel(StencilParams P2, int nops, int wpb, size_t warp_bytes, const double *__restrict__ dW,
                                      double *__restrict__ ddata, double *__restrict__ deval) {
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WarpSmem w = carve(smem + wib * warp_bytes, P2.n, P2.k, P2.nops);
    const int n = P2.n, ld = mat_ld(n, P2.nops);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P2.ne; e += nwarps) {
        int es = 0, eval_local = -2;
        load_stencil(P2, e, w, lane, &es, &eval_local);  // interior stencils: the entry point rejects boundary data
        assemble_fp64(P2, w, lane, es, -2);
        const double inv = adjoint_rhs(P2, nops, w.M, w.cols, dW, e, es, lane);
        if (!lu_solve_fp64(w.M, n, P2.nops, lane)) {
            if (lane == 0) atomicAdd(&P2.counters[0], 1ull);
            __syncwarp();
            continue;
        }
        accumulate_gradients(P2, nops, w.X, w.cols, w.M + n, ld, inv, es, e, ddata, deval, lane);
    }
}

// FP32 factor + FP64-residual refinement of the weights and the adjoint together (the forward
// build's refined solve), FP64 fallback; then the gradients
__global__ void build_backward_refined_kernel(StencilParams P2, int nops, int wpb, size_t warp_bytes,
                                              const double *__restrict__ dW, double *__restrict__ ddata,
                                              double *__restrict__ deval) {
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    char *base = smem + wib * warp_bytes;
    WarpSmem w = carve(base, P2.n, P2.k, P2.nops);
    Warp32 u = carve32(base, P2.n, P2.k, P2.nops);
    const int n = P2.n, ld = mat_ld(n, P2.nops);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P2.ne; e += nwarps) {
        int es = 0, eval_local = -2;
        load_stencil(P2, e, w, lane, &es, &eval_local);
        assemble_refined(P2, w, u, lane, es, -2);
        double inv = adjoint_rhs(P2, nops, w.M, w.cols, dW, e, es, lane);
        const bool ok = lu_factor_fp32(u.F, u.piv, n, lane);
        double est = 0.0;
        if (ok && refine_fp32_warp(P2, w, u, lane, &est)) {
            accumulate_gradients(P2, nops, w.X, w.cols, u.x, P2.nops, inv, es, e, ddata, deval, lane);
            continue;
        }
        if (lane == 0) atomicAdd(&P2.counters[2], 1ull);
        assemble_fp64(P2, w, lane, es, -2);
        inv = adjoint_rhs(P2, nops, w.M, w.cols, dW, e, es, lane);
        if (!lu_solve_fp64(w.M, n, P2.nops, lane)) {
            if (lane == 0) atomicAdd(&P2.counters[0], 1ull);
            __syncwarp();
            continue;
        }
        accumulate_gradients(P2, nops, w.X, w.cols, w.M + n, ld, inv, es, e, ddata, deval, lane);
    }
}

template <class K>
int launch_backward(rbf_ctx *ctx, K kernel, size_t wb, const StencilParams &P2, int nops, const double *dW,
                    double *ddata, double *deval) {
    wb = (wb + 15) & ~(size_t)15;
    const int wpb = (int)std::max<size_t>(1, std::min<size_t>(4, (100 * 1024) / wb));
    const size_t smem = wb * wpb;
    RBF_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, wpb * 32, smem));
    if (per_sm < 1) per_sm = 1;
    const int64_t blocks = std::min<int64_t>((P2.ne + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
    kernel<<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P2, nops, wpb, wb, dW, ddata, deval);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

}  // namespace

// P: the build's parameters (nops operators); refined: FP32 factor + FP64 refinement
int rbf_backward_launch(rbf_ctx *ctx, const StencilParams &P, bool refined, const double *dW, double *ddata,
                        double *deval) {
    if (P.ne == 0) return RBF_OK;
    if (2 * P.nops > RBF_MAX_OPS) return rbf_fail(ctx, RBF_ERR_UNSUPPORTED, "the weight adjoint takes up to %d operators",
                                                  RBF_MAX_OPS / 2);
    StencilParams P2 = P;
    const int nops = P.nops;
    P2.nops = 2 * nops;
    for (int q = 0; q < nops; q++) {
        P2.op_code[nops + q] = P.op_code[q];
        P2.op_dim[nops + q] = P.op_dim[q];
        P2.op_order[nops + q] = P.op_order[q];
    }
    if (refined)
        return launch_backward(ctx, build_backward_refined_kernel, warp_smem_bytes32(P2.n, P2.k, P2.nops), P2, nops, dW,
                               ddata, deval);
    return launch_backward(ctx, build_backward_kernel, warp_smem_bytes(P2.n, P2.k, P2.nops), P2, nops, dW, ddata, deval);
}
