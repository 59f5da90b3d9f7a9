// Reverse-mode sensitivities of the built weights with respect to the point positions
// (replaces the backward rules of _build_weights: src/solve/backward.jl:31-522 with
// src/solve/ad_shared.jl:63-157).  Given the cotangent dW of the weights (CSR order), the
// gradients Δdata (ns x dim) and Δeval (ne x dim) of L = <dW, W>.
//
// Per stencil, one warp in FP64.  The forward system is assembled in the stencil's local
// coordinates X_i = (x_i - x0) s, s = 2^-es (as the forward build), factorised once and
// solved for the weights λ (A λ = b) and the adjoint η (A η = [dW_i s^q; 0]: A is symmetric,
// and the global weights are λ s^q for an operator of order q).  With the implicit-function
// rule ΔA = -η λᵀ, Δb = η (backward.jl:31-58) and b_i = ℒφ(x0 - x_i):
//   ∂L/∂X_i = Σ_ops [ Σ_{j≠i} -(η_i λ_j + η_j λ_i) ∇φ(X_i - X_j)            (backward.jl:85-120)
//                     + Σ_m -(η_i λ_{k+m} + η_{k+m} λ_i) ∇p_m(X_i)        (backward.jl:122-145)
//                     - η_i ∇ℒφ(-X_i) ]                                   (backward.jl:160-200)
// Lane i owns point i and sums over all j (each pair is evaluated twice, no atomics).  The
// weights depend on the positions only through X, so Δdata[x_i] += s ∂L/∂X_i (atomics: a
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

// per warp: the forward system with 2 * nops right-hand sides (b, then the adjoint's), the
// local coordinates and column indices
struct BackSmem {
    double *M, *X;
    int *cols;
};

__host__ __device__ inline size_t back_warp_bytes(int n, int k, int nops) {
    const size_t d = (size_t)n * mat_ld(n, 2 * nops) + 3 * (size_t)k;
    return ((d * sizeof(double) + sizeof(int) * (size_t)k) + 15) & ~(size_t)15;
}

__global__ void build_backward_kernel(StencilParams P, int wpb, size_t warp_bytes, const double *__restrict__ dW,
                                      double *__restrict__ ddata, double *__restrict__ deval) {
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    char *base = smem + wib * warp_bytes;
    const int k = P.k, n = P.n, nops = P.nops, dim = P.dim, nmon = P.nmon;
    const int ld = mat_ld(n, 2 * nops);
    BackSmem b;
    b.M = reinterpret_cast<double *>(base);
    b.X = b.M + (size_t)n * ld;
    b.cols = reinterpret_cast<int *>(b.X + 3 * k);
    // load_stencil and the forward assembly work on a WarpSmem whose matrix has room for
    // nops right-hand sides; the backward matrix (2 * nops) reuses its storage
    WarpSmem w;
    w.M = b.M;
    w.X = b.X;
    w.cols = b.cols;
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P.ne; e += nwarps) {
        int es = 0, eval_local = -2;
        // interior stencils only (the entry point rejects boundary data): no Hermite arrays
        {
            const int32_t *nbr = P.adjl + e * k;
            double x0[3] = {0, 0, 0};
            for (int d = 0; d < dim; d++) x0[d] = P.eval[e * dim + d];
            double r2max = 0.0;
            for (int i = lane; i < k; i += 32) {
                const int g = nbr[i];
                b.cols[i] = g;
                double r2 = 0.0;
                for (int d = 0; d < 3; d++) {
                    const double dd = d < dim ? P.data[(int64_t)g * dim + d] - x0[d] : 0.0;
                    b.X[i * 3 + d] = dd;
                    r2 += dd * dd;
                }
                r2max = fmax(r2max, r2);
            }
            for (int o = 16; o > 0; o >>= 1) r2max = fmax(r2max, __shfl_xor_sync(0xffffffffu, r2max, o));
            if (r2max > 0.0) frexp(sqrt(r2max), &es);
            __syncwarp();
            for (int i = lane; i < k; i += 32)
                for (int d = 0; d < dim; d++) b.X[i * 3 + d] = ldexp(b.X[i * 3 + d], -es);
            __syncwarp();
        }
        // forward system with its nops right-hand sides (row stride mat_ld(n, nops)), then
        // moved in place to the wider stride ld, last row first
        assemble_fp64(P, w, lane, es, eval_local);
        const int ld0 = mat_ld(n, nops);
        for (int r = n - 1; r >= 1; r--) {
            // rows move to higher addresses: read the whole row before writing it
            double v0 = lane < n + nops ? b.M[r * ld0 + lane] : 0.0;
            double v1 = lane + 32 < n + nops ? b.M[r * ld0 + lane + 32] : 0.0;
            double v2 = lane + 64 < n + nops ? b.M[r * ld0 + lane + 64] : 0.0;
            __syncwarp();
            if (lane < n + nops) b.M[r * ld + lane] = v0;
            if (lane + 32 < n + nops) b.M[r * ld + lane + 32] = v1;
            if (lane + 64 < n + nops) b.M[r * ld + lane + 64] = v2;
            __syncwarp();
        }
        // adjoint right-hand sides: dW in the weights' CSR order, scaled to local units
        const int64_t rp = P.row_ptr[e];
        const bool sorted = !(P.flags & RBF_FLAG_STENCIL_ORDER);
        const bool local = (P.flags & RBF_FLAG_LOCAL_UNITS) != 0;
        for (int i = lane; i < n; i += 32) {
            int rank = i;
            if (i < k && sorted) {
                rank = 0;
                const int ci = b.cols[i];
                for (int j = 0; j < k; j++) {
                    const int cj = b.cols[j];
                    rank += (cj < ci) || (cj == ci && j < i);
                }
            }
            for (int q = 0; q < nops; q++) {
                const double g = i < k ? dW[(int64_t)q * P.nnz + rp + rank] : 0.0;
                b.M[i * ld + n + nops + q] = local ? g : ldexp(g, -es * P.op_order[q]);
            }
        }
        __syncwarp();
        const bool ok = lu_solve_fp64(b.M, n, 2 * nops, lane);
        if (!ok) {
            if (lane == 0) atomicAdd(&P.counters[0], 1ull);
            __syncwarp();
            continue;
        }
        const AvoidInf<double> AI = avoid_inf_scaled<double>(es);
        const double r0 = ldexp(1e-12, -es);  // PHS1's zero radius, local units
        // ∂L/∂X_i, lane i
        double G[3] = {0.0, 0.0, 0.0};
        for (int i = lane; i < k; i += 32) {
            double gi[3] = {0.0, 0.0, 0.0};
            const double *xi = &b.X[i * 3];
            for (int q = 0; q < nops; q++) {
                const double lam_i = b.M[i * ld + n + q], eta_i = b.M[i * ld + n + nops + q];
                for (int j = 0; j < k; j++) {
                    if (j == i) continue;
                    const double sc = -(eta_i * b.M[j * ld + n + q] + b.M[j * ld + n + nops + q] * lam_i);
                    double D[3], g[3];
                    for (int d = 0; d < dim; d++) D[d] = xi[d] - b.X[j * 3 + d];
                    grad_phi(P.phs, D, dim, sqrt(sq_norm(D, dim)), AI.a1, g);
                    for (int d = 0; d < dim; d++) gi[d] += sc * g[d];
                }
                for (int m = 0; m < nmon; m++) {
                    const double sc = -(eta_i * b.M[(k + m) * ld + n + q] + b.M[(k + m) * ld + n + nops + q] * lam_i);
                    for (int d = 0; d < dim; d++) gi[d] += sc * mono_d1<double>(P, m, d, xi);
                }
                double D[3], g[3];
                for (int d = 0; d < dim; d++) D[d] = -xi[d];
                grad_lphi(P.phs, P.op_code[q], P.op_dim[q], D, dim, sqrt(sq_norm(D, dim)), AI.a1, r0, g);
                for (int d = 0; d < dim; d++) gi[d] -= eta_i * g[d];
            }
            const double s = ldexp(1.0, -es);
            for (int d = 0; d < dim; d++) {
                atomicAdd(&ddata[(int64_t)b.cols[i] * dim + d], s * gi[d]);
                G[d] += gi[d];
            }
        }
        for (int d = 0; d < 3; d++)
            for (int o = 16; o > 0; o >>= 1) G[d] += __shfl_xor_sync(0xffffffffu, G[d], o);
        if (lane < dim) {
            const double s = ldexp(1.0, -es);
            deval[e * dim + lane] = -s * (lane == 0 ? G[0] : (lane == 1 ? G[1] : G[2]));
        }
        __syncwarp();
    }
}

}  // namespace

int rbf_backward_launch(rbf_ctx *ctx, const StencilParams &P, const double *dW, double *ddata, double *deval) {
    if (P.ne == 0) return RBF_OK;
    const size_t wb = back_warp_bytes(P.n, P.k, P.nops);
    const int wpb = (int)std::max<size_t>(1, std::min<size_t>(4, (100 * 1024) / wb));
    const size_t smem = wb * wpb;
    RBF_CUDA(ctx, cudaFuncSetAttribute(build_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_backward_kernel, wpb * 32, smem));
    if (per_sm < 1) per_sm = 1;
    const int64_t blocks = std::min<int64_t>((P.ne + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
    build_backward_kernel<<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P, wpb, wb, dW, ddata, deval);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}
