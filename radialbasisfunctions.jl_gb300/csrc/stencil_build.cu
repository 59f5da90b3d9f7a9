// Weight build kernels: one warp per stencil, the saddle-point system staged in shared
// memory, and the scatter of the solved row into its CSR slot with columns ascending.
//   plain FP64:        LU with partial pivoting in FP64.
//   FP32 + refinement: the same FP64 assembly is rounded to FP32 and factorised there;
//                      iterative refinement with FP64 residuals (including the polynomial
//                      reproduction rows P^T w = L(p)) recovers FP64 accuracy, and a stencil
//                      whose normwise backward error stays above tolerance is re-solved by
//                      the plain FP64 LU (status 3).
//
// Replaces the per-stencil loop of launch_kernel! (src/solve/execution.jl:186-265):
// classify_stencil (src/solve/types.jl:208-223), _build_stencil! /
// _build_collocation_matrix_impl! / _build_rhs! (src/solve/assembly.jl:95-217),
// _solve_system! (assembly.jl:220-222, rook Bunch-Kaufman on the raw-coordinate
// system), fill_entries! / fill_dirichlet_entry! (execution.jl:279-303) and the COO->CSC
// sort of _construct_sparse (execution.jl:105-115).  Assembly happens in scaled local
// coordinates (stencil_common.cuh), which gives the same weights to within rounding.
//
// Shared memory per warp: M[n][ld] (ld = n + nops: matrix | right-hand sides), local
// coordinates X[k][3], Hermite data (alpha, beta/s, normal, point type) and the k column
// indices.  Dominant cost: the LU update, n^3/3 FP64 FMA per stencil.
#include <algorithm>
#include <cmath>

#include "stencil_device.cuh"

#define RBF_LAUNCH_NO_VARIANT 1000
int rbf_launch_refined_reg_a(rbf_ctx *ctx, const StencilParams &P);
int rbf_launch_refined_reg_b(rbf_ctx *ctx, const StencilParams &P);

namespace {

__global__ void build_fp64_kernel(StencilParams P, int wpb, size_t warp_bytes) {
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WarpSmem w = carve(smem + wib * warp_bytes, P.n, P.k, P.nops);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P.ne; e += nwarps) {
        int es = 0, eval_local = -2;
        int st = load_stencil(P, e, w, lane, &es, &eval_local);
        if (st != 0) {
            __syncwarp();
            continue;
        }
        assemble_fp64(P, w, lane, es, eval_local);
        bool ok = lu_solve_fp64(w.M, P.n, P.nops, lane);
        if (!ok) {
            if (lane == 0) {
                if (P.status) P.status[e] = 1;
                atomicAdd(&P.counters[0], 1ull);
            }
            __syncwarp();
            continue;
        }
        scatter_row(P, e, w, lane, es, w.M + P.n, mat_ld(P.n, P.nops), 1);
        if (lane == 0 && P.status) P.status[e] = 0;
        __syncwarp();
    }
}


__global__ void build_fp32r_kernel(StencilParams P, int wpb, size_t warp_bytes) {
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    char *base = smem + wib * warp_bytes;
    WarpSmem w = carve(base, P.n, P.k, P.nops);
    Warp32 u = carve32(base, P.n, P.k, P.nops);
    const int n = P.n, nops = P.nops, ld = mat_ld(n, nops), fld = f32_ld(n);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P.ne; e += nwarps) {
        int es = 0, eval_local = -2;
        int st = load_stencil(P, e, w, lane, &es, &eval_local);
        if (st != 0) {
            __syncwarp();
            continue;
        }
        assemble_refined(P, w, u, lane, es, eval_local);
        bool ok = lu_factor_fp32(u.F, u.piv, n, lane);
        bool accepted = false;
        double est_final = 0.0;
        if (ok) {
            // x0 = A32^{-1} b; then x += A32^{-1} (b - A x) with the residual in FP64.  The
            // correction computed from the FP64 residual of x_{s-1} estimates its error; x is
            // accepted once that correction, on the weights and on the polynomial
            // multipliers, is below tol relative to x.
            for (int t = lane; t < n * nops; t += 32) {
                int i = t / nops, q = t % nops;
                u.v[t] = __double2float_rn(w.M[i * ld + n + q]);
                u.x[t] = 0.0;
            }
            __syncwarp();
            float dprev = 0.0f;
            const float tolf = (float)P.tol;
            for (int step = 0;; step++) {
                lu_apply_fp32(u.F, u.piv, u.v, n, nops, lane);
                // |d| and |x| compared in FP32 (only their ratio matters)
                float dmaxf = 0.0f, xmaxf = 0.0f;
                for (int t = lane; t < n * nops; t += 32) {
                    const float df = u.v[t];
                    u.x[t] += widen(df);
                    if (t / nops < P.k) {
                        dmaxf = fmaxf(dmaxf, fabsf(df));
                        xmaxf = fmaxf(xmaxf, fabsf(__double2float_rn(u.x[t])));
                    }
                }
                for (int o = 16; o > 0; o >>= 1) {
                    dmaxf = fmaxf(dmaxf, __shfl_xor_sync(0xffffffffu, dmaxf, o));
                    xmaxf = fmaxf(xmaxf, __shfl_xor_sync(0xffffffffu, xmaxf, o));
                }
                __syncwarp();
                // the first correction measures the FP32 solve's error, about cond(A) * 2^-24;
                // past 1e-3 (cond ~ 1e5) the double-float entries (~2^-44) could move the
                // weights by more than 1e-9, so such a stencil takes the FP64 path.  |d_s|
                // estimates the error before a correction: accept once it is below tol and
                // shrinking, so that the error left after adding it is below tol as well.
                if (step == 0) {
                    dprev = xmaxf;
                } else {
                    if (step == 1 && !(dmaxf <= 1e-3f * dprev)) break;
                    if (dmaxf <= tolf * xmaxf && dmaxf <= 0.5f * dprev) {
                        accepted = true;
                        est_final = xmaxf > 0.0f ? (double)(dmaxf / xmaxf) : 0.0;
                        break;
                    }
                    dprev = dmaxf;
                }
                if (step >= P.refine_steps || !isfinite(dmaxf)) break;
                // FP64 residual r = b - A x (A symmetric: read column i as row i); rows k..n-1
                // are the polynomial-reproduction constraints P^T w = L(p)
                if (lane == 0) atomicAdd(&P.counters[4], 1ull);
                for (int i = lane; i < n; i += 32) {
                    for (int q = 0; q < nops; q++) {
                        double acc = w.M[i * ld + n + q];
                        for (int j = 0; j < n; j++) acc = fma(-w.M[j * ld + i], u.x[j * nops + q], acc);
                        u.v[i * nops + q] = __double2float_rn(acc);
                    }
                }
                __syncwarp();
            }
        }
        if (accepted) {
            scatter_row(P, e, w, lane, es, u.x, nops, 1);
            if (lane == 0) {
                if (P.status) P.status[e] = 0;
                atomicMax(reinterpret_cast<unsigned long long *>(P.max_resid),
                          (unsigned long long)__double_as_longlong(est_final));
            }
        } else {
            // fallback: the plain FP64 assembly and solve
            if (eval_local == -2) assemble_fp64(P, w, lane, es, eval_local);
            bool ok64 = lu_solve_fp64(w.M, n, nops, lane);
            if (ok64) {
                scatter_row(P, e, w, lane, es, w.M + n, ld, 1);
                if (lane == 0) {
                    if (P.status) P.status[e] = 3;
                    atomicAdd(&P.counters[2], 1ull);
                }
            } else if (lane == 0) {
                if (P.status) P.status[e] = 1;
                atomicAdd(&P.counters[0], 1ull);
            }
        }
        __syncwarp();
    }
}


}  // namespace

size_t rbf_fp64_warp_smem(int n, int k, int nops) { return (warp_smem_bytes(n, k, nops) + 15) & ~(size_t)15; }

int rbf_build_fp64_launch(rbf_ctx *ctx, const StencilParams &P) {
    if (P.ne == 0) return RBF_OK;
    const size_t wb = rbf_fp64_warp_smem(P.n, P.k, P.nops);
    int wpb = (int)std::max<size_t>(1, std::min<size_t>(8, (100 * 1024) / wb));
    size_t smem = wb * wpb;
    RBF_CUDA(ctx, cudaFuncSetAttribute(build_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_fp64_kernel, wpb * 32, smem));
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = std::min<int64_t>((P.ne + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
    build_fp64_kernel<<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P, wpb, wb);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_build_fp32_launch(rbf_ctx *ctx, const StencilParams &P) {
    if (P.ne == 0) return RBF_OK;
    // register-resident kernels for the standard system sizes (they need 3k >= n for the
    // reciprocal-pivot buffer that reuses the split-coordinate space)
    if (3 * P.k >= P.n) {
        int st = rbf_launch_refined_reg_a(ctx, P);
        if (st != RBF_LAUNCH_NO_VARIANT) return st;
        st = rbf_launch_refined_reg_b(ctx, P);
        if (st != RBF_LAUNCH_NO_VARIANT) return st;
    }
    const size_t wb = warp_smem_bytes32(P.n, P.k, P.nops);
    int wpb = (int)std::max<size_t>(1, std::min<size_t>(8, (100 * 1024) / wb));
    size_t smem = wb * wpb;
    RBF_CUDA(ctx, cudaFuncSetAttribute(build_fp32r_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_fp32r_kernel, wpb * 32, smem));
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = std::min<int64_t>((P.ne + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
    build_fp32r_kernel<<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P, wpb, wb);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}
