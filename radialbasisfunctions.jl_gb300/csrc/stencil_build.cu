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

#include "rbf_internal.cuh"
#include "stencil_common.cuh"

namespace {

struct WarpSmem {
    double *M, *X, *HA, *HB, *HN;
    int *cols, *ptype;
};

__host__ __device__ inline int mat_ld(int n, int nops) { return (n + nops) | 1; }  // odd: no bank conflicts

__host__ __device__ inline size_t warp_smem_bytes(int n, int k, int nops) {
    size_t d = (size_t)n * mat_ld(n, nops) + 3 * (size_t)k + 2 * (size_t)k + 3 * (size_t)k;
    return d * sizeof(double) + 2 * (size_t)k * sizeof(int);
}

__device__ inline WarpSmem carve(char *base, int n, int k, int nops) {
    WarpSmem w;
    double *p = reinterpret_cast<double *>(base);
    w.M = p;
    p += (size_t)n * mat_ld(n, nops);
    w.X = p;
    p += 3 * k;
    w.HA = p;
    p += k;
    w.HB = p;
    p += k;
    w.HN = p;
    p += 3 * k;
    w.cols = reinterpret_cast<int *>(p);
    w.ptype = w.cols + k;
    return w;
}

// Loads the stencil, classifies it and fills X/cols/Hermite data.  Returns
//  0: solve needed, 2: Dirichlet identity row written, -1: eval point not in stencil.
__device__ int load_stencil(const StencilParams &P, int64_t e, const WarpSmem &w, int lane, int *es_out,
                            int *eval_local_out) {
    const int k = P.k, dim = P.dim;
    double x0[3] = {0, 0, 0};
    for (int d = 0; d < dim; d++) x0[d] = P.eval[e * dim + d];
    double r2max = 0.0;
    bool anyb = false;
    for (int i = lane; i < k; i += 32) {
        int g = P.adjl[e * k + i];
        w.cols[i] = g;
        double r2 = 0.0;
        for (int d = 0; d < dim; d++) {
            double dd = P.data[(int64_t)g * dim + d] - x0[d];
            w.X[i * 3 + d] = dd;
            r2 += dd * dd;
        }
        r2max = fmax(r2max, r2);
        if (P.isb) anyb |= (P.isb[g] != 0);
    }
    for (int o = 16; o > 0; o >>= 1) r2max = fmax(r2max, __shfl_xor_sync(0xffffffffu, r2max, o));
    anyb = __any_sync(0xffffffffu, anyb);
    int es = 0;
    if (r2max > 0.0) frexp(sqrt(r2max), &es);
    *es_out = es;
    __syncwarp();
    for (int i = lane; i < k; i += 32)
        for (int d = 0; d < dim; d++) w.X[i * 3 + d] = ldexp(w.X[i * 3 + d], -es);
    int eval_local = -1;
    if (anyb) {
        // Dirichlet eval node: identity row (execution.jl:224-228, 297-303)
        if (P.isb[e]) {
            int32_t b = P.g2b[e];
            if (P.alpha[b] == 1.0 && P.beta[b] == 0.0) {
                if (lane == 0) {
                    int64_t p = P.row_ptr[e];
                    P.col[p] = (int32_t)e;
                    for (int r = 0; r < P.nops; r++) P.val[r * P.nnz + p] = 1.0;
                    if (P.status) P.status[e] = 2;
                    atomicAdd(&P.counters[3], 1ull);
                }
                return 2;
            }
        }
        const double sinv = ldexp(1.0, -es);
        bool found = false;
        int first = 0x7fffffff;
        for (int i = lane; i < k; i += 32) {
            int g = w.cols[i];
            bool same = true;
            for (int d = 0; d < dim; d++) same &= (w.X[i * 3 + d] == 0.0);
            if (same && i < first) first = i;
            found |= same;
            if (P.isb[g]) {
                int32_t b = P.g2b[g];
                double a = P.alpha[b], bt = P.beta[b];
                w.ptype[i] = (a == 1.0 && bt == 0.0) ? PT_DIRICHLET : PT_NR;
                w.HA[i] = a;
                w.HB[i] = bt * sinv;
                for (int d = 0; d < 3; d++) w.HN[i * 3 + d] = d < dim ? P.normals[(int64_t)b * dim + d] : 0.0;
            } else {
                w.ptype[i] = PT_INTERIOR;
                w.HA[i] = 0.0;
                w.HB[i] = 0.0;
                for (int d = 0; d < 3; d++) w.HN[i * 3 + d] = 0.0;
            }
        }
        for (int o = 16; o > 0; o >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
        eval_local = (first == 0x7fffffff) ? -1 : first;
        if (eval_local < 0 && P.nmon > 0) {
            if (lane == 0) {
                if (P.status) P.status[e] = -1;
                atomicAdd(&P.counters[1], 1ull);
            }
            return -1;
        }
    } else {
        for (int i = lane; i < k; i += 32) w.ptype[i] = PT_INTERIOR;
    }
    *eval_local_out = anyb ? eval_local : -2;  // -2: interior stencil
    __syncwarp();
    return 0;
}

// Assemble [Phi P; P^T 0 | B] into M (full symmetric storage).
__device__ void assemble_fp64(const StencilParams &P, const WarpSmem &w, int lane, int es, int eval_local) {
    const int k = P.k, n = P.n, nops = P.nops, ld = mat_ld(n, nops), dim = P.dim, nmon = P.nmon;
    const bool herm = eval_local != -2;
    const AvoidInf<double> AI = avoid_inf_scaled<double>(es);
    for (int t = lane; t < n * ld; t += 32) w.M[t] = 0.0;
    __syncwarp();
    // RBF block, upper triangle pairs (i <= j) mirrored
    const int npairs = k * (k + 1) / 2;
    for (int p = lane; p < npairs; p += 32) {
        int j = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
        while (j * (j + 1) / 2 > p) j--;
        while ((j + 1) * (j + 2) / 2 <= p) j++;
        int i = p - j * (j + 1) / 2;
        double v;
        if (!herm) {
            double D[3];
            for (int d = 0; d < dim; d++) D[d] = w.X[i * 3 + d] - w.X[j * 3 + d];
            v = phs_phi_r2<double>(P.phs, sq_norm(D, dim));
        } else {
            v = colloc_entry<double>(P.phs, dim, &w.X[i * 3], &w.X[j * 3], w.ptype[i], w.ptype[j], w.HA[i], w.HB[i],
                                     &w.HN[i * 3], w.HA[j], w.HB[j], &w.HN[j * 3], AI);
        }
        w.M[i * ld + j] = v;
        w.M[j * ld + i] = v;
    }
    // polynomial block and RBF right-hand sides, one stencil point per lane
    for (int i = lane; i < k; i += 32) {
        const double *xi = &w.X[i * 3];
        const bool nr = herm && w.ptype[i] == PT_NR;
        for (int m = 0; m < nmon; m++) {
            double v = mono_val<double>(P, m, xi);
            if (nr) {
                double dn = 0.0;
                for (int d = 0; d < dim; d++)
                    if (w.HN[i * 3 + d] != 0.0) dn += w.HN[i * 3 + d] * mono_d1<double>(P, m, d, xi);
                v = w.HA[i] * v + w.HB[i] * dn;
            }
            w.M[i * ld + k + m] = v;
            w.M[(k + m) * ld + i] = v;
        }
        double D[3];
        for (int d = 0; d < dim; d++) D[d] = -xi[d];  // x0 - xi in local coordinates
        for (int r = 0; r < nops; r++) {
            double b = phs_op<double>(P.phs, P.op_code[r], P.op_dim[r], D, dim, AI);
            if (nr)
                b = w.HA[i] * b +
                    w.HB[i] * phs_op_normal<double>(P.phs, P.op_code[r], P.op_dim[r], D, &w.HN[i * 3], dim, AI);
            w.M[i * ld + n + r] = b;
        }
    }
    // polynomial right-hand sides at the eval point (local origin)
    for (int t = lane; t < nmon * nops; t += 32) {
        int m = t / nops, r = t % nops;
        double v;
        if (herm && eval_local >= 0 && w.ptype[eval_local] == PT_NR) {
            // Neumann/Robin eval node: alpha*P(x0) + beta*dP/dn(x0) (assembly.jl:452-468)
            double nrm[3] = {w.HN[eval_local * 3], w.HN[eval_local * 3 + 1], w.HN[eval_local * 3 + 2]};
            v = w.HA[eval_local] * mono_op_at_origin(P, m, RBF_OP_IDENTITY, 0) +
                w.HB[eval_local] * mono_normal_at_origin(P, m, nrm);
            v = ldexp(v, es * P.op_order[r]);
        } else {
            v = mono_op_at_origin(P, m, P.op_code[r], P.op_dim[r]);
        }
        w.M[(k + m) * ld + n + r] = v;
    }
    __syncwarp();
}

// In-place LU with partial pivoting of M[:, 0:n] applied to the right-hand sides, then
// back substitution.  Returns false if a pivot is exactly zero or not finite.
__device__ bool lu_solve_fp64(double *M, int n, int nops, int lane) {
    const int ld = mat_ld(n, nops), W = n + nops;
    for (int c = 0; c < n; c++) {
        double bv = -1.0;
        int br = n;
        for (int r = c + lane; r < n; r += 32) {
            double v = fabs(M[r * ld + c]);
            if (v > bv) {
                bv = v;
                br = r;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            double ov = __shfl_xor_sync(0xffffffffu, bv, o);
            int orr = __shfl_xor_sync(0xffffffffu, br, o);
            if (ov > bv || (ov == bv && orr < br)) {
                bv = ov;
                br = orr;
            }
        }
        if (!(bv > 0.0) || !isfinite(bv)) return false;
        if (br != c) {
            for (int cc = c + lane; cc < W; cc += 32) {
                double a = M[c * ld + cc];
                M[c * ld + cc] = M[br * ld + cc];
                M[br * ld + cc] = a;
            }
        }
        __syncwarp();
        const double inv = 1.0 / M[c * ld + c];
        for (int r = c + 1 + lane; r < n; r += 32) M[r * ld + c] *= inv;
        __syncwarp();
        const int rows = n - c - 1, cols = W - c - 1;
        if (rows > 0) {
            const int total = rows * cols;
            int r = lane / cols, cc = lane % cols;
            const int dr = 32 / cols, dc = 32 % cols;
            const double *prow = M + c * ld + c + 1;
            for (int t = lane; t < total; t += 32) {
                double *row = M + (c + 1 + r) * ld;
                row[c + 1 + cc] = fma(-row[c], prow[cc], row[c + 1 + cc]);
                r += dr;
                cc += dc;
                if (cc >= cols) {
                    cc -= cols;
                    r++;
                }
            }
        }
        __syncwarp();
    }
    for (int c = n - 1; c >= 0; c--) {
        if (lane < nops) M[c * ld + n + lane] = M[c * ld + n + lane] / M[c * ld + c];
        __syncwarp();
        const int total = c * nops;
        for (int t = lane; t < total; t += 32) {
            int r = t / nops, q = t - (t / nops) * nops;
            M[r * ld + n + q] = fma(-M[r * ld + c], M[c * ld + n + q], M[r * ld + n + q]);
        }
        __syncwarp();
    }
    return true;
}

// Writes the solved weights of stencil e into its CSR row, columns ascending.
__device__ void scatter_row(const StencilParams &P, int64_t e, const WarpSmem &w, int lane, int es,
                            const double *sol, int sol_ld, int sol_stride) {
    const int k = P.k;
    const int64_t base = P.row_ptr[e];
    for (int i = lane; i < k; i += 32) {
        const int ci = w.cols[i];
        int rank = 0;
        for (int j = 0; j < k; j++) {
            int cj = w.cols[j];
            rank += (cj < ci) || (cj == ci && j < i);
        }
        P.col[base + rank] = ci;
        for (int r = 0; r < P.nops; r++)
            P.val[r * P.nnz + base + rank] = ldexp(sol[i * sol_ld + r * sol_stride], -es * P.op_order[r]);
    }
}

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


// ---------------------------------------------------------------------------------------
// FP32 factorisation + FP64 iterative refinement
// ---------------------------------------------------------------------------------------
__host__ __device__ inline int f32_ld(int n) { return n | 1; }

__host__ __device__ inline size_t warp_smem_bytes32(int n, int k, int nops) {
    size_t b = warp_smem_bytes(n, k, nops);
    b = (b + 15) & ~(size_t)15;
    b += sizeof(double) * 2 * (size_t)n * nops;  // solution x, residual r
    b += sizeof(float) * ((size_t)n * f32_ld(n) + (size_t)n * nops);  // factors, work vector
    b += sizeof(int) * (size_t)n;  // pivots
    return (b + 15) & ~(size_t)15;
}

struct Warp32 {
    double *x, *r;
    float *F, *v;
    int *piv;
};

__device__ inline Warp32 carve32(char *base, int n, int k, int nops) {
    Warp32 w;
    size_t off = (warp_smem_bytes(n, k, nops) + 15) & ~(size_t)15;
    w.x = reinterpret_cast<double *>(base + off);
    w.r = w.x + (size_t)n * nops;
    w.F = reinterpret_cast<float *>(w.r + (size_t)n * nops);
    w.v = w.F + (size_t)n * f32_ld(n);
    w.piv = reinterpret_cast<int *>(w.v + (size_t)n * nops);
    return w;
}

// LU with partial pivoting of F (n x n, FP32), swaps applied to whole rows; piv[c] is the
// row exchanged with c at step c.
__device__ bool lu_factor_fp32(float *F, int *piv, int n, int lane) {
    const int ld = f32_ld(n);
    for (int c = 0; c < n; c++) {
        float bv = -1.0f;
        int br = n;
        for (int r = c + lane; r < n; r += 32) {
            float v = fabsf(F[r * ld + c]);
            if (v > bv) {
                bv = v;
                br = r;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            int orr = __shfl_xor_sync(0xffffffffu, br, o);
            if (ov > bv || (ov == bv && orr < br)) {
                bv = ov;
                br = orr;
            }
        }
        if (!(bv > 0.0f) || !isfinite(bv)) return false;
        if (lane == 0) piv[c] = br;
        if (br != c)
            for (int cc = lane; cc < n; cc += 32) {
                float a = F[c * ld + cc];
                F[c * ld + cc] = F[br * ld + cc];
                F[br * ld + cc] = a;
            }
        __syncwarp();
        const float inv = 1.0f / F[c * ld + c];
        for (int r = c + 1 + lane; r < n; r += 32) F[r * ld + c] *= inv;
        __syncwarp();
        const int rows = n - c - 1, cols = n - c - 1;
        if (rows > 0) {
            const int total = rows * cols;
            int r = lane / cols, cc = lane % cols;
            const int dr = 32 / cols, dc = 32 % cols;
            const float *prow = F + c * ld + c + 1;
            for (int t = lane; t < total; t += 32) {
                float *row = F + (c + 1 + r) * ld;
                row[c + 1 + cc] = fmaf(-row[c], prow[cc], row[c + 1 + cc]);
                r += dr;
                cc += dc;
                if (cc >= cols) {
                    cc -= cols;
                    r++;
                }
            }
        }
        __syncwarp();
    }
    return true;
}

// v (n x nops, FP32) := A32^{-1} v using the factors
__device__ void lu_apply_fp32(const float *F, const int *piv, float *v, int n, int nops, int lane) {
    const int ld = f32_ld(n);
    if (lane < nops)
        for (int c = 0; c < n; c++) {
            int p = piv[c];
            if (p != c) {
                float a = v[c * nops + lane];
                v[c * nops + lane] = v[p * nops + lane];
                v[p * nops + lane] = a;
            }
        }
    __syncwarp();
    for (int c = 0; c < n - 1; c++) {
        const int total = (n - c - 1) * nops;
        for (int t = lane; t < total; t += 32) {
            int r = c + 1 + t / nops, q = t % nops;
            v[r * nops + q] = fmaf(-F[r * ld + c], v[c * nops + q], v[r * nops + q]);
        }
        __syncwarp();
    }
    for (int c = n - 1; c >= 0; c--) {
        if (lane < nops) v[c * nops + lane] = v[c * nops + lane] / F[c * ld + c];
        __syncwarp();
        const int total = c * nops;
        for (int t = lane; t < total; t += 32) {
            int r = t / nops, q = t % nops;
            v[r * nops + q] = fmaf(-F[r * ld + c], v[c * nops + q], v[r * nops + q]);
        }
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
        assemble_fp64(P, w, lane, es, eval_local);
        // round the matrix to FP32
        for (int t = lane; t < n * n; t += 32) {
            int i = t / n, j = t - (t / n) * n;
            u.F[i * fld + j] = (float)w.M[i * ld + j];
        }
        __syncwarp();
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
                u.v[t] = (float)w.M[i * ld + n + q];
                u.x[t] = 0.0;
            }
            __syncwarp();
            double dprev = 0.0;
            for (int step = 0;; step++) {
                lu_apply_fp32(u.F, u.piv, u.v, n, nops, lane);
                double dmax = 0.0, xmax = 0.0;
                for (int t = lane; t < n * nops; t += 32) {
                    double d = (double)u.v[t];
                    u.x[t] += d;
                    if (t / nops < P.k) {
                        dmax = fmax(dmax, fabs(d));
                        xmax = fmax(xmax, fabs(u.x[t]));
                    }
                }
                for (int o = 16; o > 0; o >>= 1) {
                    dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
                    xmax = fmax(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
                }
                __syncwarp();
                // accept when the correction is below tol and shrinking (contraction < 1/2),
                // so that the error left after adding it is below tol as well
                if (step > 0 && dmax <= P.tol * xmax && dmax <= 0.5 * dprev) {
                    accepted = true;
                    est_final = xmax > 0 ? dmax / xmax : 0.0;
                    break;
                }
                dprev = dmax;
                if (step >= P.refine_steps || !isfinite(dmax)) break;
                // FP64 residual r = b - A x (A symmetric: read column i as row i); rows k..n-1
                // are the polynomial-reproduction constraints P^T w = L(p)
                for (int i = lane; i < n; i += 32) {
                    for (int q = 0; q < nops; q++) {
                        double acc = w.M[i * ld + n + q];
                        for (int j = 0; j < n; j++) acc = fma(-w.M[j * ld + i], u.x[j * nops + q], acc);
                        u.v[i * nops + q] = (float)acc;
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
            // fallback: the plain FP64 solve on the intact FP64 system
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
