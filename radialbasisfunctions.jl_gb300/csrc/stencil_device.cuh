// Device building blocks of the weight-build kernels, shared by stencil_build.cu and the
// register-resident refined kernels (stencil_refined_*.cu).
#pragma once
#include <algorithm>
#include <cmath>

#include "rbf_internal.cuh"
#include "stencil_common.cuh"

namespace {

// Per-warp staging of one stencil.  ptype: the points' Hermite types; in a normal-derivative
// build (RBF_FLAG_NORMAL_DOF) ptype[a] is instead the stencil position of du/dn unknown a and
// HN[3a..3a+2] its normal.
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
//  0: solve needed, 2: Dirichlet identity row written, -1: eval point not in stencil,
//  1: the stencil's du/dn unknowns differ from its size class's (normal-derivative builds).
// *eval_local_out: -2 interior stencil (plain collocation), -3 stencil with du/dn unknowns,
// else the reference's Hermite stencil (the eval point's stencil position, -1 if absent).
__device__ int load_stencil(const StencilParams &P, int64_t e, const WarpSmem &w, int lane, int *es_out,
                            int *eval_local_out) {
    const int k = P.k, dim = P.dim;
    double x0[3] = {0, 0, 0};
    for (int d = 0; d < dim; d++) x0[d] = P.eval[e * dim + d];
    double r2max = 0.0;
    bool anyb = false;
    const int32_t *nbr = P.adj_ptr ? P.adjl + P.adj_ptr[e] : P.adjl + e * k;
    for (int i = lane; i < k; i += 32) {
        int g = nbr[i];
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
    // r2max >= 0: its bit pattern orders like its value (an integer max, off the FP64 pipe)
    {
        long long m = __double_as_longlong(r2max);
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        r2max = __longlong_as_double(m);
    }
    anyb = __any_sync(0xffffffffu, anyb);
    int es = 0;
    if (r2max > 0.0) es = sqrt_frexp_exponent(r2max);
    *es_out = es;
    __syncwarp();
    for (int i = lane; i < k; i += 32)
        for (int d = 0; d < dim; d++) w.X[i * 3 + d] = scale2(w.X[i * 3 + d], -es);
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
                    if (P.sell_col)
                        for (int r = 0; r < P.nops; r++) sell_put(P, e, 0, (int32_t)e, r, 1.0);
                    if (P.status) P.status[e] = 2;
                    atomicAdd(&P.counters[3], 1ull);
                }
                return 2;
            }
        }
        if (P.flags & RBF_FLAG_NORMAL_DOF) {
            // every point is a value point; the Neumann/Robin ones also carry du/dn, numbered
            // in stencil order (the Dirichlet ones are plain value points)
            int m = 0;
            for (int i0 = 0; i0 < k; i0 += 32) {
                const int i = i0 + lane;
                bool nr = false;
                int32_t b = 0;
                if (i < k && P.isb[w.cols[i]]) {
                    b = P.g2b[w.cols[i]];
                    nr = !(P.alpha[b] == 1.0 && P.beta[b] == 0.0);
                }
                const unsigned bal = __ballot_sync(0xffffffffu, nr);
                const int a = m + __popc(bal & ((1u << lane) - 1u));
                if (nr && a < P.nnr) {
                    w.ptype[a] = i;
                    for (int d = 0; d < 3; d++) w.HN[a * 3 + d] = d < dim ? P.normals[(int64_t)b * dim + d] : 0.0;
                }
                m += __popc(bal);
            }
            if (m != P.nnr) {
                if (lane == 0) {
                    if (P.status) P.status[e] = 1;
                    atomicAdd(&P.counters[0], 1ull);
                }
                return 1;
            }
            *eval_local_out = m > 0 ? -3 : -2;
            __syncwarp();
            return 0;
        }
        const double sinv = scale2(1.0, -es);
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

// Storage policies of the FP64 assembly.  FullStore: M[n][ld] holding both triangles and the
// right-hand sides in columns n.. (the LU solves).  PackedStore: the lower triangle packed by
// rows (entry (i, j), i >= j, at i (i + 1) / 2 + j) and the right-hand sides in B[n][nops]
// (the symmetric indefinite solve).
struct FullStore {
    static constexpr bool kPacked = false;
    double *M;
    int n, ld;
    __device__ void zero(int lane) const {
        for (int t = lane; t < n * ld; t += 32) M[t] = 0.0;
    }
    __device__ void sym(int i, int j, double v) const {
        M[i * ld + j] = v;
        M[j * ld + i] = v;
    }
    __device__ void rhs(int i, int r, double v) const { M[i * ld + n + r] = v; }
};

__host__ __device__ __forceinline__ int pidx(int i, int j) { return ((i * (i + 1)) >> 1) + j; }  // i >= j

struct PackedStore {
    static constexpr bool kPacked = true;
    double *P, *B;
    int n, k, nops;
    __device__ void zero(int lane) const {  // the zero block (rows and columns k..n-1)
        const int m = n - k;
        for (int t = lane; t < m * m; t += 32) {
            const int a = t / m, b = t - (t / m) * m;
            if (b <= a) P[pidx(k + a, k + b)] = 0.0;
        }
    }
    __device__ void sym(int i, int j, double v) const { P[i >= j ? pidx(i, j) : pidx(j, i)] = v; }
    __device__ void rhs(int i, int r, double v) const { B[i * nops + r] = v; }
};

// The du/dn unknowns of a normal-derivative stencil (RBF_FLAG_NORMAL_DOF).  Only the
// normal-derivative instantiations of the assembly (ND = true) include it, so the kernels of
// the other builds keep their register budget.
template <class S>
__device__ __forceinline__ void assemble_normal_dof(const StencilParams &P, const WarpSmem &w, int lane, int es,
                                                 const S &st) {
    const int k = P.k, nops = P.nops, dim = P.dim, nmon = P.nmon;
    const int kv = k + P.nnr;
    const AvoidInf<double> AI = avoid_inf_scaled<double>(es);
    // du/dn unknowns a, b (stencil positions ptype[a], normals n_a): the functionals
    // u(x_i) and du/dn(x_a) applied to the kernel, in local units --
    //   value row i, column k + a:  -n_a . grad phi(x_i - x_a)
    //   rows/columns k + a, k + b:  -n_a^T Hess phi(x_a - x_b) n_b
    //   polynomial columns:          n_a . grad p(x_a)
    //   right-hand sides:            L applied to -n_a . grad phi(x - x_a) at the eval point
    const int m = P.nnr;
    const int nvd = k * m, ndd = m * (m + 1) / 2;
    for (int t = lane; t < nvd + ndd; t += 32) {
        int i, a;
        const bool dd = t >= nvd;
        if (!dd) {
            i = t / m;
            a = t - i * m;
        } else {
            const int p = t - nvd;  // pair (i, a), i >= a, in row order
            i = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
            while (i * (i + 1) / 2 > p) i--;
            while ((i + 1) * (i + 2) / 2 <= p) i++;
            a = p - i * (i + 1) / 2;
        }
        const double *xi = dd ? &w.X[w.ptype[i] * 3] : &w.X[i * 3];
        const double *xa = &w.X[w.ptype[a] * 3];
        const double *na = &w.HN[a * 3];
        double D[3], g[3], H[9];
        for (int d = 0; d < dim; d++) D[d] = xi[d] - xa[d];
        phs_grad_hess<double>(P.phs, D, dim, g, H, dd, AI);
        double v = 0.0;
        if (!dd) {
            for (int d = 0; d < dim; d++) v = fma(-na[d], g[d], v);
            st.sym(i, k + a, v);
        } else {
            const double *ni = &w.HN[i * 3];
            for (int c = 0; c < dim; c++) {
                double hn = 0.0;
                for (int d = 0; d < dim; d++) hn = fma(H[c * 3 + d], na[d], hn);
                v = fma(-ni[c], hn, v);
            }
            st.sym(k + i, k + a, v);
        }
    }
    for (int a = lane; a < m; a += 32) {
        const double *xa = &w.X[w.ptype[a] * 3];
        const double *na = &w.HN[a * 3];
        for (int mm = 0; mm < nmon; mm++) {
            double dn = 0.0;
            for (int d = 0; d < dim; d++) dn = fma(na[d], mono_d1<double>(P, mm, d, xa), dn);
            st.sym(k + a, kv + mm, dn);
        }
        double D[3];
        for (int d = 0; d < dim; d++) D[d] = -xa[d];
        for (int r = 0; r < nops; r++)
            st.rhs(k + a, r, phs_op_normal<double>(P.phs, P.op_code[r], P.op_dim[r], D, na, dim, AI));
    }
}

// Assemble [Phi P; P^T 0 | B] into the storage S (ND: the instantiation of the
// normal-derivative builds, which also assembles their du/dn unknowns).
template <class S, bool ND = false>
__device__ void assemble_fp64_into(const StencilParams &P, const WarpSmem &w, int lane, int es, int eval_local,
                                   const S &st) {
    const int k = P.k, nops = P.nops, dim = P.dim, nmon = P.nmon;
    const bool aug = eval_local == -3;           // du/dn unknowns: plain value-value block
    const bool herm = eval_local != -2 && !aug;  // the reference's Hermite stencil
    const int kv = aug ? k + P.nnr : k;          // unknowns before the polynomial multipliers
    const AvoidInf<double> AI = avoid_inf_scaled<double>(es);
    st.zero(lane);
    __syncwarp();
    if (S::kPacked && !herm) {
        // interior stencil, packed storage: phi(0) = 0 on the diagonal, the strict upper
        // triangle's pairs (i < j) with the Newton square root
        for (int i = lane; i < k; i += 32) st.sym(i, i, 0.0);
        const int nstrict = k * (k - 1) / 2;
        for (int p = lane; p < nstrict; p += 32) {
            int j = (int)((sqrtf(8.0f * (float)p + 1.0f) + 1.0f) * 0.5f);
            while (j * (j - 1) / 2 > p) j--;
            while ((j + 1) * j / 2 <= p) j++;
            const int i = p - j * (j - 1) / 2;
            // components held in registers (dimensions past dim contribute nothing)
            const double d0 = w.X[i * 3] - w.X[j * 3];
            const double d1 = dim > 1 ? w.X[i * 3 + 1] - w.X[j * 3 + 1] : 0.0;
            const double d2 = dim > 2 ? w.X[i * 3 + 2] - w.X[j * 3 + 2] : 0.0;
            const double r2 = dim == 1 ? d0 * d0 : (dim == 2 ? fma(d1, d1, d0 * d0) : fma(d2, d2, fma(d1, d1, d0 * d0)));
            const double r = sqrt_newton(r2);
            double v;
            switch (P.phs) {
            case 1: v = r; break;
            case 3: v = r2 * r; break;
            case 5: v = (r2 * r2) * r; break;
            default: v = (r2 * r2 * r2) * r; break;
            }
            st.sym(i, j, v);
        }
    }
    // RBF block, upper triangle pairs (i <= j) mirrored
    const int npairs = (S::kPacked && !herm) ? 0 : k * (k + 1) / 2;
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
        st.sym(i, j, v);
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
            st.sym(i, kv + m, v);
        }
        double D[3];
        for (int d = 0; d < dim; d++) D[d] = -xi[d];  // x0 - xi in local coordinates
        for (int r = 0; r < nops; r++) {
            double b = phs_op<double>(P.phs, P.op_code[r], P.op_dim[r], D, dim, AI);
            if (nr)
                b = w.HA[i] * b +
                    w.HB[i] * phs_op_normal<double>(P.phs, P.op_code[r], P.op_dim[r], D, &w.HN[i * 3], dim, AI);
            st.rhs(i, r, b);
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
            v = scale2(v, es * P.op_order[r]);
        } else {
            v = mono_op_at_origin(P, m, P.op_code[r], P.op_dim[r]);
        }
        st.rhs(kv + m, r, v);
    }
    if constexpr (ND)
        if (aug) assemble_normal_dof(P, w, lane, es, st);
    __syncwarp();
}

// Assemble [Phi P; P^T 0 | B] into M (full symmetric storage).
template <bool ND = false>
__device__ void assemble_fp64(const StencilParams &P, const WarpSmem &w, int lane, int es, int eval_local) {
    assemble_fp64_into<FullStore, ND>(P, w, lane, es, eval_local, FullStore{w.M, P.n, mat_ld(P.n, P.nops)});
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
    const int k = P.k, m = P.nnr;
    const int64_t base = P.row_ptr[e];
    const bool sorted = !(P.flags & RBF_FLAG_STENCIL_ORDER);
    const bool local = (P.flags & RBF_FLAG_LOCAL_UNITS) != 0;
    // du/dn unknowns (normal-derivative builds): columns ns + boundary ordinal after the value
    // columns; their weights scale by s^(1 - q) (one derivative in the unknown)
    for (int a = lane; a < m; a += 32) {
        const int32_t ca = (int32_t)P.ns + P.g2b[w.cols[w.ptype[a]]];
        int rank = k + a;
        if (sorted) {
            rank = k;
            for (int b = 0; b < m; b++) {
                const int32_t cb = (int32_t)P.ns + P.g2b[w.cols[w.ptype[b]]];
                rank += (cb < ca) || (cb == ca && b < a);
            }
        }
        P.col[base + rank] = ca;
        for (int r = 0; r < P.nops; r++) {
            const double v = sol[(k + a) * sol_ld + r * sol_stride];
            const double vo = local ? v : scale2(v, es * (1 - P.op_order[r]));
            P.val[r * P.nnz + base + rank] = vo;
            if (P.sell_col) sell_put(P, e, rank, ca, r, vo);
        }
    }
    for (int i = lane; i < k; i += 32) {
        const int ci = w.cols[i];
        int rank = i;
        if (sorted) {
            rank = 0;
            for (int j = 0; j < k; j++) {
                int cj = w.cols[j];
                rank += (cj < ci) || (cj == ci && j < i);
            }
        }
        P.col[base + rank] = ci;
        for (int r = 0; r < P.nops; r++) {
            const double v = sol[i * sol_ld + r * sol_stride];
            const double vo = local ? v : scale2(v, -es * P.op_order[r]);
            P.val[r * P.nnz + base + rank] = vo;
            if (P.sell_col) sell_put(P, e, rank, ci, r, vo);
        }
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
    b += sizeof(float) * 6 * (size_t)k;  // local coordinates split into float hi + lo
    b += sizeof(int) * (size_t)n;  // pivots
    return (b + 15) & ~(size_t)15;
}

struct Warp32 {
    double *x, *r;
    float *F, *v, *XH, *XL;
    int *piv;
};

__device__ inline Warp32 carve32(char *base, int n, int k, int nops) {
    Warp32 w;
    size_t off = (warp_smem_bytes(n, k, nops) + 15) & ~(size_t)15;
    w.x = reinterpret_cast<double *>(base + off);
    w.r = w.x + (size_t)n * nops;
    w.F = reinterpret_cast<float *>(w.r + (size_t)n * nops);
    w.v = w.F + (size_t)n * f32_ld(n);
    w.XH = w.v + (size_t)n * nops;
    w.XL = w.XH + 3 * (size_t)k;
    w.piv = reinterpret_cast<int *>(w.XL + 3 * (size_t)k);
    return w;
}

// ---- double-float arithmetic on the FP32 pipe (value = hi + lo, ~44 significant bits) ----
struct dfl {
    float hi, lo;
};
__device__ __forceinline__ dfl qts(float a, float b) {  // |a| >= |b|
    float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ dfl ts(float a, float b) {
    float s = a + b;
    float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    dfl s = ts(a.hi, b.hi);
    return qts(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return qts(p, e);
}
__device__ __forceinline__ dfl df_sqr(dfl a) {
    float p = a.hi * a.hi;
    float e = fmaf(a.hi, a.hi, -p);
    e = fmaf(2.0f * a.hi, a.lo, e);
    return qts(p, e);
}
// Heron/Newton from the hardware reciprocal square root: one FP32 step brings s to about
// one ulp of sqrt(hi), the double-float step to ~2^-46 relative; 1/(2s) enters only the
// correction terms, where the approximate reciprocal's error is second order.
__device__ __forceinline__ dfl df_sqrt(dfl a) {
    const float rs = rsqrtf(a.hi);
    const float h = 0.5f * rs;
    float s = a.hi * rs;
    s = fmaf(fmaf(-s, s, a.hi), h, s);
    const float e = fmaf(-s, s, a.hi) + a.lo;
    const dfl r = qts(s, e * h);
    return a.hi > 0.0f ? r : dfl{0.0f, 0.0f};
}
__device__ __forceinline__ double df_to_double(dfl a) { return widen(a.hi) + widen(a.lo); }

// Interior stencils: Phi and P in double-float.  M gets the FP64 system (hi + lo, for the
// residual and the fallback), F the FP32 factor matrix (hi).  Right-hand sides in FP64.
// Hermite stencils (a small minority) take the FP64 assembly and are rounded to F.
template <bool ND = false>
__device__ void assemble_refined(const StencilParams &P, const WarpSmem &w, const Warp32 &u, int lane, int es,
                                 int eval_local) {
    // u.F == nullptr: only the FP64 system is needed (the register kernels narrow it)
    const int k = P.k, n = P.n, nops = P.nops, ld = mat_ld(n, nops), fld = f32_ld(n), dim = P.dim, nmon = P.nmon;
    if (eval_local != -2) {  // Hermite stencil
        assemble_fp64<ND>(P, w, lane, es, eval_local);
        if (u.F) {
            for (int t = lane; t < n * n; t += 32) {
                int i = t / n, j = t - (t / n) * n;
                u.F[i * fld + j] = __double2float_rn(w.M[i * ld + j]);
            }
            __syncwarp();
        }
        return;
    }
    for (int i = lane; i < k; i += 32)
        for (int d = 0; d < 3; d++) {
            double xv = d < dim ? w.X[i * 3 + d] : 0.0;
            float hi = d2f_rn_bits(xv);
            u.XH[i * 3 + d] = hi;
            u.XL[i * 3 + d] = d2f_rn_bits(xv - widen(hi));
        }
    for (int t = lane; t < nmon * ld; t += 32) w.M[(k + t / ld) * ld + t % ld] = 0.0;  // zero block rows
    if (u.F)
        for (int t = lane; t < nmon * nmon; t += 32) u.F[(k + t / nmon) * fld + k + t % nmon] = 0.0f;
    __syncwarp();
    const int npairs = k * (k + 1) / 2;
    for (int p = lane; p < npairs; p += 32) {
        int j = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
        while (j * (j + 1) / 2 > p) j--;
        while ((j + 1) * (j + 2) / 2 <= p) j++;
        const int i = p - j * (j + 1) / 2;
        dfl r2 = {0.0f, 0.0f};
        for (int d = 0; d < dim; d++) {
            dfl dd = ts(u.XH[i * 3 + d], -u.XH[j * 3 + d]);
            dd = qts(dd.hi, dd.lo + (u.XL[i * 3 + d] - u.XL[j * 3 + d]));
            r2 = df_add(r2, df_sqr(dd));
        }
        const dfl r = df_sqrt(r2);
        dfl phi;
        switch (P.phs) {
        case 1: phi = r; break;
        case 3: phi = df_mul(r2, r); break;
        case 5: phi = df_mul(df_sqr(r2), r); break;
        default: phi = df_mul(df_mul(df_sqr(r2), r2), r); break;
        }
        const double v = df_to_double(phi);
        w.M[i * ld + j] = v;
        w.M[j * ld + i] = v;
        if (u.F) {
            u.F[i * fld + j] = phi.hi;
            u.F[j * fld + i] = phi.hi;
        }
    }
    const AvoidInf<double> AI = avoid_inf_scaled<double>(es);
    for (int i = lane; i < k; i += 32) {
        dfl xd[3];
        for (int d = 0; d < 3; d++) xd[d] = {u.XH[i * 3 + d], u.XL[i * 3 + d]};
        for (int m = 0; m < nmon; m++) {
            dfl v = {1.0f, 0.0f};
            for (int d = 0; d < dim; d++)
                for (int t = 0; t < P.exps[m][d]; t++) v = df_mul(v, xd[d]);
            const double vd = df_to_double(v);
            w.M[i * ld + k + m] = vd;
            w.M[(k + m) * ld + i] = vd;
            if (u.F) {
                u.F[i * fld + k + m] = v.hi;
                u.F[(k + m) * fld + i] = v.hi;
            }
        }
        double D[3];
        for (int d = 0; d < dim; d++) D[d] = -w.X[i * 3 + d];
        for (int r = 0; r < nops; r++) w.M[i * ld + n + r] = phs_op<double>(P.phs, P.op_code[r], P.op_dim[r], D, dim, AI);
    }
    for (int t = lane; t < nmon * nops; t += 32) {
        int m = t / nops, r = t % nops;
        w.M[(k + m) * ld + n + r] = mono_op_at_origin(P, m, P.op_code[r], P.op_dim[r]);
    }
    __syncwarp();
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

// ---- block-cooperative factorisations (block-per-stencil tiles of the batched build) ----
// The whole thread block (G threads, G a multiple of 32, every thread calling) factorises
// one system in shared memory.  Each matrix entry receives the same FMA sequence and the
// pivot is the same (largest magnitude, lowest row on ties) as in the one-warp versions
// above, so the results are bit-identical to them.  redv/redi: G/32 scratch slots.
template <class T>
__device__ __forceinline__ void block_argmax(T &bv, int &br, T *redv, int *redi, int tid, int G) {
    for (int o = 16; o > 0; o >>= 1) {
        const T ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int orr = __shfl_xor_sync(0xffffffffu, br, o);
        if (ov > bv || (ov == bv && orr < br)) {
            bv = ov;
            br = orr;
        }
    }
    if ((tid & 31) == 0) {
        redv[tid >> 5] = bv;
        redi[tid >> 5] = br;
    }
    __syncthreads();
    bv = redv[0];
    br = redi[0];
    for (int w = 1; w < G / 32; w++)
        if (redv[w] > bv || (redv[w] == bv && redi[w] < br)) {
            bv = redv[w];
            br = redi[w];
        }
}

__device__ bool lu_solve_fp64_block(double *M, int n, int nops, int tid, int G, double *redv, int *redi) {
    const int ld = mat_ld(n, nops), W = n + nops;
    for (int c = 0; c < n; c++) {
        double bv = -1.0;
        int br = n;
        for (int r = c + tid; r < n; r += G) {
            const double v = fabs(M[r * ld + c]);
            if (v > bv) {
                bv = v;
                br = r;
            }
        }
        block_argmax(bv, br, redv, redi, tid, G);
        if (!(bv > 0.0) || !isfinite(bv)) {
            __syncthreads();
            return false;
        }
        if (br != c)
            for (int cc = c + tid; cc < W; cc += G) {
                const double a = M[c * ld + cc];
                M[c * ld + cc] = M[br * ld + cc];
                M[br * ld + cc] = a;
            }
        __syncthreads();
        const double inv = 1.0 / M[c * ld + c];
        for (int r = c + 1 + tid; r < n; r += G) M[r * ld + c] *= inv;
        __syncthreads();
        const int rows = n - c - 1, cols = W - c - 1;
        if (rows > 0) {
            const int total = rows * cols;
            int r = tid / cols, cc = tid % cols;
            const int dr = G / cols, dc = G % cols;
            const double *prow = M + c * ld + c + 1;
            for (int t = tid; t < total; t += G) {
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
        __syncthreads();
    }
    for (int c = n - 1; c >= 0; c--) {
        if (tid < nops) M[c * ld + n + tid] = M[c * ld + n + tid] / M[c * ld + c];
        __syncthreads();
        const int total = c * nops;
        for (int t = tid; t < total; t += G) {
            const int r = t / nops, q = t - (t / nops) * nops;
            M[r * ld + n + q] = fma(-M[r * ld + c], M[c * ld + n + q], M[r * ld + n + q]);
        }
        __syncthreads();
    }
    return true;
}

__device__ bool lu_factor_fp32_block(float *F, int *piv, int n, int tid, int G, float *redv, int *redi) {
    const int ld = f32_ld(n);
    for (int c = 0; c < n; c++) {
        float bv = -1.0f;
        int br = n;
        for (int r = c + tid; r < n; r += G) {
            const float v = fabsf(F[r * ld + c]);
            if (v > bv) {
                bv = v;
                br = r;
            }
        }
        block_argmax(bv, br, redv, redi, tid, G);
        if (!(bv > 0.0f) || !isfinite(bv)) {
            __syncthreads();
            return false;
        }
        if (tid == 0) piv[c] = br;
        if (br != c)
            for (int cc = tid; cc < n; cc += G) {
                const float a = F[c * ld + cc];
                F[c * ld + cc] = F[br * ld + cc];
                F[br * ld + cc] = a;
            }
        __syncthreads();
        const float inv = 1.0f / F[c * ld + c];
        for (int r = c + 1 + tid; r < n; r += G) F[r * ld + c] *= inv;
        __syncthreads();
        const int rows = n - c - 1, cols = n - c - 1;
        if (rows > 0) {
            const int total = rows * cols;
            int r = tid / cols, cc = tid % cols;
            const int dr = G / cols, dc = G % cols;
            const float *prow = F + c * ld + c + 1;
            for (int t = tid; t < total; t += G) {
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
        __syncthreads();
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

}  // namespace
