/*
 * CPU oracle for the local RBF-FD weight build of RadialBasisFunctions.jl (v0.7.0).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU library is
 * compared against; it is never linked into, loaded by or called from the
 * product path.  Only tests/, __graft_entry__.smoke() and bench.py (its CPU
 * baseline leg and `--impl reference`) load it.
 *
 * It restates, in plain C, the reference's arithmetic for the hot path:
 *   - k-nearest-neighbour stencils           src/utils.jl:12-18 (KDTree + knn(sorted=true))
 *   - PHS basis functions and their operator
 *     forms, incl. Hermite 3-argument forms  src/basis/polyharmonic_spline.jl:43-376
 *   - monomial augmentation and its
 *     operator forms                         src/basis/monomial.jl:17-123,
 *                                            src/operators/monomial/monomial.jl:200-269,
 *                                            src/operators/monomial/partial.jl:377-402
 *   - collocation matrix (upper triangle)    src/solve/assembly.jl:95-115
 *   - right-hand side (one or many ops)      src/solve/assembly.jl:127-185
 *   - Hermite entry rules                    src/solve/assembly.jl:240-468, src/solve/types.jl:133-258
 *   - rook-pivoted Bunch-Kaufman solve       src/solve/assembly.jl:220-222 (LAPACK dsytrf_rook /
 *                                            dsytrs_rook, UPLO='U', restated from the published
 *                                            LAPACK 3.x algorithm, unblocked form dsytf2_rook,
 *                                            which is the path LAPACK takes for n < 64)
 *   - exact nnz count, Dirichlet identity
 *     rows, COO -> sorted sparse rows        src/solve/execution.jl:39-115,279-303
 *   - apply y = alpha*W*x + beta*y           src/operators/operators.jl:217-218,529-542
 *
 * Compile with -ffp-contract=off: Julia does not contract a*b+c into FMA, so
 * neither does the oracle.  Distances are accumulated in dimension order
 * (((0 + dx^2) + dy^2) + dz^2), as Distances.jl's reduction does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define AVOID_INF 1.0e-16 /* avoid_inf(Float64), src/RadialBasisFunctions.jl:111 */
/* The guards of r^b denominators (r^b + avoid_inf).  They are avoid_inf itself in the
 * reference's (raw) coordinates; the local-frame build (orc_build_local) sets them to
 * avoid_inf / s^b per stencil, so that every entry of the local system is exactly s^p times
 * the raw entry, the guards included. */
static _Thread_local double orc_ai1 = AVOID_INF, orc_ai2 = AVOID_INF, orc_ai3 = AVOID_INF, orc_ai5 = AVOID_INF;
#define AI_R1 orc_ai1
#define AI_R2 orc_ai2
#define AI_R3 orc_ai3
#define AI_R5 orc_ai5
#define MAXDIM 3
#define MAXN 160

enum { OP_IDENT = 0, OP_D1 = 1, OP_D2 = 2, OP_LAP = 3 };

/* ------------------------------------------------------------------------ */
/* distances                                                                  */
/* ------------------------------------------------------------------------ */
static inline double sqeuc(const double *a, const double *b, int dim) {
    double s = 0.0;
    for (int d = 0; d < dim; d++) {
        double t = a[d] - b[d];
        s = s + t * t;
    }
    return s;
}

/* ------------------------------------------------------------------------ */
/* PHS basis: value, operator forms (2-arg), normal forms (3-arg), grad, Hess */
/* polyharmonic_spline.jl: PHS1 43-119, PHS3 128-205, PHS5 214-290, PHS7 299-376 */
/* ------------------------------------------------------------------------ */
static inline double pw3(double r) { return r * r * r; }
static inline double pw5(double r) { return r * r * r * r * r; }

double orc_phs_phi(int p, const double *x, const double *y, int dim) {
    double r2 = sqeuc(x, y, dim);
    switch (p) {
    case 1: return sqrt(r2);
    case 3: return r2 * sqrt(r2);
    case 5: return (r2 * r2) * sqrt(r2);
    default: return (r2 * r2 * r2) * sqrt(r2);
    }
}

/* operator applied to phi in its first argument: (op::L)(x, xi) */
double orc_phs_op(int p, int op, int odim, const double *x, const double *xi, int dim) {
    if (op == OP_IDENT) return orc_phs_phi(p, x, xi, dim);
    double r2 = sqeuc(x, xi, dim);
    double r = sqrt(r2);
    double dd = x[odim] - xi[odim];
    switch (p) {
    case 1:
        if (op == OP_D1) return dd / (r + AI_R1);
        if (op == OP_D2) return (-(dd * dd) + r2) / (pw3(r) + AI_R3);
        return 2.0 / (r + AI_R1);
    case 3:
        if (op == OP_D1) return 3.0 * dd * r;
        if (op == OP_D2) return 3.0 * (r + (dd * dd) / (r + AI_R1));
        return 12.0 * r;
    case 5:
        if (op == OP_D1) return 5.0 * dd * pw3(r);
        if (op == OP_D2) return 5.0 * r * (3.0 * (dd * dd) + r2);
        return 30.0 * pw3(r);
    default:
        if (op == OP_D1) return 7.0 * dd * pw5(r);
        if (op == OP_D2) return 7.0 * pw3(r) * (5.0 * (dd * dd) + r2);
        return 56.0 * pw5(r);
    }
}

/* normal form (op::L)(x, xi, normal): the operator applied to the normal derivative of
 * phi in its second argument.  Returns NAN for the identity (no normal form exists,
 * which the reference rejects with an ArgumentError, src/solve/api.jl:79-94). */
double orc_phs_op_normal(int p, int op, int odim, const double *x, const double *xi,
                         const double *n, int dim) {
    if (op == OP_IDENT) return NAN;
    double r2 = sqeuc(x, xi, dim);
    double r = sqrt(r2);
    double dd = x[odim] - xi[odim];
    double nd = n[odim];
    double dn = 0.0;
    for (int d = 0; d < dim; d++) dn = dn + n[d] * (x[d] - xi[d]);
    switch (p) {
    case 1:
        if (op == OP_D1) return -nd / (r + AI_R1) + dn * dd / (pw3(r) + AI_R3);
        if (op == OP_D2)
            return (2.0 * nd * dd + dn) / (pw3(r) + AI_R3) -
                   3.0 * (dd * dd) * dn / (pw5(r) + AI_R5);
        return 2.0 * dn / (pw3(r) + AI_R3);
    case 3:
        if (op == OP_D1) return -3.0 * (nd * r + dn * dd / (r + AI_R1));
        if (op == OP_D2)
            return -3.0 * (2.0 * dd * nd + dn - dn * (dd * dd) / (r2 + AI_R2)) /
                   (r + AI_R1);
        return -12.0 * dn / (r + AI_R1);
    case 5:
        if (op == OP_D1) return -5.0 * (nd * pw3(r) + 3.0 * dn * dd * r);
        if (op == OP_D2)
            return -5.0 * (6.0 * nd * dd * r + 3.0 * dn * (r + (dd * dd) / (r + AI_R1)));
        return -90.0 * dn * r;
    default:
        if (op == OP_D1) return -7.0 * (nd * pw5(r) + 5.0 * pw3(r) * dd * dn);
        if (op == OP_D2)
            return -7.0 * (10.0 * nd * dd * pw3(r) + 5.0 * dn * (3.0 * r * (dd * dd) + pw3(r)));
        return -280.0 * dn * pw3(r);
    }
}

/* gradient of phi w.r.t. its first argument, (op::∇)(x, xi) */
void orc_phs_grad(int p, const double *x, const double *xi, int dim, double *g) {
    double r = sqrt(sqeuc(x, xi, dim));
    for (int d = 0; d < dim; d++) {
        double dd = x[d] - xi[d];
        switch (p) {
        case 1: g[d] = dd / (r + AI_R1); break;
        case 3: g[d] = 3.0 * dd * r; break;
        case 5: g[d] = 5.0 * dd * pw3(r); break;
        default: g[d] = 7.0 * dd * pw5(r); break;
        }
    }
}

/* Hessian of phi w.r.t. its first argument, (op::H)(x, xi), row-major dim x dim */
void orc_phs_hess(int p, const double *x, const double *xi, int dim, double *h) {
    double r = sqrt(sqeuc(x, xi, dim));
    for (int i = 0; i < dim; i++)
        for (int j = 0; j < dim; j++) {
            double di = x[i] - xi[i], dj = x[j] - xi[j];
            double delta = (i == j) ? 1.0 : 0.0;
            double v;
            switch (p) {
            case 1: v = delta / (r + AI_R1) - di * dj / (pw3(r) + AI_R3); break;
            case 3: v = 3.0 * (delta * r + di * dj / (r + AI_R1)); break;
            case 5: v = 5.0 * (delta * pw3(r) + 3.0 * di * dj * r); break;
            default: v = 7.0 * (delta * pw5(r) + 5.0 * di * dj * pw3(r)); break;
            }
            h[i * dim + j] = v;
        }
}

/* ------------------------------------------------------------------------ */
/* monomial basis (ordering of src/basis/monomial.jl)                          */
/* ------------------------------------------------------------------------ */
static int binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    long r = 1;
    for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
    return (int)r;
}

/* All exponent vectors (e_1..e_dim, slack) summing to deg, in the order Combinatorics'
 * multiexponents(dim+1, deg) yields them: reverse lexicographic (largest e_1 first). */
static int multiexp_rec(int dim, int deg, int pos, int remaining, int *cur, int *out, int cnt) {
    if (pos == dim) {
        for (int d = 0; d < dim; d++) out[cnt * dim + d] = cur[d];
        return cnt + 1;
    }
    for (int e = remaining; e >= 0; e--) {
        if (pos == dim - 1 && e != remaining) break; /* the last entry takes what is left */
        cur[pos] = e;
        cnt = multiexp_rec(dim, deg, pos + 1, remaining - e, cur, out, cnt);
    }
    return cnt;
}

/* Fills exps[nmon*dim] with the reference's monomial order; returns nmon (0 if deg<0). */
int orc_monomial_exponents(int dim, int deg, int *exps) {
    if (deg < 0) return 0;
    int nmon = binom(dim + deg, dim);
    memset(exps, 0, sizeof(int) * nmon * dim);
    if (deg == 0) return 1; /* constant */
    if (dim == 1) {         /* [1, x, x^2, ...] monomial.jl:37-49 */
        for (int j = 0; j <= deg; j++) exps[j] = j;
        return nmon;
    }
    if (dim == 2 && deg == 1) { /* [1,x,y] monomial.jl:51-58 */
        int t[] = {0, 0, 1, 0, 0, 1};
        memcpy(exps, t, sizeof t);
        return nmon;
    }
    if (dim == 2 && deg == 2) { /* [1,x,y,xy,x2,y2] monomial.jl:60-70 */
        int t[] = {0, 0, 1, 0, 0, 1, 1, 1, 2, 0, 0, 2};
        memcpy(exps, t, sizeof t);
        return nmon;
    }
    if (dim == 3 && deg == 1) { /* [1,x,y,z] monomial.jl:72-80 */
        int t[] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
        memcpy(exps, t, sizeof t);
        return nmon;
    }
    if (dim == 3 && deg == 2) { /* [1,x,y,z,xy,xz,yz,x2,y2,z2] monomial.jl:82-96 */
        int t[] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 1, 1, 0,
                   1, 0, 1, 0, 1, 1, 2, 0, 0, 0, 2, 0, 0, 0, 2};
        memcpy(exps, t, sizeof t);
        return nmon;
    }
    int cur[8];
    /* generic: multiexponents(dim+1, deg); the last entry is the slack exponent */
    int *tmp = (int *)malloc(sizeof(int) * nmon * (dim + 1));
    int cnt = multiexp_rec(dim + 1, deg, 0, deg, cur, tmp, 0);
    for (int j = 0; j < cnt; j++)
        for (int d = 0; d < dim; d++) exps[j * dim + d] = tmp[j * (dim + 1) + d];
    free(tmp);
    return nmon;
}

/* product of x_d^(e_d), multiplied in dimension order starting from 1 (the order of the
 * reference's _monomial_products!, monomial.jl:106-114) */
static inline double mono_prod(const int *e, const double *x, int dim) {
    double v = 1.0;
    for (int d = 0; d < dim; d++)
        for (int t = 0; t < e[d]; t++) v *= x[d];
    return v;
}

/* value of operator `op` (dimension odim) applied to each monomial at x */
void orc_mono_op(int dim, int nmon, const int *exps, int op, int odim, const double *x, double *b) {
    for (int j = 0; j < nmon; j++) {
        const int *e = exps + j * dim;
        if (op == OP_IDENT) {
            b[j] = mono_prod(e, x, dim);
        } else if (op == OP_D1 || op == OP_D2) {
            int ee[MAXDIM];
            for (int d = 0; d < dim; d++) ee[d] = e[d];
            double c = 1.0;
            int order = (op == OP_D1) ? 1 : 2;
            for (int o = 0; o < order; o++) {
                if (ee[odim] == 0) c = 0.0;
                else { c *= ee[odim]; ee[odim] -= 1; }
            }
            b[j] = mono_prod(ee, x, dim) * c;
        } else { /* Laplacian: sum of second partials in dimension order, monomial.jl:218-230 */
            double s = 0.0;
            for (int d = 0; d < dim; d++) {
                int ee[MAXDIM];
                for (int q = 0; q < dim; q++) ee[q] = e[q];
                double c = 1.0;
                for (int o = 0; o < 2; o++) {
                    if (ee[d] == 0) c = 0.0;
                    else { c *= ee[d]; ee[d] -= 1; }
                }
                s = s + mono_prod(ee, x, dim) * c;
            }
            b[j] = s;
        }
    }
}

/* normal derivative of the monomials, partial.jl:377-402 */
void orc_mono_normal(int dim, int nmon, const int *exps, const double *n, const double *x, double *b) {
    double tmp[64];
    for (int j = 0; j < nmon; j++) b[j] = 0.0;
    for (int d = 0; d < dim; d++) {
        if (n[d] == 0.0) continue;
        orc_mono_op(dim, nmon, exps, OP_D1, d, x, tmp);
        for (int j = 0; j < nmon; j++) b[j] = b[j] + n[d] * tmp[j];
    }
}

/* ------------------------------------------------------------------------ */
/* rook-pivoted Bunch-Kaufman (LAPACK dsytf2_rook / dsytrs_rook, UPLO='U')     */
/* column-major, 1-based macros                                                */
/* ------------------------------------------------------------------------ */
#define A_(i, j) a[((j)-1) * (size_t)lda + ((i)-1)]
#define B_(i, j) bm[((j)-1) * (size_t)ldb + ((i)-1)]

static int idamax_col(int n, const double *a, int lda, int i0, int j) { /* rows i0..i0+n-1 of col j */
    int best = 1;
    double bv = -1.0;
    for (int t = 0; t < n; t++) {
        double v = fabs(A_(i0 + t, j));
        if (v > bv) { bv = v; best = t + 1; }
    }
    return best;
}
static int idamax_row(int n, const double *a, int lda, int i, int j0) { /* cols j0.. of row i */
    int best = 1;
    double bv = -1.0;
    for (int t = 0; t < n; t++) {
        double v = fabs(A_(i, j0 + t));
        if (v > bv) { bv = v; best = t + 1; }
    }
    return best;
}

/* returns INFO (0 ok, >0: D(info,info) is exactly zero).  fused = 1: the rank-1 / rank-2
   updates of the leading triangle as fused multiply-adds (the form optimised BLAS kernels
   such as OpenBLAS's dsyr / dgemm evaluate), otherwise products and sums rounded separately
   as the reference Fortran BLAS writes them. */
static int sytrf_rook_u(int n, double *a, int lda, int *ipiv, int fused) {
    const double alpha = (1.0 + sqrt(17.0)) / 8.0;
    const double sfmin = 2.2250738585072014e-308;
    int info = 0;
    int k = n;
    while (k >= 1) {
        int kstep = 1, p = k, kp, imax = 0, jmax;
        double absakk = fabs(A_(k, k)), colmax, rowmax;
        if (k > 1) {
            imax = idamax_col(k - 1, a, lda, 1, k);
            colmax = fabs(A_(imax, k));
        } else colmax = 0.0;
        if (fmax(absakk, colmax) == 0.0 || isnan(absakk) || isnan(colmax)) {
            if (info == 0) info = k;
            kp = k;
        } else {
            if (!(absakk < alpha * colmax)) {
                kp = k;
            } else {
                int done = 0;
                while (!done) {
                    if (imax != k) {
                        jmax = imax + idamax_row(k - imax, a, lda, imax, imax + 1);
                        rowmax = fabs(A_(imax, jmax));
                    } else rowmax = 0.0;
                    if (imax > 1) {
                        int itemp = idamax_col(imax - 1, a, lda, 1, imax);
                        double dtemp = fabs(A_(itemp, imax));
                        if (dtemp > rowmax) { rowmax = dtemp; jmax = itemp; }
                    }
                    if (!(fabs(A_(imax, imax)) < alpha * rowmax)) {
                        kp = imax; done = 1;
                    } else if (p == jmax || rowmax <= colmax) {
                        kp = imax; kstep = 2; done = 1;
                    } else {
                        p = imax; colmax = rowmax; imax = jmax;
                    }
                }
            }
            int kk = k - kstep + 1;
            if (kstep == 2 && p != k) {
                for (int t = 1; t <= p - 1; t++) { double tt = A_(t, k); A_(t, k) = A_(t, p); A_(t, p) = tt; }
                for (int t = 1; t <= k - p - 1; t++) { double tt = A_(p + t, k); A_(p + t, k) = A_(p, p + t); A_(p, p + t) = tt; }
                { double tt = A_(k, k); A_(k, k) = A_(p, p); A_(p, p) = tt; }
            }
            if (kp != kk) {
                for (int t = 1; t <= kp - 1; t++) { double tt = A_(t, kk); A_(t, kk) = A_(t, kp); A_(t, kp) = tt; }
                if (kk > 1 && kp < kk - 1)
                    for (int t = 1; t <= kk - kp - 1; t++) { double tt = A_(kp + t, kk); A_(kp + t, kk) = A_(kp, kp + t); A_(kp, kp + t) = tt; }
                { double tt = A_(kk, kk); A_(kk, kk) = A_(kp, kp); A_(kp, kp) = tt; }
                if (kstep == 2) { double tt = A_(k - 1, k); A_(k - 1, k) = A_(kp, k); A_(kp, k) = tt; }
            }
            if (kstep == 1) {
                if (k > 1) {
                    if (fabs(A_(k, k)) >= sfmin) {
                        double d11 = 1.0 / A_(k, k);
                        /* dsyr upper: A := A - d11 * x x^T, x = A(1:k-1,k) */
                        for (int j = 1; j <= k - 1; j++) {
                            if (A_(j, k) != 0.0) {
                                double temp = -d11 * A_(j, k);
                                for (int i = 1; i <= j; i++)
                                    A_(i, j) = fused ? fma(A_(i, k), temp, A_(i, j)) : A_(i, j) + A_(i, k) * temp;
                            }
                        }
                        for (int i = 1; i <= k - 1; i++) A_(i, k) = d11 * A_(i, k);
                    } else {
                        double d11 = A_(k, k);
                        for (int i = 1; i <= k - 1; i++) A_(i, k) = A_(i, k) / d11;
                        for (int j = 1; j <= k - 1; j++) {
                            if (A_(j, k) != 0.0) {
                                double temp = -d11 * A_(j, k);
                                for (int i = 1; i <= j; i++)
                                    A_(i, j) = fused ? fma(A_(i, k), temp, A_(i, j)) : A_(i, j) + A_(i, k) * temp;
                            }
                        }
                    }
                }
            } else {
                if (k > 2) {
                    double d12 = A_(k - 1, k);
                    double d22 = A_(k - 1, k - 1) / d12;
                    double d11 = A_(k, k) / d12;
                    double t = 1.0 / (d11 * d22 - 1.0);
                    for (int j = k - 2; j >= 1; j--) {
                        double wkm1 = t * (d11 * A_(j, k - 1) - A_(j, k));
                        double wk = t * (d22 * A_(j, k) - A_(j, k - 1));
                        for (int i = j; i >= 1; i--) {
                            if (fused)
                                A_(i, j) = fma(-(A_(i, k - 1) / d12), wkm1, fma(-(A_(i, k) / d12), wk, A_(i, j)));
                            else
                                A_(i, j) = A_(i, j) - (A_(i, k) / d12) * wk - (A_(i, k - 1) / d12) * wkm1;
                        }
                        A_(j, k) = wk / d12;
                        A_(j, k - 1) = wkm1 / d12;
                    }
                }
            }
        }
        if (kstep == 1) ipiv[k - 1] = kp;
        else { ipiv[k - 1] = -p; ipiv[k - 2] = -kp; }
        k -= kstep;
    }
    return info;
}

int orc_sytrf_rook_u(int n, double *a, int lda, int *ipiv) { return sytrf_rook_u(n, a, lda, ipiv, 0); }
int orc_sytrf_rook_u_fma(int n, double *a, int lda, int *ipiv) { return sytrf_rook_u(n, a, lda, ipiv, 1); }

void orc_sytrs_rook_u(int n, int nrhs, const double *a, int lda, const int *ipiv, double *bm, int ldb) {
    int k = n;
    while (k >= 1) {
        if (ipiv[k - 1] > 0) {
            int kp = ipiv[k - 1];
            if (kp != k)
                for (int j = 1; j <= nrhs; j++) { double t = B_(k, j); B_(k, j) = B_(kp, j); B_(kp, j) = t; }
            for (int j = 1; j <= nrhs; j++) { /* dger: B(1:k-1,:) -= A(1:k-1,k) B(k,:) */
                double temp = -B_(k, j);
                if (B_(k, j) != 0.0)
                    for (int i = 1; i <= k - 1; i++) B_(i, j) = B_(i, j) + A_(i, k) * temp;
            }
            double s = 1.0 / A_(k, k);
            for (int j = 1; j <= nrhs; j++) B_(k, j) = s * B_(k, j);
            k -= 1;
        } else {
            int kp = -ipiv[k - 1];
            if (kp != k)
                for (int j = 1; j <= nrhs; j++) { double t = B_(k, j); B_(k, j) = B_(kp, j); B_(kp, j) = t; }
            kp = -ipiv[k - 2];
            if (kp != k - 1)
                for (int j = 1; j <= nrhs; j++) { double t = B_(k - 1, j); B_(k - 1, j) = B_(kp, j); B_(kp, j) = t; }
            if (k > 2) {
                for (int j = 1; j <= nrhs; j++) {
                    double temp = -B_(k, j);
                    if (B_(k, j) != 0.0)
                        for (int i = 1; i <= k - 2; i++) B_(i, j) = B_(i, j) + A_(i, k) * temp;
                }
                for (int j = 1; j <= nrhs; j++) {
                    double temp = -B_(k - 1, j);
                    if (B_(k - 1, j) != 0.0)
                        for (int i = 1; i <= k - 2; i++) B_(i, j) = B_(i, j) + A_(i, k - 1) * temp;
                }
            }
            double akm1k = A_(k - 1, k);
            double akm1 = A_(k - 1, k - 1) / akm1k;
            double ak = A_(k, k) / akm1k;
            double denom = akm1 * ak - 1.0;
            for (int j = 1; j <= nrhs; j++) {
                double bkm1 = B_(k - 1, j) / akm1k;
                double bk = B_(k, j) / akm1k;
                B_(k - 1, j) = (ak * bkm1 - bk) / denom;
                B_(k, j) = (akm1 * bk - bkm1) / denom;
            }
            k -= 2;
        }
    }
    k = 1;
    while (k <= n) {
        if (ipiv[k - 1] > 0) {
            if (k > 1)
                for (int j = 1; j <= nrhs; j++) { /* dgemv T: B(k,j) -= A(1:k-1,k) . B(1:k-1,j) */
                    double temp = 0.0;
                    for (int i = 1; i <= k - 1; i++) temp = temp + A_(i, k) * B_(i, j);
                    B_(k, j) = B_(k, j) - temp;
                }
            int kp = ipiv[k - 1];
            if (kp != k)
                for (int j = 1; j <= nrhs; j++) { double t = B_(k, j); B_(k, j) = B_(kp, j); B_(kp, j) = t; }
            k += 1;
        } else {
            if (k > 1) {
                for (int j = 1; j <= nrhs; j++) {
                    double temp = 0.0;
                    for (int i = 1; i <= k - 1; i++) temp = temp + A_(i, k) * B_(i, j);
                    B_(k, j) = B_(k, j) - temp;
                }
                for (int j = 1; j <= nrhs; j++) {
                    double temp = 0.0;
                    for (int i = 1; i <= k - 1; i++) temp = temp + A_(i, k + 1) * B_(i, j);
                    B_(k + 1, j) = B_(k + 1, j) - temp;
                }
            }
            int kp = -ipiv[k - 1];
            if (kp != k)
                for (int j = 1; j <= nrhs; j++) { double t = B_(k, j); B_(k, j) = B_(kp, j); B_(kp, j) = t; }
            kp = -ipiv[k];
            if (kp != k + 1)
                for (int j = 1; j <= nrhs; j++) { double t = B_(k + 1, j); B_(k + 1, j) = B_(kp, j); B_(kp, j) = t; }
            k += 2;
        }
    }
}
#undef A_
#undef B_

/* ------------------------------------------------------------------------ */
/* per-stencil assembly                                                        */
/* ------------------------------------------------------------------------ */
typedef struct {
    int dim, phs, poly_deg, nops;
    int op_code[8];
    int op_dim[8];
} orc_cfg;

enum { PT_INTERIOR = 0, PT_DIRICHLET = 1, PT_NR = 2 };

/* Local Hermite description of a stencil: ptype per point, alpha/beta/normal for NR points. */
typedef struct {
    int ptype[MAXN];
    double alpha[MAXN], beta[MAXN];
    double normal[MAXN * MAXDIM];
    int eval_local; /* 0-based local index of the eval point, -1 if absent */
} herm_local;

/* Hermite matrix entry, assembly.jl:251-332 */
static double herm_entry(const orc_cfg *c, const double *X, const herm_local *h, int i, int j) {
    int dim = c->dim;
    const double *xi = X + i * dim, *xj = X + j * dim;
    double phi = orc_phs_phi(c->phs, xi, xj, dim);
    int ti = h->ptype[i], tj = h->ptype[j];
    if (ti != PT_NR && tj != PT_NR) return phi;
    double g[MAXDIM];
    orc_phs_grad(c->phs, xi, xj, dim, g);
    if (ti != PT_NR && tj == PT_NR) {
        double dj = 0.0;
        for (int d = 0; d < dim; d++) dj = dj + h->normal[j * dim + d] * g[d];
        return h->alpha[j] * phi - h->beta[j] * dj;
    }
    if (ti == PT_NR && tj != PT_NR) {
        double di = 0.0;
        for (int d = 0; d < dim; d++) di = di + h->normal[i * dim + d] * g[d];
        return h->alpha[i] * phi + h->beta[i] * di;
    }
    double H[MAXDIM * MAXDIM];
    orc_phs_hess(c->phs, xi, xj, dim, H);
    double di = 0.0, dj = 0.0, d2 = 0.0;
    for (int d = 0; d < dim; d++) di = di + h->normal[i * dim + d] * g[d];
    for (int d = 0; d < dim; d++) dj = dj + h->normal[j * dim + d] * g[d];
    for (int a = 0; a < dim; a++) { /* dot(ni, H*nj) */
        double hn = 0.0;
        for (int b = 0; b < dim; b++) hn = hn + H[a * dim + b] * h->normal[j * dim + b];
        d2 = d2 + h->normal[i * dim + a] * hn;
    }
    double ai = h->alpha[i], bi = h->beta[i], aj = h->alpha[j], bj = h->beta[j];
    return ai * aj * phi - ai * bj * dj + bi * aj * di + bi * bj * d2;
}

/* Assemble A (n x n, column-major, upper triangle only, rest zero) and B (n x nops).
 * X: k points (row-major k x dim), x0: eval point, h: NULL for an interior stencil.
 * Returns 0, or -1 if a Hermite stencil needs an eval point absent from the stencil,
 * or -2 if a Neumann/Robin point needs a normal form the operator lacks. */
int orc_assemble(const orc_cfg *c, const double *X, int k, const double *x0, const herm_local *h,
                 double *A, double *B) {
    int dim = c->dim;
    int exps[64 * MAXDIM];
    int nmon = orc_monomial_exponents(dim, c->poly_deg, exps);
    int n = k + nmon;
    memset(A, 0, sizeof(double) * n * n);
    memset(B, 0, sizeof(double) * n * c->nops);
    for (int j = 0; j < k; j++)
        for (int i = 0; i <= j; i++)
            A[j * n + i] = h ? herm_entry(c, X, h, i, j) : orc_phs_phi(c->phs, X + i * dim, X + j * dim, dim);
    double pv[64], pn[64];
    for (int i = 0; i < k; i++) {
        if (nmon == 0) break;
        orc_mono_op(dim, nmon, exps, OP_IDENT, 0, X + i * dim, pv);
        if (h && h->ptype[i] == PT_NR) { /* alpha*P + beta*dnP, assembly.jl:362-386 */
            orc_mono_normal(dim, nmon, exps, h->normal + i * dim, X + i * dim, pn);
            for (int m = 0; m < nmon; m++) pv[m] = h->alpha[i] * pv[m] + h->beta[i] * pn[m];
        }
        for (int m = 0; m < nmon; m++) A[(k + m) * n + i] = pv[m];
    }
    for (int r = 0; r < c->nops; r++) {
        int op = c->op_code[r], od = c->op_dim[r];
        double *b = B + r * n;
        for (int i = 0; i < k; i++) {
            const double *xi = X + i * dim;
            if (h && h->ptype[i] == PT_NR) { /* assembly.jl:399-409 */
                double nf = orc_phs_op_normal(c->phs, op, od, x0, xi, h->normal + i * dim, dim);
                if (isnan(nf) && op == OP_IDENT) return -2;
                b[i] = h->alpha[i] * orc_phs_op(c->phs, op, od, x0, xi, dim) + h->beta[i] * nf;
            } else {
                b[i] = orc_phs_op(c->phs, op, od, x0, xi, dim);
            }
        }
        if (nmon > 0) {
            if (h) {
                if (h->eval_local < 0) return -1;
                int e = h->eval_local;
                if (h->ptype[e] == PT_NR) { /* quirk: alpha*P(x0) + beta*dnP(x0), assembly.jl:452-468 */
                    orc_mono_op(dim, nmon, exps, OP_IDENT, 0, x0, pv);
                    orc_mono_normal(dim, nmon, exps, h->normal + e * dim, x0, pn);
                    for (int m = 0; m < nmon; m++) b[k + m] = h->alpha[e] * pv[m] + h->beta[e] * pn[m];
                    continue;
                }
            }
            orc_mono_op(dim, nmon, exps, op, od, x0, b + k);
        }
    }
    return 0;
}

/* Solve one stencil: assemble + rook LDL^T + solve. w: k x nops (column-major by op).
 * Returns 0 ok, 1 singular (exact zero pivot), <0 assembly error. */
int orc_stencil_weights(const orc_cfg *c, const double *X, int k, const double *x0,
                        const herm_local *h, double *w) {
    int exps[64 * MAXDIM];
    int nmon = orc_monomial_exponents(c->dim, c->poly_deg, exps);
    int n = k + nmon;
    double *A = (double *)malloc(sizeof(double) * n * n);
    double *B = (double *)malloc(sizeof(double) * n * c->nops);
    int ipiv[MAXN];
    int st = orc_assemble(c, X, k, x0, h, A, B);
    if (st == 0) {
        int info = orc_sytrf_rook_u(n, A, n, ipiv);
        if (info != 0) st = 1;
        else {
            orc_sytrs_rook_u(n, c->nops, A, n, ipiv, B, n);
            for (int r = 0; r < c->nops; r++)
                for (int i = 0; i < k; i++) w[r * k + i] = B[r * n + i];
        }
    }
    free(A);
    free(B);
    return st;
}

/* ------------------------------------------------------------------------ */
/* global build: classify, count, solve, write sorted sparse rows             */
/* execution.jl:39-115,186-303 ; types.jl:133-223                              */
/* ------------------------------------------------------------------------ */

/* row_ptr (ne+1) from the exact count: Dirichlet eval rows hold 1 entry. */
int64_t orc_count_rows(int64_t ne, int k, const uint8_t *is_boundary, const int32_t *g2b,
                       const double *bc_alpha, const double *bc_beta, int64_t *row_ptr) {
    int64_t tot = 0;
    row_ptr[0] = 0;
    for (int64_t e = 0; e < ne; e++) {
        int dir = 0;
        if (is_boundary && is_boundary[e]) {
            int32_t b = g2b[e];
            dir = (bc_alpha[b] == 1.0 && bc_beta[b] == 0.0);
        }
        tot += dir ? 1 : k;
        row_ptr[e + 1] = tot;
    }
    return tot;
}

static int op_order(int op) { return op == OP_IDENT ? 0 : (op == OP_D1 ? 1 : 2); }

/* One stencil in its local frame: X (k points) and x0 already centred at the eval point and
 * scaled by 2^-es, Neumann/Robin beta by 2^-es, the avoid_inf guards set to avoid_inf / s^b.
 * The reference formulation is affine invariant except for the eval-node polynomial
 * right-hand side of a Neumann/Robin eval node (alpha P(x0) + beta dP/dn(x0), not an
 * operator applied), scaled here by s^q; the weights come back as w_local / s^q (q the
 * operator's differential order). */
static int orc_stencil_weights_local(const orc_cfg *c, const double *X, int k, const double *x0,
                                     const herm_local *h, int es, double *w) {
    int exps[64 * MAXDIM];
    int nmon = orc_monomial_exponents(c->dim, c->poly_deg, exps);
    int n = k + nmon;
    double *A = (double *)malloc(sizeof(double) * n * n);
    double *B = (double *)malloc(sizeof(double) * n * c->nops);
    int ipiv[MAXN];
    int st = orc_assemble(c, X, k, x0, h, A, B);
    if (st == 0 && h && h->eval_local >= 0 && h->ptype[h->eval_local] == PT_NR)
        for (int r = 0; r < c->nops; r++)
            for (int m = 0; m < nmon; m++) B[r * n + k + m] = ldexp(B[r * n + k + m], es * op_order(c->op_code[r]));
    if (st == 0) {
        int info = orc_sytrf_rook_u(n, A, n, ipiv);
        if (info != 0) st = 1;
        else {
            orc_sytrs_rook_u(n, c->nops, A, n, ipiv, B, n);
            for (int r = 0; r < c->nops; r++)
                for (int i = 0; i < k; i++) w[r * k + i] = ldexp(B[r * n + i], -es * op_order(c->op_code[r]));
        }
    }
    free(A);
    free(B);
    return st;
}

/* status per eval row: 0 ok, 1 singular, 2 Dirichlet identity row, <0 error (see orc_assemble).
 * local = 0: the reference's arithmetic (raw coordinates); local = 1: the same formulation
 * assembled per stencil in its local frame (centred at the eval point, scaled by the power of
 * two s >= the stencil radius): equal weights in exact arithmetic, far better conditioned
 * systems where the stencil is small against its distance from the origin. */
static int orc_build_impl(const orc_cfg *c, const double *data, int64_t ns, const double *eval, int64_t ne,
                          const int32_t *adjl, int k, const uint8_t *is_boundary, const double *bc_alpha,
                          const double *bc_beta, const double *normals, const int64_t *row_ptr,
                          int32_t *col, double *val, int8_t *status, int nthreads, int local) {
    int dim = c->dim;
    int32_t *g2b = NULL;
    if (is_boundary) {
        g2b = (int32_t *)malloc(sizeof(int32_t) * (ns > ne ? ns : ne));
        int32_t cnt = 0;
        for (int64_t i = 0; i < ns; i++) g2b[i] = is_boundary[i] ? cnt++ : -1;
    }
    int64_t nnz = row_ptr[ne];
    int bad = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64) reduction(| : bad)
#endif
    for (int64_t e = 0; e < ne; e++) {
        const int32_t *nb = adjl + e * (int64_t)k;
        const double *x0 = eval + e * dim;
        double X[MAXN * MAXDIM];
        double w[MAXN * 8];
        herm_local hl;
        const herm_local *hp = NULL;
        int anyb = 0;
        if (is_boundary)
            for (int i = 0; i < k; i++) anyb |= is_boundary[nb[i]];
        if (anyb && is_boundary[e] && bc_alpha[g2b[e]] == 1.0 && bc_beta[g2b[e]] == 0.0) {
            int64_t p = row_ptr[e];
            col[p] = (int32_t)e;
            for (int r = 0; r < c->nops; r++) val[r * nnz + p] = 1.0;
            status[e] = 2;
            continue;
        }
        for (int i = 0; i < k; i++)
            for (int d = 0; d < dim; d++) X[i * dim + d] = data[(int64_t)nb[i] * dim + d];
        if (anyb) {
            hl.eval_local = -1;
            for (int i = 0; i < k; i++) {
                int32_t g = nb[i];
                int same = 1;
                for (int d = 0; d < dim; d++) same &= (X[i * dim + d] == x0[d]);
                if (same && hl.eval_local < 0) hl.eval_local = i;
                if (is_boundary[g]) {
                    int32_t b = g2b[g];
                    hl.alpha[i] = bc_alpha[b];
                    hl.beta[i] = bc_beta[b];
                    hl.ptype[i] = (bc_alpha[b] == 1.0 && bc_beta[b] == 0.0) ? PT_DIRICHLET : PT_NR;
                    for (int d = 0; d < dim; d++) hl.normal[i * dim + d] = normals[(int64_t)b * dim + d];
                } else {
                    hl.alpha[i] = 0.0;
                    hl.beta[i] = 0.0;
                    hl.ptype[i] = PT_INTERIOR;
                    for (int d = 0; d < dim; d++) hl.normal[i * dim + d] = 0.0;
                }
            }
            hp = &hl;
        }
        int st;
        if (local) {
            double r2max = 0.0;
            for (int i = 0; i < k; i++) {
                double r2 = 0.0;
                for (int d = 0; d < dim; d++) r2 = r2 + (X[i * dim + d] - x0[d]) * (X[i * dim + d] - x0[d]);
                if (r2 > r2max) r2max = r2;
            }
            int es = 0;
            if (r2max > 0.0) frexp(sqrt(r2max), &es);
            for (int i = 0; i < k; i++)
                for (int d = 0; d < dim; d++) X[i * dim + d] = ldexp(X[i * dim + d] - x0[d], -es);
            if (hp)
                for (int i = 0; i < k; i++)
                    if (hl.ptype[i] == PT_NR) hl.beta[i] = ldexp(hl.beta[i], -es);
            const double zero[MAXDIM] = {0.0, 0.0, 0.0};
            orc_ai1 = ldexp(AVOID_INF, -es);
            orc_ai2 = ldexp(AVOID_INF, -2 * es);
            orc_ai3 = ldexp(AVOID_INF, -3 * es);
            orc_ai5 = ldexp(AVOID_INF, -5 * es);
            st = orc_stencil_weights_local(c, X, k, zero, hp, es, w);
            orc_ai1 = orc_ai2 = orc_ai3 = orc_ai5 = AVOID_INF;
        } else {
            st = orc_stencil_weights(c, X, k, x0, hp, w);
        }
        status[e] = (int8_t)st;
        if (st != 0) { bad = 1; continue; }
        /* scatter the row sorted by column (sparse() keeps columns sorted) */
        int64_t p = row_ptr[e];
        int ord[MAXN];
        for (int i = 0; i < k; i++) ord[i] = i;
        for (int i = 1; i < k; i++) { /* insertion sort by column */
            int t = ord[i], j = i - 1;
            while (j >= 0 && nb[ord[j]] > nb[t]) { ord[j + 1] = ord[j]; j--; }
            ord[j + 1] = t;
        }
        for (int i = 0; i < k; i++) {
            col[p + i] = nb[ord[i]];
            for (int r = 0; r < c->nops; r++) val[r * nnz + p + i] = w[r * k + ord[i]];
        }
    }
    free(g2b);
    return bad;
}

int orc_build(const orc_cfg *c, const double *data, int64_t ns, const double *eval, int64_t ne,
              const int32_t *adjl, int k, const uint8_t *is_boundary, const double *bc_alpha,
              const double *bc_beta, const double *normals, const int64_t *row_ptr,
              int32_t *col, double *val, int8_t *status, int nthreads) {
    return orc_build_impl(c, data, ns, eval, ne, adjl, k, is_boundary, bc_alpha, bc_beta, normals, row_ptr, col,
                          val, status, nthreads, 0);
}

int orc_build_local(const orc_cfg *c, const double *data, int64_t ns, const double *eval, int64_t ne,
                    const int32_t *adjl, int k, const uint8_t *is_boundary, const double *bc_alpha,
                    const double *bc_beta, const double *normals, const int64_t *row_ptr,
                    int32_t *col, double *val, int8_t *status, int nthreads) {
    return orc_build_impl(c, data, ns, eval, ne, adjl, k, is_boundary, bc_alpha, bc_beta, normals, row_ptr, col,
                          val, status, nthreads, 1);
}

/* ------------------------------------------------------------------------ */
/* apply: y = alpha * W x + beta * y for B fields (x: ns x nf, y: ne x nf, both
 * column-major = one contiguous column per field, the layout of a Julia Matrix)  */
/* ------------------------------------------------------------------------ */
void orc_spmm(int64_t ne, int64_t ns, const int64_t *row_ptr, const int32_t *col, const double *val,
              int nf, const double *x, double alpha, double beta, double *y, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (int64_t r = 0; r < ne; r++) {
        for (int f = 0; f < nf; f++) {
            double s = 0.0;
            for (int64_t p = row_ptr[r]; p < row_ptr[r + 1]; p++) s = s + val[p] * x[f * ns + col[p]];
            double prev = (beta == 0.0) ? 0.0 : beta * y[f * ne + r];
            y[f * ne + r] = alpha * s + prev;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* k nearest neighbours, sorted by (squared distance, index)                   */
/* ------------------------------------------------------------------------ */
typedef struct { double d; int32_t i; } dpair;

static inline int dless(double d1, int32_t i1, double d2, int32_t i2) {
    return d1 < d2 || (d1 == d2 && i1 < i2);
}

static void topk_insert(dpair *best, int *cnt, int k, double d, int32_t i) {
    int c = *cnt;
    if (c == k && !dless(d, i, best[k - 1].d, best[k - 1].i)) return;
    int j = (c < k) ? c : k - 1;
    while (j > 0 && dless(d, i, best[j - 1].d, best[j - 1].i)) { best[j] = best[j - 1]; j--; }
    best[j].d = d;
    best[j].i = i;
    if (c < k) *cnt = c + 1;
}

void orc_knn_brute(const double *src, int64_t ns, const double *q, int64_t nq, int dim, int k,
                   int32_t *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t t = 0; t < nq; t++) {
        dpair best[MAXN];
        int cnt = 0;
        for (int64_t s = 0; s < ns; s++) topk_insert(best, &cnt, k, sqeuc(q + t * dim, src + s * dim, dim), (int32_t)s);
        for (int j = 0; j < k; j++) out[t * k + j] = best[j].i;
    }
}

/* Uniform-grid exact kNN: cells of side h; rings of cells are scanned until the k-th
 * candidate lies within the distance already covered. */
int orc_knn_grid(const double *src, int64_t ns, const double *q, int64_t nq, int dim, int k,
                 int32_t *out, int nthreads) {
    if (k > ns || k > MAXN) return -1;
    double lo[MAXDIM], hi[MAXDIM];
    for (int d = 0; d < dim; d++) { lo[d] = INFINITY; hi[d] = -INFINITY; }
    for (int64_t s = 0; s < ns; s++)
        for (int d = 0; d < dim; d++) {
            double v = src[s * dim + d];
            if (v < lo[d]) lo[d] = v;
            if (v > hi[d]) hi[d] = v;
        }
    double vol = 1.0, ext[MAXDIM];
    for (int d = 0; d < dim; d++) { ext[d] = hi[d] - lo[d]; if (ext[d] <= 0) ext[d] = 1e-300; vol *= ext[d]; }
    double target = (double)ns / 2.0; /* about two points per cell */
    double h = pow(vol / (target > 1 ? target : 1), 1.0 / dim);
    int64_t nc[MAXDIM], ntot = 1;
    for (int d = 0; d < dim; d++) {
        int64_t m = (int64_t)(ext[d] / h) + 1;
        if (m > 4096) m = 4096;
        nc[d] = m;
        ntot *= m;
    }
    for (int d = dim; d < MAXDIM; d++) nc[d] = 1;
    double hc[MAXDIM];
    for (int d = 0; d < dim; d++) hc[d] = ext[d] / (double)nc[d];
    int64_t *cell_start = (int64_t *)calloc(ntot + 1, sizeof(int64_t));
    int64_t *cell_of = (int64_t *)malloc(sizeof(int64_t) * ns);
    int32_t *sorted = (int32_t *)malloc(sizeof(int32_t) * ns);
    for (int64_t s = 0; s < ns; s++) {
        int64_t cid = 0;
        for (int d = dim - 1; d >= 0; d--) {
            int64_t c = (int64_t)((src[s * dim + d] - lo[d]) / hc[d]);
            if (c < 0) c = 0;
            if (c >= nc[d]) c = nc[d] - 1;
            cid = cid * nc[d] + c;
        }
        cell_of[s] = cid;
        cell_start[cid + 1]++;
    }
    for (int64_t c = 0; c < ntot; c++) cell_start[c + 1] += cell_start[c];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * ntot);
    memcpy(fill, cell_start, sizeof(int64_t) * ntot);
    for (int64_t s = 0; s < ns; s++) sorted[fill[cell_of[s]]++] = (int32_t)s;
    free(fill);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t t = 0; t < nq; t++) {
        const double *qp = q + t * dim;
        int64_t qc[MAXDIM] = {0, 0, 0};
        for (int d = 0; d < dim; d++) {
            int64_t c = (int64_t)floor((qp[d] - lo[d]) / hc[d]);
            qc[d] = c;
        }
        dpair best[MAXN];
        int cnt = 0;
        for (int ring = 0;; ring++) {
            /* visit cells whose Chebyshev distance (in cells) from qc equals ring */
            int64_t r = ring;
            int64_t a0 = qc[0] - r, a1 = qc[0] + r;
            int64_t b0 = dim > 1 ? qc[1] - r : 0, b1 = dim > 1 ? qc[1] + r : 0;
            int64_t c0 = dim > 2 ? qc[2] - r : 0, c1 = dim > 2 ? qc[2] + r : 0;
            int any_inside = 0;
            for (int64_t cz = c0; cz <= c1; cz++)
                for (int64_t cy = b0; cy <= b1; cy++)
                    for (int64_t cx = a0; cx <= a1; cx++) {
                        int64_t m = llabs(cx - qc[0]);
                        if (dim > 1 && llabs(cy - qc[1]) > m) m = llabs(cy - qc[1]);
                        if (dim > 2 && llabs(cz - qc[2]) > m) m = llabs(cz - qc[2]);
                        if (m != r) continue;
                        if (cx < 0 || cx >= nc[0] || cy < 0 || cy >= nc[1] || cz < 0 || cz >= nc[2]) continue;
                        any_inside = 1;
                        int64_t cid = (cz * nc[1] + cy) * nc[0] + cx;
                        for (int64_t p = cell_start[cid]; p < cell_start[cid + 1]; p++) {
                            int32_t s = sorted[p];
                            topk_insert(best, &cnt, k, sqeuc(qp, src + (int64_t)s * dim, dim), s);
                        }
                    }
            /* distance from the query to the outside of the scanned block */
            double cover = INFINITY;
            for (int d = 0; d < dim; d++) {
                double lo_edge = lo[d] + (double)(qc[d] - r) * hc[d];
                double hi_edge = lo[d] + (double)(qc[d] + r + 1) * hc[d];
                double m1 = qp[d] - lo_edge, m2 = hi_edge - qp[d];
                if (qc[d] - r <= 0) m1 = INFINITY;
                if (qc[d] + r >= nc[d] - 1) m2 = INFINITY;
                if (m1 < cover) cover = m1;
                if (m2 < cover) cover = m2;
            }
            if (cnt == k && (best[k - 1].d < cover * cover * (1.0 - 1e-12))) break;
            if (!any_inside && cover == INFINITY) break;
            if (cover == INFINITY && cnt == k) break;
        }
        for (int j = 0; j < k; j++) out[t * k + j] = best[j].i;
    }
    free(cell_start);
    free(cell_of);
    free(sorted);
    return 0;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* global interpolation: Interpolator(x, y, basis) (src/interpolation.jl:22-37) */
/* ------------------------------------------------------------------------ */
/* Upper triangle of the collocation matrix of all n points (column-major, order
   nt = n + nmon, leading dimension nt), as _build_collocation_matrix!
   (src/solve/assembly.jl:95-115) fills it: phi(x_i, x_j) for i <= j < n, P(x_i) in the
   polynomial columns, zeros in the polynomial block. */
int orc_interp_matrix(int dim, int phs, int poly_deg, const double *x, int64_t n, double *A) {
    int exps[64 * MAXDIM];
    int nmon = orc_monomial_exponents(dim, poly_deg, exps);
    int64_t nt = n + nmon;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t j = 0; j < n; j++)
        for (int64_t i = 0; i <= j; i++) A[j * nt + i] = orc_phs_phi(phs, x + i * dim, x + j * dim, dim);
    for (int m = 0; m < nmon; m++) {
        double *col = A + (n + m) * nt;
        for (int64_t i = 0; i < n; i++) col[i] = mono_prod(exps + m * dim, x + i * dim, dim);
        for (int64_t i = n; i <= n + m; i++) col[i] = 0.0;
    }
    return nmon;
}

/* (rbfi::Interpolator)(x) (src/interpolation.jl:39-50) at m points: the RBF sum over the
   n centres in order, then the dot product of the monomial weights with P(x) in order,
   then their sum.  coef = [rbf weights (n); monomial weights (nmon)]. */
void orc_interp_eval(int dim, int phs, int poly_deg, const double *x, int64_t n, const double *coef,
                     const double *xe, int64_t m, double *out, int nthreads) {
    int exps[64 * MAXDIM];
    int nmon = orc_monomial_exponents(dim, poly_deg, exps);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t t = 0; t < m; t++) {
        const double *p = xe + t * dim;
        double rbf = 0.0;
        for (int64_t i = 0; i < n; i++) rbf = rbf + coef[i] * orc_phs_phi(phs, p, x + i * dim, dim);
        double poly = 0.0;
        for (int q = 0; q < nmon; q++) poly = poly + coef[n + q] * mono_prod(exps + q * dim, p, dim);
        out[t] = rbf + poly;
    }
}

/* ------------------------------------------------------------------------ */
/* pullback of the weight build (reverse-mode sensitivities to the points):  */
/* src/solve/ad_shared.jl:63-127 with src/solve/backward.jl:31-363, in the   */
/* reference's global coordinates                                            */
/* ------------------------------------------------------------------------ */
/* d^alpha of monomial e at x */
static double mono_dalpha(const int *e, const int *alpha, const double *x, int dim) {
    double v = 1.0;
    for (int d = 0; d < dim; d++) {
        if (alpha[d] > e[d]) return 0.0;
        double c = 1.0;
        for (int t = 0; t < alpha[d]; t++) c *= (double)(e[d] - t);
        v *= c;
        for (int t = 0; t < e[d] - alpha[d]; t++) v *= x[d];
    }
    return v;
}

/* d/dx of (L phi)(x, xi) at D = x - xi (operator_second_derivatives.jl; PHS1 rows vanish
   below r = 1e-12; the identity uses the basis gradient) */
static void grad_applied(int p, int op, int od, const double *D, int dim, double *g) {
    double r2 = 0.0;
    for (int d = 0; d < dim; d++) r2 = r2 + D[d] * D[d];
    const double r = sqrt(r2);
    if (op == OP_IDENT) {
        const double c = p == 1 ? 1.0 / (r + AI_R1) : (p == 3 ? 3.0 * r : (p == 5 ? 5.0 * pw3(r) : 7.0 * pw5(r)));
        for (int d = 0; d < dim; d++) g[d] = c * D[d];
        return;
    }
    if (p == 1 && r < 1.0e-12) {
        for (int d = 0; d < dim; d++) g[d] = 0.0;
        return;
    }
    if (op == OP_LAP) {
        const double c = p == 1 ? -2.0 / pw3(r) : (p == 3 ? 12.0 / (r + AI_R1) : (p == 5 ? 90.0 * r : 280.0 * pw3(r)));
        for (int d = 0; d < dim; d++) g[d] = c * D[d];
        return;
    }
    const double dd = D[od];
    double a, b;
    if (p == 1) { a = -1.0 / pw3(r); b = 1.0 / r; }
    else if (p == 3) { a = 3.0 / (r + AI_R1); b = 3.0 * r; }
    else if (p == 5) { a = 15.0 * r; b = 5.0 * pw3(r); }
    else { a = 35.0 * pw3(r); b = 7.0 * pw5(r); }
    for (int d = 0; d < dim; d++) g[d] = a * dd * D[d] + (d == od ? b : 0.0);
}

/* Gradients of L = sum dW .* w (w the weights in stencil order, dW: nops x ne x k) with
   respect to the data points (ddata, ns x dim, accumulated) and the eval points (deval,
   ne x dim).  Interior stencils; PHS 1/3/5/7; identity, first partials, Laplacian.
   Returns the number of singular stencils. */
int orc_build_backward(const orc_cfg *c, const double *data, int64_t ns, const double *eval, int64_t ne,
                       const int32_t *adjl, int k, const double *dW, double *ddata, double *deval, int nthreads) {
    (void)ns;
    const int dim = c->dim, nops = c->nops;
    int exps[64 * MAXDIM];
    const int nmon = orc_monomial_exponents(dim, c->poly_deg, exps);
    const int n = k + nmon;
    int bad = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : bad)
#endif
    for (int64_t e = 0; e < ne; e++) {
        const int32_t *nb = adjl + e * (int64_t)k;
        const double *x0 = eval + e * dim;
        double X[MAXN * MAXDIM];
        double *A = (double *)malloc(sizeof(double) * n * n);
        double *S = (double *)malloc(sizeof(double) * n * 2 * nops);  /* [lambda | eta], column-major */
        int *ipiv = (int *)malloc(sizeof(int) * n);
        for (int i = 0; i < k; i++)
            for (int d = 0; d < dim; d++) X[i * dim + d] = data[(int64_t)nb[i] * dim + d];
        orc_assemble(c, X, k, x0, NULL, A, S);
        for (int q = 0; q < nops; q++)
            for (int i = 0; i < n; i++)
                S[(nops + q) * n + i] = i < k ? dW[((int64_t)q * ne + e) * k + i] : 0.0;
        if (sytrf_rook_u(n, A, n, ipiv, 0) != 0) {
            bad++;
            free(A); free(S); free(ipiv);
            continue;
        }
        orc_sytrs_rook_u(n, 2 * nops, A, n, ipiv, S, n);
        const double *lam = S, *eta = S + (size_t)nops * n;
        double dX[MAXN * MAXDIM];
        double de[MAXDIM] = {0.0, 0.0, 0.0};
        for (int t = 0; t < k * dim; t++) dX[t] = 0.0;
        /* collocation: RBF pairs (backward.jl:85-131) and the polynomial block (:133-160) */
        for (int j = 0; j < k; j++)
            for (int i = 0; i < j; i++) {
                double sc = 0.0;
                for (int q = 0; q < nops; q++)
                    sc = sc - (eta[q * n + i] * lam[q * n + j] + eta[q * n + j] * lam[q * n + i]);
                double g[MAXDIM];
                orc_phs_grad(c->phs, X + i * dim, X + j * dim, dim, g);
                for (int d = 0; d < dim; d++) {
                    dX[i * dim + d] += sc * g[d];
                    dX[j * dim + d] -= sc * g[d];
                }
            }
        for (int i = 0; i < k; i++)
            for (int m = 0; m < nmon; m++) {
                double sc = 0.0;
                for (int q = 0; q < nops; q++)
                    sc = sc - (eta[q * n + i] * lam[q * n + k + m] + eta[q * n + k + m] * lam[q * n + i]);
                for (int d = 0; d < dim; d++) {
                    int al[MAXDIM] = {0, 0, 0};
                    al[d] = 1;
                    dX[i * dim + d] += sc * mono_dalpha(exps + m * dim, al, X + i * dim, dim);
                }
            }
        /* right-hand side: b_i = L phi(x0, x_i) (backward.jl:163-222) and L p_m(x0) (:223-363) */
        for (int q = 0; q < nops; q++) {
            const int op = c->op_code[q], od = c->op_dim[q];
            for (int i = 0; i < k; i++) {
                double D[MAXDIM], g[MAXDIM];
                for (int d = 0; d < dim; d++) D[d] = x0[d] - X[i * dim + d];
                grad_applied(c->phs, op, od, D, dim, g);
                for (int d = 0; d < dim; d++) {
                    de[d] += eta[q * n + i] * g[d];
                    dX[i * dim + d] -= eta[q * n + i] * g[d];
                }
            }
            for (int m = 0; m < nmon; m++)
                for (int d = 0; d < dim; d++) {
                    int al[MAXDIM] = {0, 0, 0};
                    double v = 0.0;
                    al[d] = 1;
                    if (op == OP_IDENT) {
                        v = mono_dalpha(exps + m * dim, al, x0, dim);
                    } else if (op == OP_D1) {
                        al[od] += 1;
                        v = mono_dalpha(exps + m * dim, al, x0, dim);
                    } else if (op == OP_LAP) {
                        for (int cc = 0; cc < dim; cc++) {
                            int b2[MAXDIM] = {al[0], al[1], al[2]};
                            b2[cc] += 2;
                            v += mono_dalpha(exps + m * dim, b2, x0, dim);
                        }
                    }
                    de[d] += eta[q * n + k + m] * v;
                }
        }
        for (int i = 0; i < k; i++)
            for (int d = 0; d < dim; d++) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                ddata[(int64_t)nb[i] * dim + d] += dX[i * dim + d];
            }
        for (int d = 0; d < dim; d++) deval[e * dim + d] = de[d];
        free(A);
        free(S);
        free(ipiv);
    }
    return bad;
}
