// Per-stencil math shared by the FP64 and FP32 build kernels.
//
// Every stencil is assembled in local coordinates xi = (x - x0) / s, with x0 the eval
// point and s = 2^e the smallest power of two not below the stencil radius (so the
// scaling is exact).  The RBF-FD weights do not depend on this change of variables
// (polynomial spaces are affine invariant, PHS are homogeneous): a weight for an
// operator of differential order q is w_x = w_xi / s^q, and a Neumann/Robin condition
// alpha*u + beta*du/dn reads alpha*u + (beta/s)*du/dn_xi.  The local form keeps every
// matrix entry O(1), which the FP32 factorisation needs and which makes the FP64 solve
// more accurate than the reference's raw-coordinate one.
//
// Formulas follow src/basis/polyharmonic_spline.jl (PHS1 43-119, PHS3 128-205,
// PHS5 214-290, PHS7 299-376), including the reference's Laplacian coefficients
// 2, 12, 30, 56 for r, r^3, r^5, r^7 in every dimension, and the monomial
// orders of src/basis/monomial.jl.
#pragma once
#include <cstdint>

#include "rbffd.h"

#define RBF_AVOID_INF 1.0e-16  // avoid_inf(Float64), src/RadialBasisFunctions.jl:111

enum { PT_INTERIOR = 0, PT_DIRICHLET = 1, PT_NR = 2 };

// Launch parameters of one build (passed by value, read from the constant bank).
struct StencilParams {
    int dim, phs, poly_deg, nmon, k, n, nops;
    int nnr;  // RBF_FLAG_NORMAL_DOF: the du/dn unknowns of the size class (n = k + nnr + nmon)
    int op_code[RBF_MAX_OPS];
    int op_dim[RBF_MAX_OPS];
    int op_order[RBF_MAX_OPS];
    int8_t exps[RBF_MAX_SYSTEM][3];  // monomial exponents, reference order
    int64_t ne, ns, nnz;
    const double *data;
    const double *eval;
    const int32_t *adjl;
    const uint8_t *isb;     // nullptr: no boundary
    const int32_t *g2b;
    const double *alpha;
    const double *beta;
    const double *normals;
    const int64_t *row_ptr;
    int32_t *col;
    double *val;
    int8_t *status;
    unsigned long long *counters;  // [0] singular [1] eval-not-found [2] fallback [3] identity rows
                                   // [4] FP64 residual evaluations (FP32 paths)
                                   // [5] sum of 1e6 * min(1, |x1 - seed| / |x1|) over seeded
                                   //     stencils, [6] their number, [7] deferred stencils
    double *max_resid;             // largest accepted relative residual (FP32 paths)
    int refine_steps;
    double tol;
    int flags;          // RBF_FLAG_*
    const float *seed;  // learned seed (ne x k, stencil order, local units) or nullptr
    const int64_t *adj_ptr;  // ragged adjacency: neighbours of e at adjl[adj_ptr[e] ..], or nullptr
    int32_t *defer;          // FP32 paths: room for ne stencil indices that the split-row kernel
                             // hands to the general kernel (count in counters[7]), or nullptr
    const int32_t *slots;    // split-row kernel: the stencils to build (nslots of them; a size class
    int64_t nslots;          // of a batched build), or nullptr: stencils 0 .. ne-1
    // optional sliced-ELL copy of the rows (slices of 32 rows, entry j of row r at
    // sell_off[r / 32] + 32 j + r % 32; operator q's values at sell_val + q * sell_nnz)
    const int64_t *sell_off;
    int32_t *sell_col;
    double *sell_val;
    int64_t sell_nnz;
};

// Entry `rank` of row e into the sliced-ELL copy, when there is one.
__device__ __forceinline__ void sell_put(const StencilParams &P, int64_t e, int rank, int32_t c, int q, double v) {
    const int64_t p = P.sell_off[e >> 5] + 32 * (int64_t)rank + (e & 31);
    if (q == 0) P.sell_col[p] = c;
    P.sell_val[q * P.sell_nnz + p] = v;
}

// One size class (stencil size k, polynomial degree) of a batched build of uneven stencils.
struct BinDesc {
    StencilParams P;        // k, n, nmon and monomial exponents of the class; shared arrays
    const int32_t *slots;   // the class's stencils (eval point indices), count entries
    int64_t count;
    int64_t item_start;     // first work item of the class in the persistent kernel's queue
    int tile;               // 0: one warp per stencil (4 per block), 1: the block on one stencil
    int precision;          // RBF_PREC_FP64 or RBF_PREC_FP32_REFINED
};

// x * 2^e exactly, as ldexp gives it: when x and the result are normal numbers the exponent
// field moves on the integer pipe; zeros, subnormals, infinities, NaNs and results leaving the
// normal range take ldexp (on GB300 ldexp would otherwise cost several FP64-pipe instructions).
__device__ __forceinline__ double scale2(double x, int e) {
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex != 0 && ex != 0x7ff && ex + e > 0 && ex + e < 0x7ff) return __longlong_as_double(b + ((long long)e << 52));
    return ldexp(x, e);
}

// The exponent frexp gives for sqrt(x), x > 0, from x's bit pattern on the integer pipe:
// x = m 2^E with m in [0.5, 1) puts sqrt(x) in [2^((E-1)/2), 2^(E/2)), so the exponent is
// (E + 1) >> 1 (the correctly rounded root of the largest double below 2^E, E even, stays
// below 2^(E/2): sqrt(1 - u) < 1 - u/2).  Zero, subnormal and non-finite x take the library
// path.  (frexp(sqrt(x)) would cost an FP64 square root on GB300's FP64 pipe.)
__device__ __forceinline__ int sqrt_frexp_exponent(double x) {
    const long long b = __double_as_longlong(x);
    const int bexp = (int)((b >> 52) & 0x7ff);
    if (bexp == 0 || bexp == 0x7ff || b < 0) {
        int e = 0;
        if (x > 0.0) frexp(sqrt(x), &e);
        return e;
    }
    const int E = bexp - 1022;
    return (E + 1) >> 1;
}

template <class T> __device__ __forceinline__ T rbf_sqrt(T x);
template <> __device__ __forceinline__ double rbf_sqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float rbf_sqrt<float>(float x) { return sqrtf(x); }

// float -> double by rebuilding the bit pattern on the integer pipe (normal floats and
// zero; subnormal floats, far below any entry scale here, map to zero)
__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e == 0u) return 0.0;
    const unsigned long long bits = ((unsigned long long)(u >> 31) << 63) |
                                    ((unsigned long long)(e + 896u) << 52) |
                                    ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)bits);
}
// sqrt(s) by Newton's method (Heron) from the FP32 reciprocal square root of s's leading bits:
// r0 = s y0 (relative error e ~ 2^-22), then twice r <- r + (s - r^2) y0 / 2; the first step
// leaves ~1.5 e^2, the second ~e^3, below FP64 rounding.  Five FP64 operations against the
// library square root's longer sequence; within an ulp or two of the correctly rounded root.
// s below the FP32 normal range (coincident points) takes the library root.
__device__ __forceinline__ double sqrt_newton(double s) {
    const long long b = __double_as_longlong(s);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e <= 1023 - 120 || e >= 1023 + 120) return sqrt(s);
    const float sf = __uint_as_float(((unsigned)(e - 1023 + 127) << 23) | (unsigned)((b >> 29) & 0x7fffff));
    float yf;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(sf));
    const float hf = 0.5f * yf;
    const double y = widen(yf), h = widen(hf);
    double r = s * y;
    r = fma(h, fma(-r, r, s), r);
    return fma(h, fma(-r, r, s), r);
}

template <class T> __device__ __forceinline__ T pw3(T r) { return r * r * r; }
template <class T> __device__ __forceinline__ T pw5(T r) { return r * r * r * r * r; }

// phi(|D|) from the squared distance
template <class T> __device__ __forceinline__ T phs_phi_r2(int p, T r2) {
    T r = rbf_sqrt<T>(r2);
    switch (p) {
    case 1: return r;
    case 3: return r2 * r;
    case 5: return (r2 * r2) * r;
    default: return (r2 * r2 * r2) * r;
    }
}

template <class T> __device__ __forceinline__ T sq_norm(const T *D, int dim) {
    T s = D[0] * D[0];
    for (int d = 1; d < dim; d++) s += D[d] * D[d];
    return s;
}

// The reference guards divisions by r^b with r^b + 1e-16 (avoid_inf).  In local
// coordinates r = s*r_xi, so the guard of an r^b denominator is 1e-16 / s^b: with it every
// entry is exactly s^(power) times the raw-coordinate entry, including at r = 0.
template <class T> struct AvoidInf {
    T a1, a2, a3, a5;  // 1e-16 / s^b for b = 1, 2, 3, 5
};

template <class T> __device__ __forceinline__ AvoidInf<T> avoid_inf_scaled(int es) {
    AvoidInf<T> a;
    a.a1 = (T)scale2(RBF_AVOID_INF, -es);
    a.a2 = (T)scale2(RBF_AVOID_INF, -2 * es);
    a.a3 = (T)scale2(RBF_AVOID_INF, -3 * es);
    a.a5 = (T)scale2(RBF_AVOID_INF, -5 * es);
    return a;
}

// (op::L)(x, xi) with D = x - xi
template <class T> __device__ T phs_op(int p, int op, int od, const T *D, int dim, const AvoidInf<T> &A) {
    T r2 = sq_norm(D, dim);
    if (op == RBF_OP_IDENTITY) return phs_phi_r2<T>(p, r2);
    T r = rbf_sqrt<T>(r2);
    T dd = D[od];
    switch (p) {
    case 1:
        if (op == RBF_OP_PARTIAL1) return dd / (r + A.a1);
        if (op == RBF_OP_PARTIAL2) return (-(dd * dd) + r2) / (pw3(r) + A.a3);
        return (T)2 / (r + A.a1);
    case 3:
        if (op == RBF_OP_PARTIAL1) return (T)3 * dd * r;
        if (op == RBF_OP_PARTIAL2) return (T)3 * (r + (dd * dd) / (r + A.a1));
        return (T)12 * r;
    case 5:
        if (op == RBF_OP_PARTIAL1) return (T)5 * dd * pw3(r);
        if (op == RBF_OP_PARTIAL2) return (T)5 * r * ((T)3 * (dd * dd) + r2);
        return (T)30 * pw3(r);
    default:
        if (op == RBF_OP_PARTIAL1) return (T)7 * dd * pw5(r);
        if (op == RBF_OP_PARTIAL2) return (T)7 * pw3(r) * ((T)5 * (dd * dd) + r2);
        return (T)56 * pw5(r);
    }
}

// (op::L)(x, xi, n): the operator applied to the normal derivative in the second argument
template <class T>
__device__ T phs_op_normal(int p, int op, int od, const T *D, const T *n, int dim, const AvoidInf<T> &A) {
    T r2 = sq_norm(D, dim);
    T r = rbf_sqrt<T>(r2);
    T dd = D[od], nd = n[od];
    T dn = n[0] * D[0];
    for (int d = 1; d < dim; d++) dn += n[d] * D[d];
    switch (p) {
    case 1:
        if (op == RBF_OP_PARTIAL1) return -nd / (r + A.a1) + dn * dd / (pw3(r) + A.a3);
        if (op == RBF_OP_PARTIAL2) return ((T)2 * nd * dd + dn) / (pw3(r) + A.a3) - (T)3 * (dd * dd) * dn / (pw5(r) + A.a5);
        return (T)2 * dn / (pw3(r) + A.a3);
    case 3:
        if (op == RBF_OP_PARTIAL1) return (T)-3 * (nd * r + dn * dd / (r + A.a1));
        if (op == RBF_OP_PARTIAL2) return (T)-3 * ((T)2 * dd * nd + dn - dn * (dd * dd) / (r2 + A.a2)) / (r + A.a1);
        return (T)-12 * dn / (r + A.a1);
    case 5:
        if (op == RBF_OP_PARTIAL1) return (T)-5 * (nd * pw3(r) + (T)3 * dn * dd * r);
        if (op == RBF_OP_PARTIAL2) return (T)-5 * ((T)6 * nd * dd * r + (T)3 * dn * (r + (dd * dd) / (r + A.a1)));
        return (T)-90 * dn * r;
    default:
        if (op == RBF_OP_PARTIAL1) return (T)-7 * (nd * pw5(r) + (T)5 * pw3(r) * dd * dn);
        if (op == RBF_OP_PARTIAL2) return (T)-7 * ((T)10 * nd * dd * pw3(r) + (T)5 * dn * ((T)3 * r * (dd * dd) + pw3(r)));
        return (T)-280 * dn * pw3(r);
    }
}

// gradient / Hessian of phi in the first argument, D = x - xi
template <class T>
__device__ void phs_grad_hess(int p, const T *D, int dim, T *g, T *H, bool want_h, const AvoidInf<T> &A) {
    T r = rbf_sqrt<T>(sq_norm(D, dim));
    for (int i = 0; i < dim; i++) {
        switch (p) {
        case 1: g[i] = D[i] / (r + A.a1); break;
        case 3: g[i] = (T)3 * D[i] * r; break;
        case 5: g[i] = (T)5 * D[i] * pw3(r); break;
        default: g[i] = (T)7 * D[i] * pw5(r); break;
        }
    }
    if (!want_h) return;
    for (int i = 0; i < dim; i++)
        for (int j = 0; j < dim; j++) {
            T dl = (i == j) ? (T)1 : (T)0;
            T v;
            switch (p) {
            case 1: v = dl / (r + A.a1) - D[i] * D[j] / (pw3(r) + A.a3); break;
            case 3: v = (T)3 * (dl * r + D[i] * D[j] / (r + A.a1)); break;
            case 5: v = (T)5 * (dl * pw3(r) + (T)3 * D[i] * D[j] * r); break;
            default: v = (T)7 * (dl * pw5(r) + (T)5 * D[i] * D[j] * pw3(r)); break;
            }
            H[i * 3 + j] = v;
        }
}

// Collocation entry between stencil points i and j (upper-triangle rule of
// src/solve/assembly.jl:251-332; plain phi for interior stencils).
// xi, xj local coordinates; ti/tj point types; a*, b* = alpha and beta/s; n* normals.
template <class T>
__device__ T colloc_entry(int p, int dim, const T *xi, const T *xj, int ti, int tj, T ai_, T bi_,
                          const T *ni, T aj_, T bj_, const T *nj, const AvoidInf<T> &A) {
    T D[3];
    for (int d = 0; d < dim; d++) D[d] = xi[d] - xj[d];
    T phi = phs_phi_r2<T>(p, sq_norm(D, dim));
    if (ti != PT_NR && tj != PT_NR) return phi;
    T g[3], H[9];
    bool both = (ti == PT_NR && tj == PT_NR);
    phs_grad_hess<T>(p, D, dim, g, H, both, A);
    T di = 0, dj = 0;
    for (int d = 0; d < dim; d++) {
        di += ni[d] * g[d];
        dj += nj[d] * g[d];
    }
    if (!both) {
        if (tj == PT_NR) return aj_ * phi - bj_ * dj;
        return ai_ * phi + bi_ * di;
    }
    T d2 = 0;
    for (int a = 0; a < dim; a++) {
        T hn = 0;
        for (int b = 0; b < dim; b++) hn += H[a * 3 + b] * nj[b];
        d2 += ni[a] * hn;
    }
    return ai_ * aj_ * phi - ai_ * bj_ * dj + bi_ * aj_ * di + bi_ * bj_ * d2;
}

// value of monomial m at local point x
template <class T> __device__ __forceinline__ T mono_val(const StencilParams &P, int m, const T *x) {
    T v = (T)1;
    for (int d = 0; d < P.dim; d++)
        for (int t = 0; t < P.exps[m][d]; t++) v *= x[d];
    return v;
}

// first partial of monomial m in dimension d at x
template <class T> __device__ __forceinline__ T mono_d1(const StencilParams &P, int m, int dd, const T *x) {
    int e = P.exps[m][dd];
    if (e == 0) return (T)0;
    T v = (T)e;
    for (int d = 0; d < P.dim; d++) {
        int ed = P.exps[m][d] - (d == dd ? 1 : 0);
        for (int t = 0; t < ed; t++) v *= x[d];
    }
    return v;
}

// operator applied to monomial m at the local origin (the eval point)
__device__ __forceinline__ double mono_op_at_origin(const StencilParams &P, int m, int op, int od) {
    int e0 = P.exps[m][0], e1 = P.dim > 1 ? P.exps[m][1] : 0, e2 = P.dim > 2 ? P.exps[m][2] : 0;
    int tot = e0 + e1 + e2;
    int ed = P.exps[m][od];
    switch (op) {
    case RBF_OP_IDENTITY: return tot == 0 ? 1.0 : 0.0;
    case RBF_OP_PARTIAL1: return (tot == 1 && ed == 1) ? 1.0 : 0.0;
    case RBF_OP_PARTIAL2: return (tot == 2 && ed == 2) ? 2.0 : 0.0;
    default: return (tot == 2 && (e0 == 2 || e1 == 2 || e2 == 2)) ? 2.0 : 0.0;
    }
}

// normal derivative of monomial m at the local origin
__device__ __forceinline__ double mono_normal_at_origin(const StencilParams &P, int m, const double *n) {
    int tot = 0, which = -1;
    for (int d = 0; d < P.dim; d++) {
        tot += P.exps[m][d];
        if (P.exps[m][d] == 1) which = d;
    }
    return (tot == 1 && which >= 0) ? n[which] : 0.0;
}
