/*
 * rbffd.h -- C ABI of the GB300 (sm_103a) local RBF-FD library.
 *
 * One shared library (librbffd_gb300.so) exposes the hot path of
 * RadialBasisFunctions.jl's local RBF-FD operators as plain C entry points:
 * k-nearest-neighbour stencils, per-stencil assembly + dense solve, scatter into
 * sparse rows (CSR), and the sparse apply.  Every entry point returns an int status
 * (RBF_OK = 0, negative = error; the message is in rbf_last_error()).
 *
 * Pointers: every array argument may be a host pointer (pageable or pinned) or a
 * device pointer of the context's GPU; the library detects which and copies host
 * data through the context's stream.  Calls are stream-ordered on the context's
 * stream and return after the result is complete (host outputs are written, device
 * outputs are ready to use on that stream).
 *
 * Indices are 0-based int32 (point counts < 2^31).  Points are AoS doubles
 * (dim values per point, the memory layout of Vector{SVector{dim,Float64}}).
 */
#ifndef RBFFD_H
#define RBFFD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define RBF_OK 0
#define RBF_ERR_ARGUMENT -1        /* ArgumentError in the reference              */
#define RBF_ERR_DIMENSION -2       /* DimensionMismatch in the reference          */
#define RBF_ERR_CUDA -3            /* CUDA runtime error                          */
#define RBF_ERR_SINGULAR -4        /* a stencil system is exactly singular        */
#define RBF_ERR_UNSUPPORTED -5     /* combination not supported (e.g. no normal form) */
#define RBF_ERR_NOT_FOUND -6       /* Hermite eval point absent from its stencil  */
#define RBF_ERR_INTERNAL -7

/* ---- operator and precision vocabulary ----------------------------------- */
enum rbf_op_code {
    RBF_OP_IDENTITY = 0,  /* Regrid()(basis) = basis           (operators/regridding.jl:7)  */
    RBF_OP_PARTIAL1 = 1,  /* Partial(1, dim) / one entry of Jacobian (operators/partial.jl) */
    RBF_OP_PARTIAL2 = 2,  /* Partial(2, dim)                                                */
    RBF_OP_LAPLACIAN = 3  /* Laplacian()                       (operators/laplacian.jl:7)   */
};

enum rbf_precision {
    RBF_PREC_FP64 = 0,          /* plain FP64 solve (the oracle-matched drop-in)            */
    RBF_PREC_FP32_REFINED = 1,  /* FP32 factor + FP64-residual iterative refinement         */
    RBF_PREC_LEARNED = 2        /* learned seed + FP32 refinement, FP64 fallback            */
};

#define RBF_MAX_OPS 8
#define RBF_MAX_STENCIL 64   /* k <= 64 */
#define RBF_MAX_SYSTEM 80    /* k + nmon <= 80 */

/* Build configuration: basis, augmentation, the operators that share one
 * factorisation (one right-hand side each), and the solve precision. */
typedef struct rbf_build_cfg {
    int32_t dim;                  /* 1, 2 or 3                                      */
    int32_t phs;                  /* PHS order: 1, 3, 5 or 7                        */
    int32_t poly_deg;             /* -1 (none) .. 4                                 */
    int32_t nops;                 /* 1 .. RBF_MAX_OPS                               */
    int32_t op_code[RBF_MAX_OPS]; /* enum rbf_op_code                               */
    int32_t op_dim[RBF_MAX_OPS];  /* 0-based dimension of partial derivatives       */
    int32_t precision;            /* enum rbf_precision                             */
    int32_t refine_steps;         /* max refinement steps for FP32 paths (0: default 6) */
    double tol;                   /* FP32 paths: accept when the correction computed from the
                                     FP64 residual is below tol relative to the weights
                                     (0: default 1e-9); otherwise the FP64 solve is used */
    int32_t flags;                /* RBF_FLAG_* bits                                 */
    const float *seed;            /* RBF_PREC_LEARNED: predicted weights, ne x k floats in
                                     stencil order and local units (device pointer); the
                                     starting point of the refinement where the register
                                     kernels serve the system size (3k >= n), otherwise
                                     unused (the first FP32 solve reaches the same error
                                     floor from any start)                            */
    /* Optional sliced-ELL copy written by the build next to the CSR (device pointers;
       all of them or none): sell_slice_off from rbf_sell_offsets on this build's row_ptr,
       room for sell_nnz columns and nops * sell_nnz values (operator q's at
       sell_val + q * sell_nnz).  rbf_spmv_sell applies it.                          */
    const int64_t *sell_slice_off;
    int32_t *sell_col;
    double *sell_val;
    int64_t sell_nnz;
} rbf_build_cfg;

/* flags */
#define RBF_FLAG_STENCIL_ORDER 1  /* write each row in stencil (adjl) order, not column order */
#define RBF_FLAG_LOCAL_UNITS 2    /* weights in the stencil's local units: w * s^q, s the power of
                                     two above the stencil radius, q the operator order */
#define RBF_FLAG_FP64_LU 4        /* RBF_PREC_FP64 in rbf_build: solve by LU with partial pivoting
                                     (the batched build's solver, bit-identical to it) instead of
                                     the default symmetric indefinite (Bunch-Kaufman) LDL^T */
#define RBF_FLAG_NORMAL_DOF 8     /* rbf_build_batched with a Hermite boundary: the augmented
                                     (Hermite-Birkhoff) formulation, no counterpart in the
                                     reference.  Every Neumann/Robin stencil point carries two
                                     unknowns, u and du/dn (outward normal): the system of a
                                     stencil with m such neighbours is k + m + nmon.  Rows: a
                                     Dirichlet eval point keeps its identity row; every other row
                                     holds the operator's weights on u at its k points (columns =
                                     data indices) and on du/dn at its m Neumann/Robin points
                                     (column ns + b, b the point's boundary ordinal), k + m
                                     entries, columns ascending.  The operator has ns + nb
                                     columns: apply it to [u; du/dn at the boundary points].
                                     Neumann/Robin eval points take the operator itself (not the
                                     boundary condition).  PHS 3, 5 and 7 (r has no normal
                                     derivative at r = 0).  Row layout from
                                     rbf_build_count_normal_dof. */

/* Hermite boundary description (src/solve/types.jl:18-42,178-182).  Boundary
 * conditions are B u = alpha*u + beta*du/dn; Dirichlet is (1,0), Neumann (0,1).
 * alpha/beta/normals are indexed by boundary ordinal (the i-th point with
 * is_boundary set), as the reference's global_to_boundary map does. */
typedef struct rbf_hermite {
    const uint8_t *is_boundary; /* one flag per data point                          */
    const double *alpha;        /* n_boundary                                       */
    const double *beta;         /* n_boundary                                       */
    const double *normals;      /* n_boundary x dim (AoS)                           */
    int64_t n_boundary;
} rbf_hermite;

/* Per-build statistics (optional output). */
typedef struct rbf_build_stats {
    int64_t n_stencils;      /* eval rows solved (Dirichlet identity rows excluded) */
    int64_t n_identity_rows; /* Dirichlet eval rows                                 */
    int64_t n_fallback;      /* FP32 paths: stencils that fell back to the FP64 solve */
    int64_t n_singular;      /* stencils with an exactly singular system            */
    double max_residual;     /* FP32 paths: largest accepted relative correction (error
                                estimate of the accepted weights)                      */
    float ms_knn, ms_build, ms_total;
    int64_t n_residuals;     /* FP32 paths: FP64 residual evaluations over all stencils  */
    double seed_rel_err_mean; /* RBF_PREC_LEARNED: mean over seeded stencils of
                                 min(1, |x1 - seed| / |x1|), x1 the weights after the first
                                 FP32 solve -- the seed's error as judged by the solver   */
} rbf_build_stats;

typedef struct rbf_ctx rbf_ctx;

/* ---- context -------------------------------------------------------------- */
/* Create a context on CUDA device `device` with its own non-blocking stream.
 * Replaces the reference's device keyword / KernelAbstractions backend
 * (src/operators/operators.jl:117-126, src/solve/execution.jl:140-148). */
int rbf_ctx_create(int device, rbf_ctx **out);
int rbf_ctx_destroy(rbf_ctx *ctx);
/* Run on a caller-owned cudaStream_t (e.g. the stream of a Julia task or a torch
 * stream); NULL restores the context's own stream.  The legacy default stream is
 * selected by its handle cudaStreamLegacy ((void *)1).  A caller whose buffers are
 * allocated and freed in stream order on another stream (a caching allocator) must
 * bind that stream here: the library does not order its work against other streams. */
int rbf_ctx_set_stream(rbf_ctx *ctx, void *cuda_stream);
/* Benchmark hook: with timing on, rbf_knn and rbf_spmm record CUDA events around their
 * device work (staging copies excluded) and rbf_ctx_last_ms returns its duration. */
int rbf_ctx_set_timing(rbf_ctx *ctx, int32_t on);
int rbf_ctx_last_ms(rbf_ctx *ctx, float *ms);
const char *rbf_last_error(const rbf_ctx *ctx);
const char *rbf_version(void);

/* ---- k nearest neighbours ------------------------------------------------- */
/* Replaces find_neighbors(data, eval_points, k), src/utils.jl:12-18
 * (NearestNeighbors.KDTree + knn(tree, eval, k, true)).  idx_out is ne x k
 * (row-major), each row sorted by ascending distance, exact ties broken by the
 * smaller point index (self first when eval == data). */
int rbf_knn(rbf_ctx *ctx, const double *data, int64_t ns, const double *eval, int64_t ne,
            int32_t dim, int32_t k, int32_t *idx_out);

/* ---- weight build ---------------------------------------------------------- */
/* Exact row layout of the sparse weights: row_ptr_out[ne+1] (int64, 0-based) and
 * the total number of stored entries.  Interior and Neumann/Robin eval rows hold
 * k entries, Dirichlet eval rows hold 1 (src/solve/execution.jl:16-69).
 * herm may be NULL (no boundary). */
int rbf_build_count(rbf_ctx *ctx, int64_t ns, int64_t ne, int32_t k, const rbf_hermite *herm,
                    int64_t *row_ptr_out, int64_t *nnz_out);

/* Build the weights of cfg->nops operators on the stencils adjl (ne x k, 0-based).
 * Replaces _build_weights(ℒ, data, eval_points, adjl, basis; device)
 * (src/solve/api.jl:26-35, and its Hermite twin api.jl:167-196) down to
 * build_weights_kernel (src/solve/execution.jl:128-174).  The result is
 * cfg->nops CSR matrices (ne x ns) sharing one structure: row_ptr (from
 * rbf_build_count), col[nnz] with columns ascending within each row, and
 * val[op * nnz + p].  status_out (optional, ne int8): 0 solved, 1 singular,
 * 2 Dirichlet identity row, 3 solved by the FP64 fallback of an FP32 path.
 * Returns RBF_ERR_SINGULAR if any stencil is singular (the reference raises
 * from bunchkaufman!, src/solve/assembly.jl:220-222). */
int rbf_build(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns,
              const double *eval, int64_t ne, const int32_t *adjl, int32_t k,
              const rbf_hermite *herm, const int64_t *row_ptr, int32_t *col, double *val,
              int8_t *status_out, rbf_build_stats *stats);

/* A built operator whose device arrays the library allocated (rbf_build_csr): cfg->nops CSR
 * matrices ne x ns sharing one structure, row_ptr[ne + 1], col[nnz] (columns ascending within
 * each row) and val[op * nnz + p].  Release it with rbf_csr_free. */
typedef struct rbf_csr {
    int64_t ne, ns, nnz;
    int32_t nops;
    int64_t *row_ptr;
    int32_t *col;
    double *val;
} rbf_csr;

/* rbf_build_count, the allocation of the arrays on the context's device, and rbf_build in one
 * call: the boundary in the form that returns its own sparse matrix, as _build_weights does
 * (src/solve/api.jl:26-35, 167-196).  Arguments and status as rbf_build; on an error nothing
 * stays allocated and *out is zeroed. */
int rbf_build_csr(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns,
                  const double *eval, int64_t ne, const int32_t *adjl, int32_t k,
                  const rbf_hermite *herm, int8_t *status_out, rbf_build_stats *stats, rbf_csr *out);
/* Frees the arrays of an rbf_build_csr result and zeroes *csr (a zeroed csr is a no-op). */
int rbf_csr_free(rbf_ctx *ctx, rbf_csr *csr);

/* Reverse-mode sensitivities of a build with respect to the point positions: given the
 * cotangent dW of the built values (val layout: dW[op * nnz + p], the row_ptr / column
 * order of the forward rbf_build with the same cfg->flags), writes ddata (ns x dim) and
 * deval (ne x dim) = the gradients of L = sum(dW .* val).  With eval == NULL the eval
 * points are the data points and the full gradient is ddata + deval.  Replaces the
 * pullback of _build_weights (src/solve/ad_shared.jl:63-157 with the stencil rules of
 * src/solve/backward.jl:31-222: backward_linear_solve!, backward_collocation!,
 * backward_rhs!).  Supports PHS 1/3/5/7, the identity, first partials and the Laplacian,
 * interior stencils (no Hermite rows; every row holds k entries), up to RBF_MAX_OPS / 2
 * operators.  Each stencil system is re-assembled and solved once for the weights and the
 * adjoint together: cfg->precision RBF_PREC_FP64 factorises in FP64; otherwise an FP32
 * factorisation is refined with FP64 residuals to cfg->tol (default 1e-11, relative) with the
 * FP64 solve as fallback, as the refined build does. */
int rbf_build_backward(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns,
                       const double *eval, int64_t ne, const int32_t *adjl, int32_t k,
                       const int64_t *row_ptr, const double *dW, double *ddata, double *deval);

/* ---- global interpolation ------------------------------------------------------ */
/* Interpolator(x, y, basis) (src/interpolation.jl:22-37): the weights of the global RBF
 * interpolant of the n points x (AoS, dim doubles each) with values y.  The collocation
 * matrix of all points, [Phi P; P^T 0] of order nt = n + nmon (nmon = C(dim + poly_deg,
 * dim)), is assembled on the device (8 nt^2 bytes of device memory), factorised by rook
 * Bunch-Kaufman and solved; coef (nt doubles) receives the RBF weights then the monomial
 * weights (rbf_weights, monomial_weights).  RBF_ERR_SINGULAR if a pivot is exactly zero
 * (bunchkaufman!(A, true) raises). */
int rbf_interp_fit(rbf_ctx *ctx, int32_t dim, int32_t phs, int32_t poly_deg, const double *x,
                   int64_t n, const double *y, double *coef);

/* (rbfi::Interpolator)(x) for m points xe (src/interpolation.jl:39-52): out[t] =
 * sum_i coef[i] phi(xe_t, x_i) + sum_q coef[n + q] p_q(xe_t). */
int rbf_interp_eval(rbf_ctx *ctx, int32_t dim, int32_t phs, int32_t poly_deg, const double *x,
                    int64_t n, const double *coef, const double *xe, int64_t m, double *out);

/* The dense symmetric-indefinite factorisation the interpolator uses, for any symmetric
 * matrix: bunchkaufman!(Symmetric(A, :U), true) -> LAPACK dsytrf_rook (UPLO = 'U'), the
 * same pivots and per-entry arithmetic as the unblocked dsytf2_rook (its rank-1 / rank-2
 * updates as fused multiply-adds, as optimised BLAS kernels evaluate them).  On return A
 * holds U and D as dsytrf_rook leaves them, except that each step's interchanges are also
 * applied to the factor columns computed before it (the form LAPACK's dsyconvf_rook
 * produces with WAY = 'C'; the 2x2 blocks of D stay in place); ipiv is LAPACK's rook ipiv
 * (1-based, negative for 2x2 blocks).  info > 0: D(info, info) is exactly zero. */
int rbf_sytrf_rook(rbf_ctx *ctx, int64_t n, double *A, int64_t lda, int32_t *ipiv, int64_t *info);

/* Solve A X = B (nrhs columns, leading dimension ldb, overwritten) with the factors of
 * rbf_sytrf_rook (ldiv! of the BunchKaufman object, LAPACK dsytrs_rook's result). */
int rbf_sytrs_rook(rbf_ctx *ctx, int64_t n, int32_t nrhs, const double *A, int64_t lda,
                   const int32_t *ipiv, double *B, int64_t ldb);

/* ---- apply ------------------------------------------------------------------ */
/* Y = alpha * W X + beta * Y for nf fields, W the op_index-th operator of a built
 * CSR (ne x ns).  Replaces _eval_op / mul! (src/operators/operators.jl:217-218,
 * 529-542).  layout 0: column-major (field f of X at X[f*ldx + i], the layout of a
 * Julia Matrix); layout 1: interleaved (X[i*ldx + f]).  beta == 0 ignores Y. */
int rbf_spmm(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *row_ptr, const int32_t *col,
             const double *val, int32_t nf, int32_t layout, const double *X, int64_t ldx,
             double alpha, double beta, double *Y, int64_t ldy);

/* Transpose a built CSR (ne x ns) into CSC form: col_ptr_out[ns+1], row_out[nnz],
 * val_out[nnz] -- the SparseMatrixCSC layout the reference returns
 * (src/solve/execution.jl:105-115).  Rows within a column are ascending. */
int rbf_csr_to_csc(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *row_ptr,
                   const int32_t *col, const double *val, int64_t *col_ptr_out,
                   int32_t *row_out, double *val_out);

/* Operator algebra on built weights (operators of the same data and stencils share
 * row_ptr / col; every array a device pointer):
 *   rbf_weights_axpby: out = alpha * a + beta * b entry-wise over nnz values (b may be
 *     NULL: out = alpha * a) -- op1 + op2, op1 - op2, alpha * op, op / alpha, -op on
 *     RadialBasisOperator (src/operators/operator_algebra.jl:245-295, _combine_weights /
 *     _scale_weights, :307-309 and :288-289).
 *   rbf_weights_directional: out = sum_i v_i * W_i over the nd gradient value arrays of one
 *     Jacobian build (operator i at val + i * nnz); v: nd doubles (constant direction,
 *     per_row = 0) or ne * nd (one direction per row, per_row = 1) --
 *     _combine_directional_weights (src/operators/directional.jl:69-82).
 * Products and sums are rounded separately, in the reference's evaluation order. */
int rbf_weights_axpby(rbf_ctx *ctx, int64_t nnz, double alpha, const double *a, double beta,
                      const double *b, double *out);
int rbf_weights_directional(rbf_ctx *ctx, int64_t ne, const int64_t *row_ptr, int32_t nd,
                            const double *val, int64_t nnz, const double *v, int32_t per_row,
                            double *out);

/* Sliced-ELL copy of one operator, for operators applied many times (the time-stepping
 * use of _eval_op / mul!, src/operators/operators.jl:217-218, 529-542; same product, a
 * different memory layout).  Slices of 32 rows; inside slice s, entry j of row r sits at
 * slice_off[s] + 32 j + (r - 32 s) for j below the slice's longest row (shorter rows are
 * padded with column 0, value 0).  On GB300 the CSR apply of a locality-ordered operator
 * is bound by the FP64 pipe (cross-lane reductions, padding); the sliced apply does one
 * FMA per entry with fully coalesced loads.  Device pointers only.
 *   rbf_sell_offsets: slice_off[ceil(ne/32) + 1] from a CSR row_ptr; *sell_nnz = the
 *                     sliced entry count (slice_off[last]; = nnz for equal row lengths).
 *   rbf_sell_from_csr: fill sell_col[sell_nnz], sell_val[sell_nnz] from the CSR.
 *   rbf_spmv_sell: y = alpha * W x + beta * y (beta == 0 ignores y). */
int rbf_sell_offsets(rbf_ctx *ctx, int64_t ne, const int64_t *row_ptr, int64_t *slice_off,
                     int64_t *sell_nnz);
int rbf_sell_from_csr(rbf_ctx *ctx, int64_t ne, const int64_t *row_ptr, const int32_t *col,
                      const double *val, const int64_t *slice_off, int32_t *sell_col,
                      double *sell_val);
int rbf_spmv_sell(rbf_ctx *ctx, int64_t ne, const int64_t *slice_off, const int32_t *sell_col,
                  const double *sell_val, const double *x, double alpha, double beta, double *y);

/* The sliced copy in a locality order, for operators on unordered points applied many times
 * (the same product as _eval_op / mul!, src/operators/operators.jl:217-218, 529-542).  The
 * caller's point order stays the operator's interface; inside, the rows sit in the order
 * row_at (slice s holds rows row_at[32 s .. 32 s + 31]) and each column is replaced by its
 * position in the order col_at, so that rows applied together gather nearby x values.  The
 * orders are permutations, e.g. the Morton orders rbf_reorder_points returns for the eval and
 * the data points (the same array when eval == data).  Device pointers only.
 *   rbf_sell_offsets_perm: slice_off[ceil(ne/32) + 1] over the rows in the order row_at.
 *   rbf_sell_from_csr_perm: fill sell_col / sell_val from the CSR (each row's entries in CSR
 *     order; row_at and col_at are range-checked).
 *   rbf_spmv_sell_perm: y = alpha * W x + beta * y with x and y in the caller's order; x_work
 *     (ns doubles, not aliasing x) receives x in the order col_at; row_at and col_at must be the
 *     arrays the copy was made with. */
int rbf_sell_offsets_perm(rbf_ctx *ctx, int64_t ne, const int64_t *row_ptr, const int32_t *row_at, int64_t *slice_off,
                          int64_t *sell_nnz);
int rbf_sell_from_csr_perm(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *row_ptr, const int32_t *col,
                           const double *val, const int32_t *row_at, const int32_t *col_at, const int64_t *slice_off,
                           int32_t *sell_col, double *sell_val);
int rbf_spmv_sell_perm(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *slice_off, const int32_t *sell_col,
                       const double *sell_val, const int32_t *row_at, const int32_t *col_at, const double *x,
                       double *x_work, double alpha, double beta, double *y);

/* ---- learned stencil surrogate (no counterpart in the reference) ------------ */
/* Kernels of the MLP that predicts stencil weights (training and inference run on
 * them).  All arrays are device pointers; bf16 matrices are row-major with leading
 * dimensions that are multiples of 8 and 16-byte aligned rows.
 * rbf_mlp_gemm: C = A * B^T (+ bias), A M x K, B N x K, K a multiple of 32, FP32
 * accumulation on the tensor cores; epi 0: none, 1: GELU, 2: multiply by GELU'(aux);
 * writes any of Zf (FP32 before the epilogue), Cf (FP32), Cb (bf16). */
int rbf_mlp_gemm(rbf_ctx *ctx, int32_t M, int32_t N, int32_t K, const void *A, int32_t lda, const void *B,
                 int32_t ldb, const float *bias, int32_t epi, const float *aux, int32_t ldaux, float *Cf,
                 int32_t ldcf, void *Cb, int32_t ldcb, float *Zf, int32_t ldz);
int rbf_mlp_transpose(rbf_ctx *ctx, int32_t rows, int32_t cols, const void *in, int32_t ldi, void *out,
                      int32_t ldo);
int rbf_mlp_to_bf16(rbf_ctx *ctx, int32_t rows, int32_t cols, int32_t pad_cols, const float *in, int32_t ldi,
                    void *out, int32_t ldo);
/* network inputs: for every stencil the k offsets x_i - x0 (stencil order) divided by the
 * power of two s >= the stencil radius (the solver's local units), bf16, row stride ldo.
 * data holds n_data points; an adjl entry outside [0, n_data) is an RBF_ERR_ARGUMENT. */
int rbf_mlp_features(rbf_ctx *ctx, const double *data, int64_t n_data, const double *eval, int32_t dim,
                     const int32_t *adjl, int64_t ne, int32_t k, void *out, int32_t ldo);
/* The same product on the 5th-generation tensor cores (tcgen05.mma, accumulators in tensor
 * memory): C = act(A * B^T + bias), act GELU (gelu_on) or identity, exactly one of Cf (FP32)
 * or Cb (bf16) with row stride ldc (16-byte aligned rows), bias (optional) 16-byte aligned.
 * K a multiple of 32.  Used for the surrogate's inference. */
int rbf_mlp_gemm_tc(rbf_ctx *ctx, int32_t M, int32_t N, int32_t K, const void *A, int32_t lda, const void *B,
                    int32_t ldb, const float *bias, int32_t gelu_on, float *Cf, void *Cb, int32_t ldc);
/* *failed = 1 if a tensor-core GEMM since the last call gave up waiting on its pipeline
 * (its output is then incomplete); synchronises the context's stream. */
int rbf_mlp_tc_status(rbf_ctx *ctx, int32_t *failed);
/* Self-test of the tensor-core GEMM's bounded waits: one small launch (M = 256, N = 32,
 * K = 64) whose producer issues no copy and whose waits give up after 4096 polls, so that
 * the timeout path runs with nothing in flight: the block raises its abort flag, frees its
 * tensor memory and returns.  *failed receives the error flag that launch left (1 means the
 * timeout was detected and reported); an error flag left by an earlier GEMM stays set for
 * the next rbf_mlp_tc_status. */
int rbf_mlp_tc_selftest_timeout(rbf_ctx *ctx, int32_t *failed);
/* mean squared error over rows x cols and its gradient (bf16, zero in the padding) */
int rbf_mlp_mse(rbf_ctx *ctx, int32_t rows, int32_t cols, const float *Y, int32_t ldy, const float *T,
                int32_t ldt, void *dY, int32_t ldd, int32_t pad_cols, float *loss);
int rbf_mlp_colsum(rbf_ctx *ctx, int32_t rows, int32_t cols, const void *in, int32_t ldi, float *out);
/* Adam step (t = step >= 1) on FP32 parameters; p_bf16 (optional) receives their bf16 copy */
int rbf_mlp_adam(rbf_ctx *ctx, int64_t n, float *p, const float *g, float *m, float *v, float lr, float b1,
                 float b2, float eps, int32_t step, void *p_bf16);

/* ---- locality reordering ------------------------------------------------------ */
/* Replaces reorder_points!(x, k) (src/utils.jl:45-55, a SymRCM ordering of the stencil
 * graph): a permutation perm_out[n] with x_new[i] = x[perm_out[i]] that orders the points
 * along a Morton curve over a grid of about two points per cell (within a cell by original
 * index), so that stencils gather nearby entries in the apply.  data_out (optional, n x
 * dim) receives the permuted points. */
int rbf_reorder_points(rbf_ctx *ctx, const double *data, int64_t n, int32_t dim, int32_t *perm_out,
                       double *data_out);

/* ---- batched build of uneven stencils (no counterpart in the reference) ------ */
/* Ragged stencils: the neighbours of eval point e are adj_idx[adj_ptr[e] .. adj_ptr[e+1])
 * (adj_ptr[0] = 0, 1 <= length <= RBF_MAX_STENCIL, ne + 1 entries), first entry the
 * nearest as find_neighbors orders them.  rbf_build_count_ragged is rbf_build_count for
 * them (Dirichlet eval rows hold 1 entry, every other row its stencil's length). */
int rbf_build_count_ragged(rbf_ctx *ctx, int64_t ns, int64_t ne, const int64_t *adj_ptr,
                           const rbf_hermite *herm, int64_t *row_ptr_out, int64_t *nnz_out);
/* Row layout of a RBF_FLAG_NORMAL_DOF build of ragged stencils: a Dirichlet eval row holds
 * 1 entry, every other row its stencil's length plus the number of its Neumann/Robin
 * neighbours (their du/dn columns). */
int rbf_build_count_normal_dof(rbf_ctx *ctx, int64_t ns, int64_t ne, const int64_t *adj_ptr,
                               const int32_t *adj_idx, const rbf_hermite *herm, int64_t *row_ptr_out,
                               int64_t *nnz_out);
/* Builds every stencil of a ragged batch in one persistent launch.  Stencils are binned
 * by size class (stencil length k, polynomial degree: system size n = k + nmon) and each
 * class runs with the tile shape the autotuner chose for it: one warp per stencil, or the
 * whole 128-thread block on one stencil.  poly_deg_per (optional, ne entries in -1..6)
 * overrides cfg->poly_deg per stencil.  precision: RBF_PREC_FP64 or RBF_PREC_FP32_REFINED.
 * tune: 0 cached choices (a heuristic for classes never tuned), 1 autotune the classes
 * not tuned yet (timing both tiles on up to 16384 stencils of each class with at least
 * 1024), 2 re-tune every class.  Output layout and errors as rbf_build. */
int rbf_build_batched(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns,
                      const double *eval, int64_t ne, const int64_t *adj_ptr, const int32_t *adj_idx,
                      const int8_t *poly_deg_per, const rbf_hermite *herm, const int64_t *row_ptr,
                      int32_t *col, double *val, int8_t *status_out, rbf_build_stats *stats,
                      int32_t tune);
/* The context's tuning table, one line per size class (tile chosen and trial times). */
int rbf_tuning_report(rbf_ctx *ctx, char *buf, int64_t len);

/* ---- build -> apply in one CUDA graph (no counterpart in the reference) ------ */
/* A time loop over moving points (update_weights! then the operator call,
 * src/operators/operators.jl:589-602, 217-218) re-builds the weights on fixed stencils and
 * applies them every step.  A plan captures that pair -- counter reset, build kernel, SpMV
 * y = W[op_index] x -- once into a CUDA graph on device buffers fixed at creation (every
 * pointer must be a device pointer; row_ptr from rbf_build_count, uniform stencils, no
 * boundary, precision FP64 or FP32-refined).  rbf_plan_launch enqueues the graph on the
 * context's stream; coordinates in data/eval and the field x may be rewritten in place
 * between launches.  rbf_plan_counters reads the last launch's singular / fallback /
 * FP64-residual counts (synchronising the stream). */
typedef struct rbf_plan rbf_plan;
int rbf_plan_create(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns,
                    const double *eval, int64_t ne, const int32_t *adjl, int32_t k,
                    const int64_t *row_ptr, int32_t *col, double *val, int32_t op_index,
                    const double *x, double *y, rbf_plan **out);
int rbf_plan_launch(rbf_plan *plan);
int rbf_plan_counters(rbf_plan *plan, int64_t *singular, int64_t *fallback, int64_t *residuals);
int rbf_plan_destroy(rbf_plan *plan);

/* ---- allocation-free apply (no counterpart in the reference) ---------------- */
/* Same contract as rbf_spmm, for callers that cannot allocate device memory while
 * applying an operator (code inside another framework's memory pool, or a time-stepping
 * loop that must stay off the allocator).  Every array must be a device pointer; nothing
 * is staged or allocated.  The column-major multi-field case (layout 0, nf > 1) stages
 * X and Y through one fixed 32 MiB device array that the library holds on every GPU it is
 * loaded on until exit: it is rejected (RBF_ERR_ARGUMENT) when nf*(ns+ne) exceeds
 * 4,194,304 doubles.  The first call on a device looks up that array's address (set-up
 * once per device); make that first call before any stream capture.  All calls share the
 * array, so calls that overlap on the GPU race; each call overwrites what it reads.  Like
 * every entry point it returns after its work on the context's stream is complete; with
 * rbf_ctx_set_timing on, rbf_ctx_last_ms gives its device time. */
int rbf_spmm_noalloc(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *row_ptr, const int32_t *col,
                     const double *val, int32_t nf, int32_t layout, const double *X, int64_t ldx,
                     double alpha, double beta, double *Y, int64_t ldy);

/* ---- diagnostics (no counterpart in the reference) ------------------------ */
/* Measured FMA throughput of the context's GPU in TFLOP/s (fp64 != 0: FP64,
 * else FP32), used as the roofline denominator of the build kernels. */
int rbf_diag_fma_peak(rbf_ctx *ctx, int32_t fp64, double *tflops);
/* Number of kernels this context has launched so far. */
int64_t rbf_ctx_kernel_launches(const rbf_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* RBFFD_H */
