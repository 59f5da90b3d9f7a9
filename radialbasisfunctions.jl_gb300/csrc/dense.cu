// Global interpolation on the device: Interpolator(x, y, basis) (src/interpolation.jl:22-37)
// and its evaluation (src/interpolation.jl:39-52).
//
// Fit.  The collocation matrix of all n points, [Φ P; Pᵀ 0] of order nt = n + nmon (upper
// triangle, column-major, as _build_collocation_matrix! fills it, src/solve/assembly.jl:95-115),
// is factorised by rook-pivoted Bunch-Kaufman (bunchkaufman!(A, true) -> LAPACK dsytrf_rook,
// UPLO = 'U') and solved.  The factorisation follows the unblocked dsytf2_rook step by step,
// one launch per column k = nt .. 1: every SM applies the rank-1 or rank-2 update of the
// current step to the leading upper triangle (the per-element arithmetic is LAPACK's, with
// the update's multiply-adds fused as optimised BLAS kernels evaluate them, so the factors
// equal the oracle's restatement in that form bit for bit) and the step's interchanges to the
// factor columns already computed (columns > k: the converted form of LAPACK's
// dsyconvf_rook, one row permutation kept in perm, which the blocked solve needs).  The
// pivot decisions are made on the device, so the whole factorisation is queued without a host
// sync: the block that owns the next pivot column updates it first and settles the common
// case (a 1x1 pivot without interchange depends on that column alone); the last block to
// finish (an atomic count, no waiting) writes the columns that must follow the update (the
// 1x1 scaling, the 2x2 multipliers) and otherwise runs the full rook search (block arg-max
// reductions, first index on ties as idamax).  A launch whose column a 2x2 pivot consumed
// does nothing.  Step records are double-buffered: a decision never overwrites the record
// that blocks of the running launch read.
//
// Roofline: each 1x1 step reads and writes the k(k-1)/2 entries of the leading triangle once
// (16 bytes and one FP64 FMA per entry); on GB300 the FP64 pipe and HBM give similar bounds
// (~0.5 T FMA/s vs ~7 TB/s / 16 B = 0.44 T entries/s), so the unblocked order costs little
// against a blocked one (which would be FP64-bound at the same rate) and keeps LAPACK's
// per-step rounding.
//
// Solve (converted form, A = P U D Uᵀ Pᵀ): b[perm], U⁻¹ by 64-column chunks from the bottom
// (one block for the chunk's triangle, every SM for the rows above), D⁻¹ (1x1 / 2x2 blocks as
// dsytrs_rook), U⁻ᵀ by chunks from the top, scatter through perm.
//
// Evaluation: one thread per eval point, the centres staged through shared memory in tiles;
// the RBF sum runs over the centres in order, then the monomial dot product, as the
// reference's loop (bit-identical to the oracle's evaluation).
#include <algorithm>
#include <climits>

#include "rbf_internal.cuh"

namespace {

constexpr int PIV_THREADS = 1024;
constexpr int SOLVE_CHUNK = 64;
constexpr double BK_ALPHA_NUM = 1.0;  // alpha = (1 + sqrt(17)) / 8 (dsytf2_rook)

#define A_(i, j) A[((int64_t)(j)-1) * lda + ((i)-1)]
// loads of the pivot decision, made by the last block of an update launch after the other
// blocks' writes: through L2 (never a line this SM cached earlier in the launch)
#define AG(i, j) __ldcg(&A_(i, j))

// one pivot step (dsytf2_rook): mode 0: 1x1, update with d11 = 1/A(k,k), then the column is
// scaled by d11; 1: 1x1 tiny pivot, the column already divided by d11 = A(k,k); 2: 2x2 (d11,
// d12, d22, t as dsytf2_rook, multipliers in wk / wkm1 / u / v); 3: no update
struct RookStep {
    int k, kstep, mode, nswap;
    int sw_a[2], sw_b[2];  // the step's interchanges, in order (1-based rows)
    double d11, d12, d22, t;
};

struct RookState {
    RookStep step[2];  // step[slot]: applied by the current launch; step[1 - slot]: the next one
    int slot;
    int spec;  // 1: the next step was decided during the current launch by its column's owner
    int info;  // first k with an exactly zero (or NaN) pivot column, 0 if none
    int err;   // 1: rook search did not terminate within its bound
};

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// block arg-max of |x| with idamax semantics: the first index of the largest value, NaNs
// never chosen; returns (index, value) to every thread; index INT_MAX if nothing qualifies
struct ArgMax {
    double v;
    int i;
};

__device__ __forceinline__ void am_merge(ArgMax &a, const ArgMax &b) {
    if (b.v > a.v || (b.v == a.v && b.i < a.i)) a = b;
}

__device__ ArgMax block_argmax(ArgMax a, ArgMax *red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        ArgMax b;
        b.v = __shfl_xor_sync(0xffffffffu, a.v, o);
        b.i = __shfl_xor_sync(0xffffffffu, a.i, o);
        am_merge(a, b);
    }
    __syncthreads();  // red may still be read from a previous call
    if (lane == 0) red[w] = a;
    __syncthreads();
    if (w == 0) {
        a = lane < (int)(blockDim.x >> 5) ? red[lane] : ArgMax{-1.0, INT_MAX};
        for (int o = 16; o > 0; o >>= 1) {
            ArgMax b;
            b.v = __shfl_xor_sync(0xffffffffu, a.v, o);
            b.i = __shfl_xor_sync(0xffffffffu, a.i, o);
            am_merge(a, b);
        }
        if (lane == 0) red[0] = a;
    }
    __syncthreads();
    return red[0];
}

// idamax over rows i0 .. i0+cnt-1 of column j (1-based result row, i0 if none qualifies)
__device__ int col_argmax(const double *A, int64_t lda, int i0, int cnt, int j, ArgMax *red) {
    ArgMax a{-1.0, INT_MAX};
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
        const double v = fabs(AG(i0 + t, j));
        if (v > a.v) a = ArgMax{v, t};
    }
    const ArgMax r = block_argmax(a, red);
    return i0 + (r.i == INT_MAX ? 0 : r.i);
}

// idamax over columns j0 .. j0+cnt-1 of row i (1-based result column)
__device__ int row_argmax(const double *A, int64_t lda, int i, int j0, int cnt, ArgMax *red) {
    ArgMax a{-1.0, INT_MAX};
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
        const double v = fabs(AG(i, j0 + t));
        if (v > a.v) a = ArgMax{v, t};
    }
    const ArgMax r = block_argmax(a, red);
    return j0 + (r.i == INT_MAX ? 0 : r.i);
}

__device__ __forceinline__ void swap_el(double *A, int64_t lda, int i1, int j1, int i2, int j2) {
    const double t = AG(i1, j1);
    A_(i1, j1) = AG(i2, j2);
    A_(i2, j2) = t;
}

// the column writes of step S that must follow its update (after every block has read the
// pivot columns): the 1x1 column scaling, the 2x2 multipliers
__device__ void finish_step(double *A, int64_t lda, const RookStep &S, const double *wk, const double *wkm1) {
    const int k = S.k;
    if (S.mode == 0) {
        for (int i = 1 + threadIdx.x; i <= k - 1; i += blockDim.x) A_(i, k) = dmul(S.d11, AG(i, k));
    } else if (S.mode == 2) {
        for (int j = 1 + threadIdx.x; j <= k - 2; j += blockDim.x) {
            A_(j, k) = wk[j - 1] / S.d12;
            A_(j, k - 1) = wkm1[j - 1] / S.d12;
        }
    }
    __syncthreads();
}

// One block: the pivot decision of column k (dsytf2_rook), its interchanges in the leading
// submatrix and what the update needs, recorded in *out for the update launch of column k.
__device__ __noinline__ void rook_decide(double *A, int64_t lda, int k, int32_t *ipiv, RookState *st, RookStep *out,
                                         int32_t *perm, double *wk, double *wkm1, double *u, double *v, ArgMax *red) {
    const double alpha = (BK_ALPHA_NUM + sqrt(17.0)) / 8.0;
    const double sfmin = 2.2250738585072014e-308;
    // ---- pivot decision (dsytf2_rook)
    const double absakk = fabs(AG(k, k));
    int imax = 0;
    double colmax = 0.0;
    if (k > 1) {
        imax = col_argmax(A, lda, 1, k - 1, k, red);
        colmax = fabs(AG(imax, k));
    }
    int kstep = 1, p = k, kp = k, mode = 3;
    bool zero_col = false;
    if (fmax(absakk, colmax) == 0.0 || isnan(absakk) || isnan(colmax)) {
        zero_col = true;
    } else if (!(absakk < alpha * colmax)) {
        kp = k;
    } else {
        int jmax = 0;
        bool done = false;
        // rowmax strictly grows along the search, which ends within k iterations
        for (int it = 0; it <= k + 1 && !done; it++) {
            double rowmax;
            if (imax != k) {
                jmax = row_argmax(A, lda, imax, imax + 1, k - imax, red);
                rowmax = fabs(AG(imax, jmax));
            } else {
                rowmax = 0.0;
            }
            if (imax > 1) {
                const int itemp = col_argmax(A, lda, 1, imax - 1, imax, red);
                const double dtemp = fabs(AG(itemp, imax));
                if (dtemp > rowmax) {
                    rowmax = dtemp;
                    jmax = itemp;
                }
            }
            if (!(fabs(AG(imax, imax)) < alpha * rowmax)) {
                kp = imax;
                done = true;
            } else if (p == jmax || rowmax <= colmax) {
                kp = imax;
                kstep = 2;
                done = true;
            } else {
                p = imax;
                colmax = rowmax;
                imax = jmax;
            }
        }
        if (!done) {  // cannot happen for finite input; keep the step harmless
            if (threadIdx.x == 0) st->err = 1;
            kp = k;
            kstep = 1;
            p = k;
        }
    }
    // ---- interchanges in the leading submatrix
    const int kq = k - kstep + 1;
    if (!zero_col) {
        if (kstep == 2 && p != k) {
            for (int t = 1 + threadIdx.x; t <= p - 1; t += blockDim.x) swap_el(A, lda, t, k, t, p);
            for (int t = 1 + threadIdx.x; t <= k - p - 1; t += blockDim.x) swap_el(A, lda, p + t, k, p, p + t);
            if (threadIdx.x == 0) swap_el(A, lda, k, k, p, p);
            __syncthreads();
        }
        if (kp != kq) {
            for (int t = 1 + threadIdx.x; t <= kp - 1; t += blockDim.x) swap_el(A, lda, t, kq, t, kp);
            if (kq > 1 && kp < kq - 1)
                for (int t = 1 + threadIdx.x; t <= kq - kp - 1; t += blockDim.x)
                    swap_el(A, lda, kp + t, kq, kp, kp + t);
            __syncthreads();
            if (threadIdx.x == 0) {
                swap_el(A, lda, kq, kq, kp, kp);
                if (kstep == 2) swap_el(A, lda, k - 1, k, kp, k);
            }
            __syncthreads();
        }
    }
    // ---- the pivot block and what the update needs
    double d11 = 0.0, d12 = 0.0, d22 = 0.0, tt = 0.0;
    if (!zero_col) {
        if (kstep == 1) {
            if (k > 1) {
                const double akk = AG(k, k);
                if (fabs(akk) >= sfmin) {
                    mode = 0;
                    d11 = 1.0 / akk;
                } else {
                    mode = 1;
                    d11 = akk;
                    for (int i = 1 + threadIdx.x; i <= k - 1; i += blockDim.x) A_(i, k) = AG(i, k) / d11;
                }
            }
        } else if (k > 2) {
            mode = 2;
            d12 = AG(k - 1, k);
            d22 = AG(k - 1, k - 1) / d12;
            d11 = AG(k, k) / d12;
            tt = 1.0 / dsub(dmul(d11, d22), 1.0);
            for (int j = 1 + threadIdx.x; j <= k - 2; j += blockDim.x) {
                const double ajkm1 = AG(j, k - 1), ajk = AG(j, k);
                wkm1[j - 1] = dmul(tt, dsub(dmul(d11, ajkm1), ajk));
                wk[j - 1] = dmul(tt, dsub(dmul(d22, ajk), ajkm1));
                u[j - 1] = ajk / d12;
                v[j - 1] = ajkm1 / d12;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (zero_col && __ldcg(&st->info) == 0) st->info = k;
        int ns = 0;
        if (!zero_col) {
            if (kstep == 2 && p != k) {
                out->sw_a[ns] = k;
                out->sw_b[ns] = p;
                ns++;
            }
            if (kp != kq) {
                out->sw_a[ns] = kq;
                out->sw_b[ns] = kp;
                ns++;
            }
        }
        for (int s = 0; s < ns; s++) {
            const int a = out->sw_a[s] - 1, b = out->sw_b[s] - 1;
            const int32_t t = perm[a];
            perm[a] = perm[b];
            perm[b] = t;
        }
        out->nswap = ns;
        out->k = k;
        out->kstep = kstep;
        out->mode = mode;
        out->d11 = d11;
        out->d12 = d12;
        out->d22 = d22;
        out->t = tt;
        if (kstep == 1) {
            ipiv[k - 1] = kp;
        } else {
            ipiv[k - 1] = -p;
            ipiv[k - 2] = -kp;
        }
    }
    __syncthreads();
}

// The common case of the next decision, made by the block that owns column k while the other
// blocks still update: a 1x1 pivot without interchange (|A(k,k)| >= alpha * colmax) depends
// on column k alone.  Anything else (a zero column, the rook search) is left to the last
// block.  Returns whether *out now holds the step.
__device__ __noinline__ bool rook_speculate(double *A, int64_t lda, int k, int32_t *ipiv, RookStep *out, ArgMax *red) {
    __shared__ bool s_ok;
    const double alpha = (BK_ALPHA_NUM + sqrt(17.0)) / 8.0;
    const double sfmin = 2.2250738585072014e-308;
    const double absakk = fabs(AG(k, k));
    int imax = 0;
    double colmax = 0.0;
    if (k > 1) {
        imax = col_argmax(A, lda, 1, k - 1, k, red);
        colmax = fabs(AG(imax, k));
    }
    if (fmax(absakk, colmax) == 0.0 || isnan(absakk) || isnan(colmax) || absakk < alpha * colmax) return false;
    int mode = 3;
    double d11 = 0.0;
    if (k > 1) {
        const double akk = AG(k, k);
        if (fabs(akk) >= sfmin) {
            mode = 0;
            d11 = 1.0 / akk;
        } else {
            mode = 1;
            d11 = akk;
            for (int i = 1 + threadIdx.x; i <= k - 1; i += blockDim.x) A_(i, k) = AG(i, k) / d11;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        out->k = k;
        out->kstep = 1;
        out->mode = mode;
        out->nswap = 0;
        out->d11 = d11;
        out->d12 = out->d22 = out->t = 0.0;
        ipiv[k - 1] = k;
        s_ok = true;
    }
    __syncthreads();
    return s_ok;
}

__global__ void __launch_bounds__(PIV_THREADS) rook_pivot_kernel(double *A, int64_t lda, int k, int32_t *ipiv,
                                                                 RookState *st, int32_t *perm, double *wk,
                                                                 double *wkm1, double *u, double *v) {
    __shared__ ArgMax red[32];
    rook_decide(A, lda, k, ipiv, st, &st->step[0], perm, wk, wkm1, u, v, red);
}

// The update of step kk: rank-1 / rank-2 update of the leading upper triangle (one column per
// block at a time, each block's columns largest first) and the step's interchanges applied to
// the factor columns kk+1..nt (the converted form).  The block that owns the next pivot column
// updates it first and decides the next step when the common case allows; the last block to
// finish (an atomic count, no waiting) writes this step's columns and makes the decision
// otherwise.
constexpr int UPD_THREADS = 256;
constexpr int UPD_UNROLL = 4;

__global__ void __launch_bounds__(UPD_THREADS, 6) rook_step_kernel(double *A, int64_t lda, int kk, int nt, int32_t *ipiv,
                                                                   RookState *st, int32_t *perm, double *wk,
                                                                   double *wkm1, double *u, double *v,
                                                                   unsigned int *count) {
    __shared__ ArgMax red[32];
    __shared__ bool s_last;
    const int slot = st->slot;
    const RookStep *S = &st->step[slot];
    if (S->k != kk) return;
    const int k = kk, mode = S->mode, next = k - S->kstep;
    const int nb = gridDim.x, bid = blockIdx.x;
    RookStep *nxt = &st->step[1 - slot];
    bool spec = next >= 1 && bid == (next - 1) % nb;
    const int hi = mode == 0 || mode == 1 ? k - 1 : (mode == 2 ? k - 2 : 0);
    if (bid + 1 <= hi) {
        const double *colk = &A_(1, k);
        for (int j = bid + 1 + ((hi - bid - 1) / nb) * nb; j >= 1; j -= nb) {
            double *colj = &A_(1, j);
            if (mode == 2) {
                const double a = wk[j - 1], b = wkm1[j - 1];
                for (int i = threadIdx.x; i < j; i += blockDim.x) colj[i] = __fma_rn(-v[i], b, __fma_rn(-u[i], a, colj[i]));
            } else {
                const double xj = colk[j - 1];
                if (xj != 0.0) {
                    const double temp = dmul(-S->d11, xj);
                    for (int i0 = threadIdx.x; i0 < j; i0 += UPD_UNROLL * UPD_THREADS) {
                        double c[UPD_UNROLL], x[UPD_UNROLL];
#pragma unroll
                        for (int q = 0; q < UPD_UNROLL; q++) {
                            const int i = i0 + q * UPD_THREADS;
                            if (i < j) {
                                c[q] = colj[i];
                                x[q] = colk[i];
                            }
                        }
#pragma unroll
                        for (int q = 0; q < UPD_UNROLL; q++) {
                            const int i = i0 + q * UPD_THREADS;
                            if (i < j) colj[i] = __fma_rn(x[q], temp, c[q]);
                        }
                    }
                }
            }
            if (spec && j == next) {
                __syncthreads();
                if (rook_speculate(A, lda, next, ipiv, nxt, red) && threadIdx.x == 0) {
                    __threadfence();
                    st->spec = 1;
                }
                spec = false;
            }
        }
    }
    if (spec) {  // the owner had no column to update (a step without update)
        __syncthreads();
        if (rook_speculate(A, lda, next, ipiv, nxt, red) && threadIdx.x == 0) {
            __threadfence();
            st->spec = 1;
        }
    }
    const int ns = S->nswap;
    if (ns) {
        const int a0 = S->sw_a[0], b0 = S->sw_b[0], a1 = S->sw_a[1], b1 = S->sw_b[1];
        const int64_t tid = (int64_t)bid * blockDim.x + threadIdx.x, nth = (int64_t)nb * blockDim.x;
        for (int64_t j = k + 1 + tid; j <= nt; j += nth) {
            swap_el(A, lda, a0, (int)j, b0, (int)j);
            if (ns > 1) swap_el(A, lda, a1, (int)j, b1, (int)j);
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(count, 1u) == (unsigned)nb - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    finish_step(A, lda, *S, wk, wkm1);
    if (next >= 1 && __ldcg(&st->spec) == 0) rook_decide(A, lda, next, ipiv, st, nxt, perm, wk, wkm1, u, v, red);
    if (threadIdx.x == 0) {
        st->spec = 0;
        st->slot = 1 - slot;
        *count = 0;
    }
}

__global__ void rook_init_kernel(RookState *st, int nt, int32_t *perm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        RookState s = {};
        *st = s;
    }
    for (int64_t i = t; i < nt; i += (int64_t)gridDim.x * blockDim.x) perm[i] = (int32_t)i;
}

// ---- solve in the converted form ----------------------------------------------------------
// 2x2 structure from ipiv: blk[k-1] = 1 for the upper row k of a 2x2 pivot block (k-1, k),
// whose A(k-1, k) is D's off-diagonal entry and not part of U
__global__ void rook_blocks_kernel(const int32_t *ipiv, int nt, int8_t *blk) {
    // sequential: pivot types are decided from the top (k = nt) down
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int k = nt;
    while (k >= 1) {
        if (ipiv[k - 1] > 0 || k == 1) {
            blk[k - 1] = 0;
            k -= 1;
        } else {
            blk[k - 1] = 1;
            blk[k - 2] = 2;
            k -= 2;
        }
    }
}

// the row permutation of the converted factor from ipiv: every step's interchanges in order
__global__ void rook_perm_kernel(const int32_t *ipiv, int nt, int32_t *perm) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int i = 0; i < nt; i++) perm[i] = i;
    int k = nt;
    while (k >= 1) {
        if (ipiv[k - 1] > 0 || k == 1) {
            const int kp = ipiv[k - 1] > 0 ? ipiv[k - 1] : k;
            if (kp != k) {
                const int32_t t = perm[k - 1];
                perm[k - 1] = perm[kp - 1];
                perm[kp - 1] = t;
            }
            k -= 1;
        } else {
            const int p = -ipiv[k - 1], kp = -ipiv[k - 2];
            if (p != k) {
                const int32_t t = perm[k - 1];
                perm[k - 1] = perm[p - 1];
                perm[p - 1] = t;
            }
            if (kp != k - 1) {
                const int32_t t = perm[k - 2];
                perm[k - 2] = perm[kp - 1];
                perm[kp - 1] = t;
            }
            k -= 2;
        }
    }
}

__global__ void ipiv_check_kernel(const int32_t *ipiv, int nt, int *bad) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += (int64_t)gridDim.x * blockDim.x) {
        const int v = ipiv[i] < 0 ? -ipiv[i] : ipiv[i];
        if (v < 1 || v > nt) atomicOr(bad, 1);
    }
}

__global__ void gather_kernel(const double *b, const int32_t *perm, int nt, double *y) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = b[perm[i]];
}

__global__ void scatter_kernel(const double *z, const int32_t *perm, int nt, double *x) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += (int64_t)gridDim.x * blockDim.x)
        x[perm[i]] = z[i];
}

// U entry (i, k) of the unit upper factor (1-based), zero for D's off-diagonal entries
__device__ __forceinline__ double u_entry(const double *A, int64_t lda, const int8_t *blk, int i, int k) {
    return (i == k - 1 && blk[k - 1] == 1) ? 0.0 : A_(i, k);
}

// back substitution, chunk [c0, c1]: the chunk's triangle on one block
__global__ void usolve_tri_kernel(const double *A, int64_t lda, const int8_t *blk, int c0, int c1, double *y) {
    for (int k = c1; k >= c0; k--) {
        const double yk = y[k - 1];
        for (int i = c0 + threadIdx.x; i <= k - 1; i += blockDim.x) y[i - 1] -= u_entry(A, lda, blk, i, k) * yk;
        __syncthreads();
    }
}

// rows 1 .. c0-1 minus the chunk's columns
__global__ void usolve_gemv_kernel(const double *A, int64_t lda, const int8_t *blk, int c0, int c1, double *y) {
    __shared__ double yc[SOLVE_CHUNK];
    for (int t = threadIdx.x; t <= c1 - c0; t += blockDim.x) yc[t] = y[c0 - 1 + t];
    __syncthreads();
    for (int i = 1 + blockIdx.x * blockDim.x + threadIdx.x; i <= c0 - 1; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = c0; k <= c1; k++) s += u_entry(A, lda, blk, i, k) * yc[k - c0];
        y[i - 1] -= s;
    }
}

// D^-1 (dsytrs_rook's 1x1 and 2x2 block solves)
__global__ void dsolve_kernel(const double *A, int64_t lda, const int8_t *blk, int nt, double *y) {
    for (int k = 1 + blockIdx.x * blockDim.x + threadIdx.x; k <= nt; k += gridDim.x * blockDim.x) {
        if (blk[k - 1] == 0) {
            y[k - 1] = (1.0 / A_(k, k)) * y[k - 1];
        } else if (blk[k - 1] == 1) {
            const double akm1k = A_(k - 1, k);
            const double akm1 = A_(k - 1, k - 1) / akm1k;
            const double ak = A_(k, k) / akm1k;
            const double denom = akm1 * ak - 1.0;
            const double bkm1 = y[k - 2] / akm1k, bk = y[k - 1] / akm1k;
            y[k - 2] = (ak * bkm1 - bk) / denom;
            y[k - 1] = (akm1 * bk - bkm1) / denom;
        }
    }
}

// forward substitution with U^T, chunk [c0, c1]: partial dots over rows < c0, one block per column
__global__ void ltsolve_dots_kernel(const double *A, int64_t lda, const int8_t *blk, int c0, int c1, const double *z,
                                    double *part) {
    __shared__ double red[32];
    const int k = c0 + blockIdx.x;
    if (k > c1) return;
    double s = 0.0;
    for (int i = 1 + threadIdx.x; i <= c0 - 1; i += blockDim.x) s += u_entry(A, lda, blk, i, k) * z[i - 1];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) part[k - c0] = s;
    }
}

__global__ void ltsolve_tri_kernel(const double *A, int64_t lda, const int8_t *blk, int c0, int c1, const double *part,
                                   double *z) {
    // one warp: z(k) -= part(k) + sum_{c0 <= i < k} U(i,k) z(i), k ascending
    const int lane = threadIdx.x & 31;
    if (threadIdx.x >= 32) return;
    for (int k = c0; k <= c1; k++) {
        double s = 0.0;
        for (int i = c0 + lane; i <= k - 1; i += 32) s += u_entry(A, lda, blk, i, k) * z[i - 1];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) z[k - 1] -= part[k - c0] + s;
        __syncwarp();
    }
}

// ---- assembly and evaluation ----------------------------------------------------------------
struct MonoTable {
    int nmon, dim;
    int8_t e[RBF_MAX_SYSTEM][3];
};

__device__ __forceinline__ double sqeuc(const double *a, const double *b, int dim) {
    double s = 0.0;
    for (int d = 0; d < dim; d++) {
        const double t = dsub(a[d], b[d]);
        s = dadd(s, dmul(t, t));
    }
    return s;
}

__device__ __forceinline__ double phi_r2(int p, double r2) {
    const double r = sqrt(r2);
    switch (p) {
    case 1: return r;
    case 3: return dmul(r2, r);
    case 5: return dmul(dmul(r2, r2), r);
    default: return dmul(dmul(dmul(r2, r2), r2), r);
    }
}

__device__ __forceinline__ double mono_prod(const MonoTable &M, int m, const double *x) {
    double v = 1.0;
    for (int d = 0; d < M.dim; d++)
        for (int t = 0; t < M.e[m][d]; t++) v = dmul(v, x[d]);
    return v;
}

__global__ void interp_assemble_kernel(const double *x, int n, int phs, MonoTable M, double *A, int64_t lda) {
    const int nt = n + M.nmon, dim = M.dim;
    // column j (1-based) on one block; rows i <= j
    for (int j = 1 + blockIdx.x; j <= nt; j += gridDim.x) {
        if (j <= n) {
            double xj[3];
            for (int d = 0; d < dim; d++) xj[d] = x[(int64_t)(j - 1) * dim + d];
            for (int i = 1 + threadIdx.x; i <= j; i += blockDim.x) {
                double xi[3];
                for (int d = 0; d < dim; d++) xi[d] = x[(int64_t)(i - 1) * dim + d];
                A_(i, j) = phi_r2(phs, sqeuc(xi, xj, dim));
            }
        } else {
            const int m = j - n - 1;
            for (int i = 1 + threadIdx.x; i <= j; i += blockDim.x) {
                double v = 0.0;
                if (i <= n) {
                    double xi[3];
                    for (int d = 0; d < dim; d++) xi[d] = x[(int64_t)(i - 1) * dim + d];
                    v = mono_prod(M, m, xi);
                }
                A_(i, j) = v;
            }
        }
    }
}

constexpr int EVAL_TILE = 256;

__global__ void __launch_bounds__(EVAL_TILE) interp_eval_kernel(const double *x, int n, int phs, MonoTable M,
                                                                 const double *coef, const double *xe, int64_t m,
                                                                 double *out) {
    __shared__ double sx[EVAL_TILE * 3];
    __shared__ double sw[EVAL_TILE];
    const int dim = M.dim;
    const int64_t nblk_pts = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < m; base += nblk_pts) {
        const int64_t t = base + threadIdx.x;
        double p[3] = {0.0, 0.0, 0.0};
        if (t < m)
            for (int d = 0; d < dim; d++) p[d] = xe[t * dim + d];
        double rbf = 0.0;
        for (int c0 = 0; c0 < n; c0 += EVAL_TILE) {
            const int cnt = min(EVAL_TILE, n - c0);
            __syncthreads();
            for (int q = threadIdx.x; q < cnt * dim; q += blockDim.x) sx[q] = x[(int64_t)c0 * dim + q];
            for (int q = threadIdx.x; q < cnt; q += blockDim.x) sw[q] = coef[c0 + q];
            __syncthreads();
            for (int i = 0; i < cnt; i++) rbf = dadd(rbf, dmul(sw[i], phi_r2(phs, sqeuc(p, &sx[i * dim], dim))));
        }
        if (t < m) {
            double poly = 0.0;
            for (int q = 0; q < M.nmon; q++) poly = dadd(poly, dmul(coef[n + q], mono_prod(M, q, p)));
            out[t] = dadd(rbf, poly);
        }
    }
}

#undef A_

}  // namespace

// ---- host-side drivers --------------------------------------------------------------------------
int rbf_sytrf_rook_device(rbf_ctx *ctx, int nt, double *dA, int64_t lda, int32_t *dipiv, int32_t *dperm,
                          int64_t *info) {
    if (nt == 0) {
        *info = 0;
        return RBF_OK;
    }
    DevBuf st, scratch;
    RBF_TRY(st.alloc(ctx, sizeof(RookState) + 16));
    RBF_TRY(scratch.alloc(ctx, sizeof(double) * 4 * (size_t)nt));
    double *wk = scratch.as<double>(), *wkm1 = wk + nt, *u = wkm1 + nt, *v = u + nt;
    RookState *s = st.as<RookState>();
    unsigned int *count = reinterpret_cast<unsigned int *>(s + 1);
    RBF_CUDA(ctx, cudaMemsetAsync(count, 0, sizeof(unsigned int), ctx->stream));
    rook_init_kernel<<<std::max(1, std::min(ctx->num_sms * 4, (nt + 255) / 256)), 256, 0, ctx->stream>>>(s, nt, dperm);
    rook_pivot_kernel<<<1, PIV_THREADS, 0, ctx->stream>>>(dA, lda, nt, dipiv, s, dperm, wk, wkm1, u, v);
    RBF_CHECK_LAUNCH(ctx);
    // one wave of resident blocks: the columns are dealt round-robin, no second wave's tail
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rook_step_kernel, UPD_THREADS, 0));
    const int maxb = ctx->num_sms * std::max(1, per_sm);
    for (int k = nt; k >= 1; k--) {
        // one block per column of the leading triangle (grid-stride), at least one block,
        // which makes the next decision
        const int nb = std::max(1, std::min(maxb, k - 1));
        rook_step_kernel<<<nb, UPD_THREADS, 0, ctx->stream>>>(dA, lda, k, nt, dipiv, s, dperm, wk, wkm1, u, v, count);
    }
    RBF_CHECK_LAUNCH(ctx);
    RookState h;
    RBF_CUDA(ctx, cudaMemcpyAsync(&h, s, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h.err) return rbf_fail(ctx, RBF_ERR_INTERNAL, "rook pivot search did not terminate");
    *info = h.info;
    return RBF_OK;
}

int rbf_sytrs_rook_device(rbf_ctx *ctx, int nt, const double *dA, int64_t lda, const int32_t *dipiv,
                          const int32_t *dperm, const double *db, double *dx) {
    if (nt == 0) return RBF_OK;
    DevBuf blk, work, pbuf;
    if (!dperm) {
        RBF_TRY(pbuf.alloc(ctx, sizeof(int32_t) * (size_t)nt));
        rook_perm_kernel<<<1, 1, 0, ctx->stream>>>(dipiv, nt, pbuf.as<int32_t>());
        dperm = pbuf.as<int32_t>();
    }
    RBF_TRY(blk.alloc(ctx, (size_t)nt));
    RBF_TRY(work.alloc(ctx, sizeof(double) * ((size_t)nt + SOLVE_CHUNK)));
    int8_t *b8 = blk.as<int8_t>();
    double *y = work.as<double>(), *part = y + nt;
    const int g = std::max(1, std::min(ctx->num_sms * 4, (nt + 255) / 256));
    rook_blocks_kernel<<<1, 1, 0, ctx->stream>>>(dipiv, nt, b8);
    gather_kernel<<<g, 256, 0, ctx->stream>>>(db, dperm, nt, y);
    for (int c1 = nt; c1 >= 1; c1 -= SOLVE_CHUNK) {
        const int c0 = std::max(1, c1 - SOLVE_CHUNK + 1);
        usolve_tri_kernel<<<1, 64, 0, ctx->stream>>>(dA, lda, b8, c0, c1, y);
        if (c0 > 1) {
            const int gb = std::max(1, std::min(ctx->num_sms * 4, (c0 - 1 + 255) / 256));
            usolve_gemv_kernel<<<gb, 256, 0, ctx->stream>>>(dA, lda, b8, c0, c1, y);
        }
    }
    dsolve_kernel<<<g, 256, 0, ctx->stream>>>(dA, lda, b8, nt, y);
    for (int c0 = 1; c0 <= nt; c0 += SOLVE_CHUNK) {
        const int c1 = std::min(nt, c0 + SOLVE_CHUNK - 1);
        if (c0 > 1) {
            ltsolve_dots_kernel<<<c1 - c0 + 1, 256, 0, ctx->stream>>>(dA, lda, b8, c0, c1, y, part);
        } else {
            RBF_CUDA(ctx, cudaMemsetAsync(part, 0, sizeof(double) * SOLVE_CHUNK, ctx->stream));
        }
        ltsolve_tri_kernel<<<1, 32, 0, ctx->stream>>>(dA, lda, b8, c0, c1, part, y);
    }
    scatter_kernel<<<g, 256, 0, ctx->stream>>>(y, dperm, nt, dx);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_check_ipiv_device(rbf_ctx *ctx, int nt, const int32_t *dipiv, bool *ok) {
    DevBuf flag;
    RBF_TRY(flag.alloc(ctx, sizeof(int)));
    RBF_CUDA(ctx, cudaMemsetAsync(flag.ptr, 0, sizeof(int), ctx->stream));
    const int g = std::max(1, std::min(ctx->num_sms * 4, (nt + 255) / 256));
    ipiv_check_kernel<<<g, 256, 0, ctx->stream>>>(dipiv, nt, flag.as<int>());
    RBF_CHECK_LAUNCH(ctx);
    int h = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&h, flag.ptr, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *ok = h == 0;
    return RBF_OK;
}

static MonoTable mono_table(int dim, int nmon, const int8_t (*exps)[3]) {
    MonoTable M = {};
    M.nmon = nmon;
    M.dim = dim;
    for (int m = 0; m < nmon; m++)
        for (int d = 0; d < 3; d++) M.e[m][d] = exps[m][d];
    return M;
}

int rbf_interp_assemble_device(rbf_ctx *ctx, int dim, int phs, int nmon, const int8_t (*exps)[3], const double *dx,
                               int n, double *dA, int64_t lda) {
    const MonoTable M = mono_table(dim, nmon, exps);
    const int nt = n + M.nmon;
    if (nt == 0) return RBF_OK;
    interp_assemble_kernel<<<std::min(nt, ctx->num_sms * 8), 256, 0, ctx->stream>>>(dx, n, phs, M, dA, lda);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_interp_eval_device(rbf_ctx *ctx, int dim, int phs, int nmon, const int8_t (*exps)[3], const double *dx, int n,
                           const double *dcoef, const double *dxe, int64_t m, double *dout) {
    const MonoTable M = mono_table(dim, nmon, exps);
    if (m == 0) return RBF_OK;
    const int64_t blocks = std::min<int64_t>((m + EVAL_TILE - 1) / EVAL_TILE, (int64_t)ctx->num_sms * 16);
    interp_eval_kernel<<<(unsigned)blocks, EVAL_TILE, 0, ctx->stream>>>(dx, n, phs, M, dcoef, dxe, m, dout);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}
