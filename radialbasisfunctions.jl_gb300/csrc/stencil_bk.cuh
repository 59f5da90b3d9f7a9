// Plain FP64 stencil solve by symmetric indefinite factorisation (Bunch-Kaufman LDL^T), one
// warp per stencil, the system packed in shared memory.
//
// The reference solves each stencil's saddle-point system [A P; P^T 0] with
// bunchkaufman!(Symmetric(A, :U), true) (src/solve/assembly.jl:220-222): a symmetric
// indefinite factorisation, n^3/3 flops.  On GB300 the FP64 pipe retires two lanes per SM
// cycle, so this path is bound by its FP64 instruction count, and the design minimises it:
//   * only the lower triangle is stored and updated (half of an LU's work), packed by rows;
//   * each elimination step spreads the trailing triangle's entries evenly over the 32 lanes
//     (one FMA per entry and lane slot, no lane holding a short row idle);
//   * pivot search and pivot decisions use integer keys and FP32 comparisons, the pivot
//     reciprocal an FP32 seed and two Newton steps (four FMAs instead of a division);
//   * the right-hand sides are eliminated with the matrix (forward substitution folded into
//     the steps); the back substitution with L^T runs one row of L per step.
// Pivoting follows Bunch and Kaufman's partial strategy (alpha = (1 + sqrt 17) / 8: a 1x1
// pivot on the diagonal, or on the largest off-diagonal entry's diagonal, or a 2x2 block);
// the reference's LAPACK routine uses the rook variant of the same strategy, so the two
// differ in pivot order and agree to within rounding.
#pragma once
#include "stencil_device.cuh"

namespace {

// Per-warp workspace: the packed system and the step vectors beside WarpSmem's stencil data.
struct BKSmem {
    WarpSmem w;        // X, HA, HB, HN (in the work area), cols, ptype (w.M unused)
    double *P;         // lower triangle, packed by rows: (i, j), i >= j, at pidx(i, j)
    double *B;         // right-hand sides, n x nops; on return the solution in pivot order
    double *l1, *l2;   // multipliers of the current step's pivot column(s), indexed by row
    double *w1, *w2;   // the pivot column(s) before scaling, indexed by row
    double *dinv;      // per step: the inverse of its pivot block (e11, e21, e22)
    double *sol;       // solution in the original unknown order, n x nops
    int *orig;         // original index of the unknown at each position
    int *blk;          // 1: 1x1 pivot at this position, 2: first row of a 2x2 block, 0: second row
};

// Work area shared by the phases: the stencil data (X, HA, HB, HN: 8k doubles) is read only by
// the assembly, the step vectors (l1, l2, w1, w2, dinv: 7n) only by the factorisation and
// the D solve, and the solution in the original order (n x nops) is written after both.
__host__ __device__ inline size_t bk_work_doubles(int n, int k, int nops) {
    size_t m = 8 * (size_t)k;
    m = m > 7 * (size_t)n ? m : 7 * (size_t)n;
    return m > (size_t)n * nops ? m : (size_t)n * nops;
}

__host__ __device__ inline size_t bk_warp_bytes(int n, int k, int nops) {
    const size_t d = (size_t)n * (n + 1) / 2 + (size_t)n * nops + bk_work_doubles(n, k, nops);
    const size_t i = 2 * (size_t)k + 2 * (size_t)n;
    return ((d * sizeof(double) + i * sizeof(int)) + 15) & ~(size_t)15;
}

__device__ inline BKSmem carve_bk(char *base, int n, int k, int nops) {
    BKSmem s;
    double *p = reinterpret_cast<double *>(base);
    s.P = p;
    p += (size_t)n * (n + 1) / 2;
    s.B = p;
    p += (size_t)n * nops;
    double *work = p;
    s.l1 = work;
    s.l2 = work + n;
    s.w1 = work + 2 * n;
    s.w2 = work + 3 * n;
    s.dinv = work + 4 * n;
    s.sol = work;
    s.w.M = nullptr;
    s.w.X = work;
    s.w.HA = work + 3 * k;
    s.w.HB = work + 4 * k;
    s.w.HN = work + 5 * k;
    int *ip = reinterpret_cast<int *>(work + bk_work_doubles(n, k, nops));
    s.w.cols = ip;
    s.w.ptype = ip + k;
    s.orig = ip + 2 * k;
    s.blk = ip + 2 * k + n;
    return s;
}

// Magnitude key of a matrix entry for a warp argmax (__reduce_max_sync): the high word of |v|
// (exponent and 20 mantissa bits, monotonic in |v|) with its low 7 bits replaced by 127 - idx,
// so that the largest magnitude wins and, within 2^-13 relative, the lowest index.  NaN and
// infinity give the largest keys (the caller then rejects the stencil).
__device__ __forceinline__ unsigned mag_key(double v, int idx) {
    const unsigned hi = (unsigned)__double2hiint(v) & 0x7fffffffu;
    return (hi & ~127u) | (unsigned)(127 - idx);
}

// FP32 value of |v| from its bits on the integer pipe (truncated mantissa; magnitudes below
// the FP32 normal range become 0, above it infinity): the pivot decisions compare these.
__device__ __forceinline__ float abs_f32(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    const int e = (int)(b >> 52);
    if (e >= 1023 + 128) return __int_as_float(0x7f800000);
    if (e <= 1023 - 127) return 0.0f;
    return __uint_as_float(((unsigned)(e - 1023 + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}

__device__ __forceinline__ bool finite64(double v) {
    return ((unsigned)__double2hiint(v) & 0x7ff00000u) != 0x7ff00000u;
}

// 1/d: the FP32 approximate reciprocal of d's leading bits, refined by two Newton steps
// r <- r + r (1 - d r) (each squares the relative error: ~2^-22 -> 2^-44 -> rounding level).
// Pivots outside the FP32 seed's range take the division.
__device__ __forceinline__ double recip64(double d) {
    const long long b = __double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023 - 120 || e > 1023 + 120) return 1.0 / d;
    const unsigned fb = ((unsigned)((unsigned long long)b >> 32) & 0x80000000u) | ((unsigned)(e - 1023 + 127) << 23) |
                        (unsigned)((b >> 29) & 0x7fffff);
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(__uint_as_float(fb)));
    double r = widen(rf);
    double t = fma(-d, r, 1.0);
    r = fma(r, t, r);
    t = fma(-d, r, 1.0);
    return fma(r, t, r);
}

// Symmetric interchange of positions p < q: rows and columns of the packed lower triangle (the
// computed columns of L included), the right-hand-side rows and the unknowns' bookkeeping.
__device__ void bk_swap(const BKSmem &s, int p, int q, int n, int nops, int lane) {
    double *P = s.P;
    for (int j = lane; j < p; j += 32) {  // (p, j) <-> (q, j), j < p
        const double a = P[pidx(p, j)];
        P[pidx(p, j)] = P[pidx(q, j)];
        P[pidx(q, j)] = a;
    }
    for (int j = p + 1 + lane; j < q; j += 32) {  // (j, p) <-> (q, j), p < j < q
        const double a = P[pidx(j, p)];
        P[pidx(j, p)] = P[pidx(q, j)];
        P[pidx(q, j)] = a;
    }
    for (int i = q + 1 + lane; i < n; i += 32) {  // (i, p) <-> (i, q), i > q
        const double a = P[pidx(i, p)];
        P[pidx(i, p)] = P[pidx(i, q)];
        P[pidx(i, q)] = a;
    }
    for (int t = lane; t < nops; t += 32) {
        const double a = s.B[p * nops + t];
        s.B[p * nops + t] = s.B[q * nops + t];
        s.B[q * nops + t] = a;
    }
    if (lane == 0) {
        const double a = P[pidx(p, p)];
        P[pidx(p, p)] = P[pidx(q, q)];
        P[pidx(q, q)] = a;
        const int o = s.orig[p];
        s.orig[p] = s.orig[q];
        s.orig[q] = o;
    }
}

// Rank-1 (TWO = false) or rank-2 update of the trailing triangle (i, j), k0 <= j <= i < n:
// A(i, j) -= l1(i) w1(j) [+ l2(i) w2(j)].  Entries are enumerated from the longest row
// (i = n - 1) upwards and dealt to the lanes round-robin, so every lane gets the same count
// (to within one) whatever the row lengths.
template <bool TWO>
__device__ __forceinline__ void bk_update(const BKSmem &s, int k0, int n, int lane) {
    double *P = s.P;
    int i = n - 1, len = n - k0, b = lane;
    while (len > 0 && b >= len) {
        b -= len;
        i--;
        len--;
    }
    while (len > 0) {
        const double a1 = s.l1[i];
        const double a2 = TWO ? s.l2[i] : 0.0;
        double *row = P + pidx(i, k0);
        const int rl = len;
        for (; b < rl; b += 32) {
            double v = row[b];
            v = fma(-a1, s.w1[k0 + b], v);
            if (TWO) v = fma(-a2, s.w2[k0 + b], v);
            row[b] = v;
        }
        b -= rl;
        i--;
        len--;
        while (len > 0 && b >= len) {
            b -= len;
            i--;
            len--;
        }
    }
}

// Factorise and solve the packed system of one stencil in place: on success s.sol holds the
// solution (n x nops) in the original unknown order.  Returns false if a pivot column is
// exactly zero or the system is not finite (the stencil is singular).
__device__ bool bk_solve(const BKSmem &s, int n, int nops, int lane) {
    constexpr float kAlpha = 0.6403882032022076f;  // (1 + sqrt(17)) / 8
    double *P = s.P, *B = s.B;
    for (int i = lane; i < n; i += 32) s.orig[i] = i;
    __syncwarp();
    for (int k = 0; k < n;) {
        // largest entry of column k below the diagonal
        unsigned key = 0u;
        for (int i = k + 1 + lane; i < n; i += 32) key = max(key, mag_key(P[pidx(i, k)], i));
        key = __reduce_max_sync(0xffffffffu, key);
        const int imax = 127 - (int)(key & 127u);
        const double akk = P[pidx(k, k)];
        const double cm = k + 1 < n ? P[pidx(imax, k)] : 0.0;
        if (!finite64(akk) || !finite64(cm)) return false;
        const float absakk = abs_f32(akk), colmax = abs_f32(cm);
        // a column below 2^-126 in an O(1)-scaled system (or exactly zero): singular
        if (absakk == 0.0f && colmax == 0.0f) return false;
        int kp = k, kstep = 1;
        if (absakk < kAlpha * colmax) {
            // largest off-diagonal entry of row imax within the trailing matrix
            unsigned rk = 0u;
            for (int j = k + lane; j < n; j += 32)
                if (j != imax) rk = max(rk, mag_key(j < imax ? P[pidx(imax, j)] : P[pidx(j, imax)], j));
            rk = __reduce_max_sync(0xffffffffu, rk);
            const int jmax = 127 - (int)(rk & 127u);
            const double rm = jmax < imax ? P[pidx(imax, jmax)] : P[pidx(jmax, imax)];
            if (!finite64(rm)) return false;
            const float rowmax = abs_f32(rm);
            if (absakk * rowmax >= kAlpha * colmax * colmax) {
                kp = k;
            } else if (abs_f32(P[pidx(imax, imax)]) >= kAlpha * rowmax) {
                kp = imax;
            } else {
                kp = imax;
                kstep = 2;
            }
        }
        const int kk = k + kstep - 1;
        __syncwarp();
        if (kp != kk) bk_swap(s, kk, kp, n, nops, lane);
        __syncwarp();
        if (kstep == 1) {
            const double d = P[pidx(k, k)];
            const double r = recip64(d);
            for (int i = k + 1 + lane; i < n; i += 32) {
                const double w = P[pidx(i, k)];
                s.w1[i] = w;
                s.l1[i] = w * r;
            }
            if (lane == 0) {
                s.dinv[3 * k] = r;
                s.dinv[3 * k + 1] = 0.0;
                s.dinv[3 * k + 2] = 0.0;
                s.blk[k] = 1;
            }
            __syncwarp();
            bk_update<false>(s, k + 1, n, lane);
            for (int t = lane; t < (n - k - 1) * nops; t += 32) {  // forward substitution of the RHS
                const int i = k + 1 + t / nops, q = t - (t / nops) * nops;
                B[i * nops + q] = fma(-s.l1[i], B[k * nops + q], B[i * nops + q]);
            }
            __syncwarp();
            for (int i = k + 1 + lane; i < n; i += 32) P[pidx(i, k)] = s.l1[i];
        } else {
            // 2x2 block D = [a b; b c] at (k, k+1), inverted as LAPACK's dsytf2 does it (scaled by
            // 1/b, which avoids overflow): d11 = c/b, d22 = a/b, d21 = (1/(d11 d22 - 1)) / b
            const double a = P[pidx(k, k)], bb = P[pidx(k + 1, k)], c = P[pidx(k + 1, k + 1)];
            const double ib = recip64(bb);
            const double d11 = c * ib, d22 = a * ib;
            const double d21 = recip64(fma(d11, d22, -1.0)) * ib;
            for (int i = k + 2 + lane; i < n; i += 32) {
                const double x1 = P[pidx(i, k)], x2 = P[pidx(i, k + 1)];
                s.w1[i] = x1;
                s.w2[i] = x2;
                s.l1[i] = d21 * fma(d11, x1, -x2);
                s.l2[i] = d21 * fma(d22, x2, -x1);
            }
            if (lane == 0) {
                s.dinv[3 * k] = d21 * d11;
                s.dinv[3 * k + 1] = -d21;
                s.dinv[3 * k + 2] = d21 * d22;
                s.blk[k] = 2;
                s.blk[k + 1] = 0;
            }
            __syncwarp();
            bk_update<true>(s, k + 2, n, lane);
            for (int t = lane; t < (n - k - 2) * nops; t += 32) {
                const int i = k + 2 + t / nops, q = t - (t / nops) * nops;
                B[i * nops + q] = fma(-s.l2[i], B[(k + 1) * nops + q], fma(-s.l1[i], B[k * nops + q], B[i * nops + q]));
            }
            __syncwarp();
            for (int i = k + 2 + lane; i < n; i += 32) {
                P[pidx(i, k)] = s.l1[i];
                P[pidx(i, k + 1)] = s.l2[i];
            }
            if (lane == 0) P[pidx(k + 1, k)] = 0.0;  // L is unit lower with a zero in the block
        }
        __syncwarp();
        k += kstep;
    }
    // D^-1, block by block
    for (int t = lane; t < n * nops; t += 32) {
        const int k = t / nops, q = t - (t / nops) * nops;
        const int bt = s.blk[k];
        if (bt == 1) {
            B[t] *= s.dinv[3 * k];
        } else if (bt == 2) {
            const double y0 = B[k * nops + q], y1 = B[(k + 1) * nops + q];
            B[k * nops + q] = fma(s.dinv[3 * k], y0, s.dinv[3 * k + 1] * y1);
            B[(k + 1) * nops + q] = fma(s.dinv[3 * k + 1], y0, s.dinv[3 * k + 2] * y1);
        }
    }
    __syncwarp();
    // L^T x = z from the bottom: once x_i is final, x_j -= L(i, j) x_i for j < i
    for (int i = n - 1; i > 0; i--) {
        const double *Li = P + pidx(i, 0);
        for (int t = lane; t < i * nops; t += 32) {
            const int j = t / nops, q = t - (t / nops) * nops;
            B[t] = fma(-Li[j], B[i * nops + q], B[t]);
        }
        __syncwarp();
    }
    // back to the original unknown order
    for (int t = lane; t < n * nops; t += 32) {
        const int j = t / nops, q = t - (t / nops) * nops;
        s.sol[s.orig[j] * nops + q] = B[t];
    }
    __syncwarp();
    return true;
}

// One stencil e on one warp, plain FP64 by Bunch-Kaufman: load, assemble (packed), factorise,
// solve, scatter (ND: the normal-derivative builds' instantiation).
template <bool ND = false>
__device__ void solve_fp64_bk_warp(const StencilParams &P, int64_t e, const BKSmem &s, int lane) {
    int es = 0, eval_local = -2;
    const int st = load_stencil(P, e, s.w, lane, &es, &eval_local);
    if (st != 0) {
        __syncwarp();
        return;
    }
    assemble_fp64_into<PackedStore, ND>(P, s.w, lane, es, eval_local, PackedStore{s.P, s.B, P.n, P.k + P.nnr, P.nops});
    if (!bk_solve(s, P.n, P.nops, lane)) {
        if (lane == 0) {
            if (P.status) P.status[e] = 1;
            atomicAdd(&P.counters[0], 1ull);
        }
        __syncwarp();
        return;
    }
    scatter_row(P, e, s.w, lane, es, s.sol, P.nops, 1);
    if (lane == 0 && P.status) P.status[e] = 0;
    __syncwarp();
}

}  // namespace
