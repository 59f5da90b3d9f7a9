// Split-row register refined build for systems of 33..40 rows with one operator (the
// k = 30, degree-2 stencils of the 3D workloads: 40 x 40 systems).
//
// The register kernel of stencil_refined_reg.cuh gives every lane two full rows, so for
// n = 40 the second row slot holds real rows in 8 lanes only: 80 registers of matrix per
// lane, a third of the elimination FMAs on padding, and (with the full FP64 system of
// 13 KB per warp in shared memory) 12 resident warps per SM.  Here
//   * rows 0..31 ("main" rows) stay one per lane, in registers;
//   * rows 32..n-1 ("extra" rows) are cut into 4 pieces of ceil(n/4) columns, and lane
//     l holds piece l & 3 of extra row 32 + (l >> 2): 50 registers of matrix for n = 40,
//     every lane doing useful work in the extra-row updates;
//   * the FP64 system in shared memory is the packed lower triangle (A is symmetric) and
//     the right-hand side: 6.9 KB instead of 13.1 KB per warp;
//   * interior stencils only.  Stencils with a boundary point (Hermite rows) and the rare
//     stencil whose refinement fails go to a list that the general refined kernel
//     (FP32 factor, FP64 refinement, FP64 fallback) finishes in a second launch.
// Together: 16 resident warps per SM.  The FP32 factorisation is a Gauss-Jordan inversion
// (pivot choice by magnitude, ties to the lower row, as the register kernel's LU; the rows
// not yet used as pivots evolve exactly as in the LU), run as one rolled loop over the steps
// with each row a shifting register window, so the code stays small and every solve of the
// refinement is one product with the inverse instead of two serial substitutions.
// Multipliers of an extra row reach the lanes that need them by shuffle within the row's
// group of four lanes.  The acceptance rule is the register kernel's.
#pragma once
#include "stencil_refined_reg.cuh"

namespace {

template <int N>
struct SplitLU {
    static constexpr int NX = N - 32;        // extra rows
    static constexpr int PW = (N + 3) / 4;   // columns per piece
    float a[N];                              // main row: lane
    float b[PW];                             // piece (lane & 3) of extra row 32 + (lane >> 2)
    int mstep, xstep;  // step at which the row was the pivot; N + 1: not yet; -1: padding
};

template <int N>
__global__ void __launch_bounds__(128, 4) build_refined_split_kernel(StencilParams P, int wpb, size_t warp_bytes) {
    using LU = SplitLU<N>;
    constexpr int NX = LU::NX, PW = LU::PW;
    static_assert(NX >= 1 && NX <= 8, "split layout: 33..40 rows");
    static_assert(PW % 2 == 0, "pieces are published as float2");
    static_assert(N == 4 * PW, "the inversion shifts whole rows of four pieces");
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const SplitSmem s = carve_split(smem + wib * warp_bytes, N, P.k);
    uint16_t *pairs = reinterpret_cast<uint16_t *>(smem + wpb * warp_bytes);
    for (int p = threadIdx.x; p < P.k * (P.k - 1) / 2; p += blockDim.x) {
        int j = 1;
        while ((j + 1) * j / 2 <= p) j++;
        pairs[p] = (uint16_t)((p - j * (j - 1) / 2) | (j << 8));
    }
    __syncthreads();
    const int g = lane >> 2, q = lane & 3;
    const bool xvalid = g < NX;
    const int gx = 32 + (xvalid ? g : 0);  // extra row of this lane's group
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    const int64_t count = P.slots ? P.nslots : P.ne;
    for (int64_t t = (int64_t)blockIdx.x * wpb + wib; t < count; t += nwarps) {
        const int64_t e = P.slots ? (int64_t)P.slots[t] : t;
        // a learned seed is read first so that its latency hides behind the load and assembly
        const float seed_main = (P.seed && lane < P.k) ? __ldg(&P.seed[e * P.k + lane]) : 0.0f;
        const float seed_x = (P.seed && lane < NX && 32 + lane < P.k) ? __ldg(&P.seed[e * P.k + 32 + lane]) : 0.0f;
        int es = 0;
        if (load_interior(P, e, s, lane, &es) != 0) {
            split_defer(P, e, lane);
            __syncwarp();
            continue;
        }
        assemble_packed<false>(P, s, lane, es, pairs);  // FP64 entries: the residuals run in FP64
        LU L;
        const int ti = tri(lane);
#pragma unroll
        for (int cc = 0; cc < N; cc++) L.a[cc] = narrow(s.Mp[cc > lane ? tri(cc) + lane : ti + cc]);
#pragma unroll
        for (int t = 0; t < PW; t++) {
            const int col = q * PW + t;
            L.b[t] = (xvalid && col < N) ? narrow(pk_at(s.Mp, gx, col < N ? col : 0)) : 0.0f;
        }
        L.mstep = N + 1;
        L.xstep = xvalid ? N + 1 : -1;
        // start of the refinement: x0 = 0 and rhs = b, or with a learned seed x0 = [w_pred; 0]
        // and rhs = b - A32 x0, formed from the FP32 rows before they are factorised
        float rm = narrow(s.bv[lane]);
        float rx = xvalid ? narrow(s.bv[gx]) : 0.0f;
        if (P.seed) {
            s.xs[lane] = seed_main;
            s.x[lane] = widen(seed_main);
            if (lane < NX) {
                s.xs[32 + lane] = seed_x;
                s.x[32 + lane] = widen(seed_x);
            }
            __syncwarp();
            float am = 0.0f, ax = 0.0f;
#pragma unroll
            for (int j = 0; j < N; j++) am = fmaf(L.a[j], s.xs[j], am);
#pragma unroll
            for (int t = 0; t < PW; t++) ax = fmaf(L.b[t], s.xs[q * PW + t < N ? q * PW + t : 0], ax);  // b = 0 past N
            ax += __shfl_xor_sync(0xffffffffu, ax, 1);
            ax += __shfl_xor_sync(0xffffffffu, ax, 2);
            rm -= am;
            rx = xvalid ? rx - ax : 0.0f;
        } else {
            s.x[lane] = 0.0;
            if (lane < NX) s.x[32 + lane] = 0.0;
        }
        __syncwarp();

        // ---- FP32 Gauss-Jordan inversion with partial pivoting, rows in place.  Every row is a
        // window of N registers: before step c it holds columns c..N-1 of the row, then the
        // row's entries of the c inverse columns formed so far.  Step c eliminates column c
        // (window position 0) from every row but the pivot row, shifts each window left by one
        // and appends the row's entry of the new inverse column: minus the multiplier, or 1 in
        // the pivot row, which is left unscaled (a row may carry any scale factor through the
        // later steps; the pivot row's row of the inverse is multiplied by its reciprocal
        // pivot at the end).  Every step runs the same code, so the loop stays rolled and the
        // solves become products with the inverse: no serial substitution chains.
        bool ok = true;
        float rsc = 1.0f, xsc = 1.0f;  // reciprocal pivots of this lane's main and extra rows
#pragma unroll 1
        for (int c = 0; c < N; c++) {
            // pivot-row buffers alternate by step: the publish of step c + 1 cannot overwrite
            // the row that step c is still reading, so one warp barrier per step suffices
            float *const rowbuf = s.rowbuf + (c & 1) * 4 * PW;
            const unsigned km = L.mstep == N + 1 ? (__float_as_uint(fabsf(L.a[0])) & ~63u) | (unsigned)(63 - lane) : 0u;
            const unsigned kx =
                (L.xstep == N + 1 && q == 0) ? (__float_as_uint(fabsf(L.b[0])) & ~63u) | (unsigned)(63 - gx) : 0u;
            const unsigned key = __reduce_max_sync(0xffffffffu, max(km, kx));
            const int brow = 63 - (int)(key & 63u);
            const bool pm = brow == lane;           // this lane's main row is the pivot row
            const bool px = xvalid && brow == gx;  // this lane's extra row is the pivot row
            if (pm) {
#pragma unroll
                for (int q4 = 0; q4 < N / 4; q4++)
                    reinterpret_cast<float4 *>(rowbuf)[q4] =
                        make_float4(L.a[4 * q4], L.a[4 * q4 + 1], L.a[4 * q4 + 2], L.a[4 * q4 + 3]);
            } else if (px) {
#pragma unroll
                for (int t = 0; t < PW; t += 2)
                    reinterpret_cast<float2 *>(rowbuf)[(q * PW + t) >> 1] = make_float2(L.b[t], L.b[t + 1]);
            }
            __syncwarp();
            const float pvt = rowbuf[0];
            // approximate reciprocal (the FP32 inverse only preconditions the refinement); a
            // zero, subnormal (flushed) or non-finite pivot gives an infinite or NaN reciprocal,
            // which reaches the inverse's entries: the check after the loop fails it
            float inv;
            asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(pvt));
            if (pm) {
                L.mstep = c;
                rsc = inv;
            }
            if (px) {
                L.xstep = c;
                xsc = inv;
            }
            // main row: window position j - 1 <- j minus the multiplier times the pivot row
            {
                const float m = pm ? 0.0f : L.a[0] * inv;
#pragma unroll
                for (int q4 = 0; q4 < N / 4; q4++) {
                    const float4 v = reinterpret_cast<const float4 *>(rowbuf)[q4];
                    const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int t = 0; t < 4; t++) {
                        const int j = 4 * q4 + t;
                        if (j >= 1) L.a[j >= 1 ? j - 1 : 0] = fmaf(-m, vv[t], L.a[j]);
                    }
                }
                L.a[N - 1] = pm ? 1.0f : -m;
            }
            // extra row: the multiplier comes from the piece holding window position 0, the
            // entry shifted into a piece's last slot from the next piece of the same row
            {
                // every lane takes part in the shuffle (the pivot row's lanes then drop it)
                const float mxs = __shfl_sync(0xffffffffu, L.b[0] * inv, lane & ~3);
                const float mx = px ? 0.0f : mxs;
                const float nxt = __shfl_down_sync(0xffffffffu, L.b[0], 1);
                const float vn = rowbuf[q < 3 ? (q + 1) * PW : 0];
                // the piece's pivot-row entries as aligned pairs (q * PW is even)
                const float2 *const rb2 = reinterpret_cast<const float2 *>(rowbuf + q * PW);
                float pr[PW];
#pragma unroll
                for (int t = 0; t < PW / 2; t++) {
                    const float2 v = rb2[t];
                    pr[2 * t] = v.x;
                    pr[2 * t + 1] = v.y;
                }
#pragma unroll
                for (int t = 0; t + 1 < PW; t++) L.b[t] = fmaf(-mx, pr[t + 1], L.b[t + 1]);
                L.b[PW - 1] = q < 3 ? fmaf(-mx, vn, nxt) : (px ? 1.0f : -mx);
            }
        }
        // rows of the inverse: the unscaled pivot rows times their reciprocal pivots; the
        // factorisation fails if any entry of the inverse is not finite
        bool fin = true;
#pragma unroll
        for (int j = 0; j < N; j++) {
            L.a[j] *= rsc;
            fin &= isfinite(L.a[j]);
        }
#pragma unroll
        for (int t = 0; t < PW; t++) {
            L.b[t] *= xsc;
            fin &= isfinite(L.b[t]);
        }
        ok = __all_sync(0xffffffffu, fin);

        // ---- refinement: products with the FP32 inverse, FP64 residuals
        bool accepted = false;
        double est_final = 0.0;
        int nres = 0;
        if (ok) {
            // x = A32^{-1} r.  The row pivoted at step c holds row c of the inverse, its window
            // position s the column of the row pivoted at step s: every row puts its right-hand
            // side at its own pivot step, and each row's dot product is unknown c.
            float *const rp = s.rowbuf;  // free once the inversion is done (16-byte aligned)
            auto solve = [&]() {
                rp[L.mstep] = rm;
                if (xvalid && q == 0) rp[L.xstep] = rx;
                __syncwarp();
                float dm = 0.0f, dx = 0.0f;
#pragma unroll
                for (int q4 = 0; q4 < N / 4; q4++) {
                    const float4 v = reinterpret_cast<const float4 *>(rp)[q4];
                    dm = fmaf(L.a[4 * q4], v.x, dm);
                    dm = fmaf(L.a[4 * q4 + 1], v.y, dm);
                    dm = fmaf(L.a[4 * q4 + 2], v.z, dm);
                    dm = fmaf(L.a[4 * q4 + 3], v.w, dm);
                }
#pragma unroll
                for (int t = 0; t < PW; t += 2) {
                    const float2 v = reinterpret_cast<const float2 *>(rp)[(q * PW + t) >> 1];
                    dx = fmaf(L.b[t], v.x, dx);
                    dx = fmaf(L.b[t + 1], v.y, dx);
                }
                dx += __shfl_xor_sync(0xffffffffu, dx, 1);
                dx += __shfl_xor_sync(0xffffffffu, dx, 2);
                s.xs[L.mstep] = dm;
                if (xvalid && q == 0) s.xs[L.xstep] = dx;
                __syncwarp();
            };
            // FP64 residual r = b - A x: rows 0..31 one per lane, rows 32..N-1 as (row, quarter
            // of the columns) over the four lanes of the row's group, summed by shuffles
            auto residual = [&]() {
                nres++;
                double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
#pragma unroll 1
                for (int j = 0; j < (N & ~3); j += 4) {
                    c0 = fma(-s.Mp[j + 0 > lane ? tri(j + 0) + lane : ti + j + 0], s.x[j + 0], c0);
                    c1 = fma(-s.Mp[j + 1 > lane ? tri(j + 1) + lane : ti + j + 1], s.x[j + 1], c1);
                    c2 = fma(-s.Mp[j + 2 > lane ? tri(j + 2) + lane : ti + j + 2], s.x[j + 2], c2);
                    c3 = fma(-s.Mp[j + 3 > lane ? tri(j + 3) + lane : ti + j + 3], s.x[j + 3], c3);
                }
#pragma unroll
                for (int j = N & ~3; j < N; j++) c0 = fma(-s.Mp[j > lane ? tri(j) + lane : ti + j], s.x[j], c0);
                // an extra row that is a polynomial-reproduction row (gx >= k) is zero past column
                // k: its four pieces cover columns 0..k-1 only
                double ex = 0.0;
                const int tg = tri(gx);
                const int ncol = gx >= P.k ? P.k : N, pw = (ncol + 3) >> 2;
                for (int t = 0; t < pw; t++) {
                    const int j = q * pw + t;
                    if (j < ncol) ex = fma(-s.Mp[j <= gx ? tg + j : tri(j) + gx], s.x[j], ex);
                }
                ex += __shfl_xor_sync(0xffffffffu, ex, 1);
                ex += __shfl_xor_sync(0xffffffffu, ex, 2);
                rm = narrow(s.bv[lane] + ((c0 + c1) + (c2 + c3)));
                rx = xvalid ? narrow(s.bv[gx] + ex) : 0.0f;
            };
            // After acceptance: the polynomial-reproduction rows (k..N-1) once more in FP64 and
            // one correction through the inverse.  A product with a Gauss-Jordan inverse is not
            // backward stable (unlike the LU substitutions): it leaves a residual of about
            // cond * 2^-24 of the last step, and in these rows that residual is a violation of
            // the exact reproduction of polynomials, which the apply of a smooth field
            // amplifies by sum |w| (~1/h^2).  The correction shrinks it by the same factor.  The
            // rows' zero block leaves k products per row; the rows share the warp's lanes in one
            // pass.
            auto polish_rhs = [&]() {
                // lane (t, h): row k + t, column block h of c3 blocks (c3 lanes per row)
                const int k = P.k, nm = N - k;
                const int c3 = nm >= 32 ? 1 : 32 / nm, cw = (k + c3 - 1) / c3;
                const int t0 = lane / c3, h = lane - t0 * c3;
                for (int tb = 0; tb < nm; tb += 32 / c3) {
                    const int t = tb + t0;
                    double acc = 0.0;
                    if (t < nm && t0 < 32 / c3) {
                        const int ti2 = tri(k + t);
                        for (int jj = 0; jj < cw; jj++) {
                            const int j = h * cw + jj;
                            if (j < k) acc = fma(-s.Mp[ti2 + j], s.x[j], acc);
                        }
                    }
                    for (int o = 1; o < c3; o++) {
                        const double v = __shfl_down_sync(0xffffffffu, acc, o);
                        if (h == 0) acc += v;
                    }
                    if (t < nm && t0 < 32 / c3 && h == 0) s.xs[k + t] = narrow(s.bv[k + t] + acc);
                }
                __syncwarp();
                rm = lane >= k ? s.xs[lane] : 0.0f;
                rx = (xvalid && gx >= k) ? s.xs[gx] : 0.0f;
                __syncwarp();
            };  // the loop below solves with these right-hand sides and corrects the weights
            // One call site of the solve serves the refinement steps and the polish (the
            // kernel's code size sets its instruction-fetch stalls).
            const float tolf = (float)P.tol;
            float dprev = 0.0f;
            bool polishing = false;
            for (int step = 0;; step++) {
                solve();
                if (polishing) {
                    for (int t = lane; t < P.k; t += 32) s.x[t] += widen(s.xs[t]);  // the weights
                    __syncwarp();
                    break;
                }
                float dmaxf = 0.0f, xmaxf = 0.0f;
                for (int t = lane; t < N; t += 32) {
                    const float d = s.xs[t];
                    s.x[t] += widen(d);
                    if (t < P.k) {
                        dmaxf = fmaxf(dmaxf, fabsf(d));
                        xmaxf = fmaxf(xmaxf, fabsf(narrow(s.x[t])));
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    dmaxf = fmaxf(dmaxf, __shfl_xor_sync(0xffffffffu, dmaxf, o));
                    xmaxf = fmaxf(xmaxf, __shfl_xor_sync(0xffffffffu, xmaxf, o));
                }
                __syncwarp();
                if (step == 0) {
                    // the first solve reaches the FP32 floor from any start; with a seed,
                    // |d0| / |x| is the surrogate's error as judged by the solve
                    if (P.seed && lane == 0 && xmaxf > 0.0f) {
                        atomicAdd(&P.counters[5], (unsigned long long)(1e6f * fminf(1.0f, dmaxf / xmaxf)));
                        atomicAdd(&P.counters[6], 1ull);
                    }
                    dprev = xmaxf;
                } else {
                    // contraction |d1| / |d0| past 1e-3: the stencil takes the general path;
                    // accept once |d_s| is below tol relative to x and shrinking
                    if (step == 1 && !(dmaxf <= 1e-3f * dprev)) break;
                    if (dmaxf <= tolf * xmaxf && dmaxf <= 0.5f * dprev) {
                        accepted = true;
                        est_final = xmaxf > 0.0f ? (double)(dmaxf / xmaxf) : 0.0;
                        polish_rhs();
                        polishing = true;
                        continue;
                    }
                    dprev = dmaxf;
                }
                if (step >= P.refine_steps || !isfinite(dmaxf)) break;
                residual();
            }
        }
        if (lane == 0 && ok) atomicAdd(&P.counters[4], (unsigned long long)nres);
        if (accepted) {
            WarpSmem w;
            w.cols = s.cols;
            scatter_row(P, e, w, lane, es, s.x, 1, 1);
            if (lane == 0) {
                if (P.status) P.status[e] = 0;
                atomicMax(reinterpret_cast<unsigned long long *>(P.max_resid),
                          (unsigned long long)__double_as_longlong(est_final));
            }
        } else {
            split_defer(P, e, lane);
        }
        __syncwarp();
    }
}

template <int N>
int launch_refined_split(rbf_ctx *ctx, const StencilParams &P) {
    const size_t wb = split_smem_bytes(N, P.k);
    const int wpb = 4;
    const size_t smem = wb * wpb + sizeof(uint16_t) * (size_t)(P.k * (P.k + 1) / 2);
    RBF_CUDA(ctx, cudaFuncSetAttribute(build_refined_split_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_refined_split_kernel<N>, wpb * 32,
                                                                smem));
    if (per_sm < 1) per_sm = 1;
    const int64_t count = P.slots ? P.nslots : P.ne;
    if (count == 0) return RBF_OK;
    const int64_t blocks = std::min<int64_t>((count + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
    build_refined_split_kernel<N><<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P, wpb, wb);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

}  // namespace
