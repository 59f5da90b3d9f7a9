// Per-stencil solves shared by the one-launch-per-size kernels (stencil_build.cu) and
// the persistent batched kernel (batched.cu).
#pragma once
#include "stencil_device.cuh"

namespace {

// One stencil e on one warp, plain FP64: load, assemble, LU, scatter.
__device__ void solve_fp64_warp(const StencilParams &P, int64_t e, const WarpSmem &w, int lane) {
    int es = 0, eval_local = -2;
    int st = load_stencil(P, e, w, lane, &es, &eval_local);
    if (st != 0) {
        __syncwarp();
        return;
    }
    assemble_fp64(P, w, lane, es, eval_local);
    bool ok = lu_solve_fp64(w.M, P.n, P.nops, lane);
    if (!ok) {
        if (lane == 0) {
            if (P.status) P.status[e] = 1;
            atomicAdd(&P.counters[0], 1ull);
        }
        __syncwarp();
        return;
    }
    scatter_row(P, e, w, lane, es, w.M + P.n, mat_ld(P.n, P.nops), 1);
    if (lane == 0 && P.status) P.status[e] = 0;
    __syncwarp();
}

// FP32-factor refinement of one stencil on one warp (u.F holds the factors): x0 = A32^{-1} b,
// then x += A32^{-1} (b - A x) with the residual in FP64.  Returns whether x (in u.x) is
// accepted; *est_final: the size of the last correction relative to x.
__device__ bool refine_fp32_warp(const StencilParams &P, const WarpSmem &w, const Warp32 &u, int lane,
                                 double *est_final_out) {
    const int n = P.n, nops = P.nops, ld = mat_ld(n, nops);
    bool accepted = false;
    double est_final = 0.0;
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
            if (t / nops < P.k + P.nnr) {  // the weights (value and du/dn unknowns)
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
    *est_final_out = est_final;
    return accepted;
}

// Scatter of an accepted refined solution, or the plain FP64 fallback on one warp.
__device__ void finish_fp32r_warp(const StencilParams &P, int64_t e, const WarpSmem &w, const Warp32 &u, int lane,
                                  int es, int eval_local, bool accepted, double est_final) {
    const int n = P.n, nops = P.nops, ld = mat_ld(n, nops);
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

// One stencil e on one warp, FP32 factorisation + FP64 refinement, FP64 fallback (ND: the
// normal-derivative builds' instantiation).
template <bool ND = false>
__device__ void solve_fp32r_warp(const StencilParams &P, int64_t e, const WarpSmem &w, const Warp32 &u, int lane) {
    int es = 0, eval_local = -2;
    int st = load_stencil(P, e, w, lane, &es, &eval_local);
    if (st != 0) {
        __syncwarp();
        return;
    }
    assemble_refined<ND>(P, w, u, lane, es, eval_local);
    const bool ok = lu_factor_fp32(u.F, u.piv, P.n, lane);
    double est_final = 0.0;
    const bool accepted = ok && refine_fp32_warp(P, w, u, lane, &est_final);
    finish_fp32r_warp(P, e, w, u, lane, es, eval_local, accepted, est_final);
}

}  // namespace
