// Templates of the register-resident refined build (instantiated in stencil_refined_*.cu).
#pragma once
#include <type_traits>

#include "stencil_device.cuh"

namespace {
// ---------------------------------------------------------------------------------------
// Register-resident FP32 factorisation for the system sizes of the standard workloads.
// Lane l owns rows l and l+32 of the augmented matrix [A | b] (N rows, W = N + R columns,
// fully in registers; N and R are template parameters so every column index is static).
// LU with partial pivoting without moving rows: the pivot row of step c is published
// through a shared buffer, every row not yet used as a pivot keeps its multiplier in
// column c and is updated in columns c+1..W-1.  The factors stay in registers through all
// refinement solves (forward substitution in pivot order, back substitution by columns).
// ---------------------------------------------------------------------------------------
// Number of column blocks per row for the residual so that N*JB (row, block) pairs fill the
// 32 lanes with the fewest FMA rounds.
__host__ __device__ constexpr int residual_blocks(int n) {
    int best = 1, best_cost = 1 << 30;
    for (int jb = 1; jb <= 32; jb *= 2) {
        const int cost = ((n * jb + 31) / 32) * ((n + jb - 1) / jb);
        if (cost < best_cost) {
            best_cost = cost;
            best = jb;
        }
    }
    return best;
}

// Shared memory of one warp in the register kernels: the FP64 system (WarpSmem), then the
// FP64 solution, the FP32 increments, the split coordinates, pivots, reciprocal pivots and
// the pivot-row broadcast buffer (16-byte aligned, rounded up to whole float4s).
__host__ __device__ inline size_t reg_smem_bytes(int n, int k, int nops) {
    size_t b = (warp_smem_bytes(n, k, nops) + 15) & ~(size_t)15;
    b += sizeof(double) * (size_t)n * nops;                  // x
    b += sizeof(float) * (size_t)n * nops;                   // xs
    b += sizeof(float) * 6 * (size_t)k;                      // XH, XL
    b += sizeof(int) * (size_t)n + sizeof(float) * (size_t)n;  // piv, rcp
    b = (b + 15) & ~(size_t)15;
    b += sizeof(float) * (((size_t)n + 3) & ~(size_t)3);     // rowbuf
    return (b + 15) & ~(size_t)15;
}

struct RegSmem {
    Warp32 u;  // u.F is unused (nullptr)
    float *rcp, *rowbuf;
};

__device__ inline RegSmem carve_reg(char *base, int n, int k, int nops) {
    RegSmem r;
    size_t off = (warp_smem_bytes(n, k, nops) + 15) & ~(size_t)15;
    r.u.x = reinterpret_cast<double *>(base + off);
    r.u.r = nullptr;
    r.u.F = nullptr;
    r.u.v = reinterpret_cast<float *>(r.u.x + (size_t)n * nops);
    r.u.XH = r.u.v + (size_t)n * nops;
    r.u.XL = r.u.XH + 3 * (size_t)k;
    r.u.piv = reinterpret_cast<int *>(r.u.XL + 3 * (size_t)k);
    r.rcp = reinterpret_cast<float *>(r.u.piv + n);
    size_t o2 = (size_t)(reinterpret_cast<char *>(r.rcp + n) - base);
    o2 = (o2 + 15) & ~(size_t)15;
    r.rowbuf = reinterpret_cast<float *>(base + o2);
    return r;
}

// double -> float on the integer pipe, mantissa truncated (the FP32 factor only needs
// FP32 accuracy): the exponent is rebased and the top 23 mantissa bits taken in one funnel
// shift; magnitudes below FLT_MIN map to a signed zero (the entries here are bounded, so
// there is no overflow case)
__device__ __forceinline__ float narrow(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const unsigned mag = __funnelshift_l(lo, hi - 0x38000000u, 3);
    return __uint_as_float((hi & 0x7fffffffu) < 0x38100000u ? sign : (sign | mag));
}

template <int N, int R>
struct RegLU {
    static constexpr int ROWS = (N + 31) / 32;
    static constexpr int W = N;  // matrix only; right-hand sides go through reglu_forward/back
    float a[ROWS][W];
    int step[ROWS];  // elimination step at which the row was the pivot; N+1: not yet; -1: padding
};

// Compile-time loop: f(std::integral_constant<int, I>) for I = B, B+S, ... while I != E.
template <int I, int E, int S, class F>
__device__ __forceinline__ void static_for(F &&f) {
    if constexpr (I != E) {
        f(std::integral_constant<int, I>{});
        static_for<I + S, E, S>(f);
    }
}

// Factor in place; returns false on an exactly zero or non-finite pivot.  rowbuf: W floats,
// piv: N ints, rcp: N floats (pivot rows and reciprocal pivots, in elimination order).
template <int N, int R>
__device__ bool reglu_factor(RegLU<N, R> &L, float *rowbuf, int *piv, float *rcp, int lane) {
    constexpr int ROWS = RegLU<N, R>::ROWS, W = RegLU<N, R>::W;
    bool ok = true;
    static_for<0, N, 1>([&](auto cI) {
        constexpr int c = decltype(cI)::value;
        // pivot: largest |a| among rows not yet used (magnitude bits with the 6 low bits
        // replaced by 63 - row, so one max-reduction also breaks near-ties to the lower row)
        unsigned key = 0u;
#pragma unroll
        for (int s = 0; s < ROWS; s++) {
            const unsigned kk = (__float_as_uint(fabsf(L.a[s][c])) & ~63u) | (unsigned)(63 - (lane + 32 * s));
            key = max(key, L.step[s] == N + 1 ? kk : 0u);
        }
        key = __reduce_max_sync(0xffffffffu, key);
        const int brow = 63 - (int)(key & 63u);
        const int pl = brow & 31, ps = brow >> 5;
        // the slot ps is the same in every lane: one branch per slot publishes the row
        // straight from its registers
#pragma unroll
        for (int s = 0; s < ROWS; s++) {
            if (s == ps && lane == pl) {
                L.step[s] = c;
#pragma unroll
                for (int q4 = c / 4; q4 < (W + 3) / 4; q4++) {
                    float4 v;
                    v.x = (4 * q4 + 0 < W) ? L.a[s][(4 * q4 + 0 < W) ? 4 * q4 + 0 : 0] : 0.0f;
                    v.y = (4 * q4 + 1 < W) ? L.a[s][(4 * q4 + 1 < W) ? 4 * q4 + 1 : 0] : 0.0f;
                    v.z = (4 * q4 + 2 < W) ? L.a[s][(4 * q4 + 2 < W) ? 4 * q4 + 2 : 0] : 0.0f;
                    v.w = (4 * q4 + 3 < W) ? L.a[s][(4 * q4 + 3 < W) ? 4 * q4 + 3 : 0] : 0.0f;
                    reinterpret_cast<float4 *>(rowbuf)[q4] = v;
                }
            }
        }
        __syncwarp();
        const float pvt = rowbuf[c];
        ok &= (pvt != 0.0f) && isfinite(pvt);
        // correctly rounded reciprocal without the division's slow path (a zero or
        // non-finite pivot has already failed the factorisation)
        const float inv = __frcp_rn(pvt);
        if (lane == 0) {
            piv[c] = brow;
            rcp[c] = inv;
        }
        // elimination; up to 40 rows it is branch-free: rows already used as pivots (and
        // padding rows) get a zero multiplier, which leaves them unchanged (larger systems
        // keep the branch, which needs fewer live registers)
#pragma unroll
        for (int s = 0; s < ROWS; s++) {
            const bool act = L.step[s] == N + 1;
            if constexpr (N > 40)
                if (!act) continue;
            const float l = act ? L.a[s][c] * inv : 0.0f;
            L.a[s][c] = act ? l : L.a[s][c];
#pragma unroll
            for (int q4 = (c + 1) / 4; q4 < (W + 3) / 4; q4++) {
                const float4 v = reinterpret_cast<const float4 *>(rowbuf)[q4];
                const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int cc = 4 * q4 + t;
                    if (cc > c && cc < W) L.a[s][cc < W ? cc : 0] = fmaf(-l, vv[t], L.a[s][cc < W ? cc : 0]);
                }
            }
        }
        __syncwarp();
    });
    return ok;
}

// Back substitution of right-hand sides held per row (already forward-substituted); x
// (N x R floats, row-major) is written to xs.
template <int N, int R>
__device__ void reglu_back(RegLU<N, R> &L, float (&rhs)[RegLU<N, R>::ROWS][R], const int *piv, const float *rcp,
                           float *xs, int lane) {
    constexpr int ROWS = RegLU<N, R>::ROWS;
    static_for<N - 1, -1, -1>([&](auto cI) {
        constexpr int c = decltype(cI)::value;
        const int p = piv[c];
        const int pl = p & 31, ps = p >> 5;
        const float rc = rcp[c];
        float xq[R];
#pragma unroll
        for (int q = 0; q < R; q++) {
            float v = rhs[0][q];
#pragma unroll
            for (int t = 1; t < ROWS; t++)
                if (ps == t) v = rhs[t][q];
            xq[q] = __shfl_sync(0xffffffffu, v, pl) * rc;
        }
        if (lane < R) {
#pragma unroll
            for (int q = 0; q < R; q++)
                if (q == lane) xs[c * R + q] = xq[q];
        }
#pragma unroll
        for (int s = 0; s < ROWS; s++)
            if (L.step[s] >= 0 && L.step[s] < c) {
#pragma unroll
                for (int q = 0; q < R; q++) rhs[s][q] = fmaf(-L.a[s][c], xq[q], rhs[s][q]);
            }
    });
    __syncwarp();
}

// Forward substitution of right-hand sides (held per row) with the stored multipliers.
template <int N, int R>
__device__ void reglu_forward(RegLU<N, R> &L, float (&rhs)[RegLU<N, R>::ROWS][R], const int *piv, int lane) {
    constexpr int ROWS = RegLU<N, R>::ROWS;
    static_for<0, N, 1>([&](auto cI) {
        constexpr int c = decltype(cI)::value;
        const int p = piv[c];
        const int pl = p & 31, ps = p >> 5;
        float yq[R];
#pragma unroll
        for (int q = 0; q < R; q++) {
            float v = rhs[0][q];
#pragma unroll
            for (int t = 1; t < ROWS; t++)
                if (ps == t) v = rhs[t][q];
            yq[q] = __shfl_sync(0xffffffffu, v, pl);
        }
#pragma unroll
        for (int s = 0; s < ROWS; s++)
            if (L.step[s] > c) {
#pragma unroll
                for (int q = 0; q < R; q++) rhs[s][q] = fmaf(-L.a[s][c], yq[q], rhs[s][q]);
            }
    });
}

template <int N, int R>
__global__ void __launch_bounds__(128, 3) build_refined_reg_kernel(StencilParams P, int wpb, size_t warp_bytes) {
    constexpr int ROWS = RegLU<N, R>::ROWS, W = RegLU<N, R>::W;
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    char *base = smem + wib * warp_bytes;
    WarpSmem w = carve(base, P.n, P.k, P.nops);
    const RegSmem rs = carve_reg(base, P.n, P.k, P.nops);
    const Warp32 &u = rs.u;
    const int ld = mat_ld(N, R);
    float *rowbuf = rs.rowbuf;
    float *xs = u.v;  // N x R floats
    // upper-triangle pair table of the RBF block, shared by the block's warps
    uint16_t *pairs = reinterpret_cast<uint16_t *>(smem + wpb * warp_bytes);
    for (int p = threadIdx.x; p < P.k * (P.k + 1) / 2; p += blockDim.x) {
        int j = 0;
        while ((j + 1) * (j + 2) / 2 <= p) j++;
        pairs[p] = (uint16_t)((p - j * (j + 1) / 2) | (j << 8));
    }
    __syncthreads();
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P.ne; e += nwarps) {
        // a learned seed is read here, at the top of the stencil, so that its latency hides
        // behind the load and assembly (lane t holds entry t and t + 32; one operator)
        float seed_reg[ROWS];
#pragma unroll
        for (int s = 0; s < ROWS; s++) {
            const int i = lane + 32 * s;
            seed_reg[s] = (R == 1 && P.seed && i < P.k) ? __ldg(&P.seed[e * P.k + i]) : 0.0f;
        }
        int es = 0, eval_local = -2;
        int st = load_stencil(P, e, w, lane, &es, &eval_local);
        if (st != 0) {
            __syncwarp();
            continue;
        }
        assemble_refined(P, w, u, lane, es, eval_local, pairs);
        float *rcp = rs.rcp;
        RegLU<N, R> L;
#pragma unroll
        for (int s = 0; s < ROWS; s++) {
            const int r = lane + 32 * s;
            const bool act = r < N;
            L.step[s] = act ? N + 1 : -1;
#pragma unroll
            for (int cc = 0; cc < N; cc++) L.a[s][cc] = act ? narrow(w.M[r * ld + cc]) : 0.0f;
        }
        __syncwarp();
        // start of the refinement: x0 = 0 and rhs = b, or with a learned seed x0 = [w_pred; 0]
        // and rhs = b - A32 x0, formed here from the FP32 rows while they are still unfactored
        float rhs[ROWS][R];
        if (P.seed) {
            if constexpr (R == 1) {
#pragma unroll
                for (int s = 0; s < ROWS; s++) {
                    const int t = lane + 32 * s;
                    if (t < N) {
                        xs[t] = seed_reg[s];
                        u.x[t] = widen(seed_reg[s]);
                    }
                }
            } else {
                for (int t = lane; t < N * R; t += 32) {
                    const int i = t / R;
                    const float sv = i < P.k ? __ldg(&P.seed[e * P.k + i]) : 0.0f;
                    xs[t] = sv;
                    u.x[t] = widen(sv);
                }
            }
            __syncwarp();
#pragma unroll
            for (int s = 0; s < ROWS; s++) {
                const int i = lane + 32 * s;
#pragma unroll
                for (int q = 0; q < R; q++) {
                    float acc = i < N ? (float)w.M[(i < N ? i : 0) * ld + N + q] : 0.0f;
                    static_for<0, N, 1>([&](auto jI) {
                        constexpr int j = decltype(jI)::value;
                        acc = fmaf(-L.a[s][j], xs[j * R + q], acc);
                    });
                    rhs[s][q] = acc;
                }
            }
        } else {
            for (int t = lane; t < N * R; t += 32) u.x[t] = 0.0;
#pragma unroll
            for (int s = 0; s < ROWS; s++) {
                const int i = lane + 32 * s;
#pragma unroll
                for (int q = 0; q < R; q++) rhs[s][q] = i < N ? (float)w.M[(i < N ? i : 0) * ld + N + q] : 0.0f;
            }
        }
        __syncwarp();
        const bool ok = reglu_factor<N, R>(L, rowbuf, u.piv, rcp, lane);
        bool accepted = false;
        double est_final = 0.0;
        int nres = 0;
        if (ok) {
            // FP64 residual r = b - A x into rhs; rows k..N-1 are the polynomial reproduction
            // constraints.  The N x N products are spread evenly over the warp as (row, block
            // of JB columns) pairs; partial sums meet by shuffles and the row owner picks its
            // entry up from shared memory.
            auto residual = [&]() {
                nres++;
                constexpr int JB = residual_blocks(N);
                constexpr int JL = (N + JB - 1) / JB;
                float *rbuf = xs;  // N x R floats, free until the next back substitution
#pragma unroll 1
                for (int pass = 0; pass < (N * JB + 31) / 32; pass++) {
                    const int pr = pass * 32 + lane;
                    const int i = pr / JB, jb = pr % JB;
                    double acc[R];
#pragma unroll
                    for (int q = 0; q < R; q++) acc[q] = 0.0;
                    if (i < N) {
                        const int j0 = jb * JL;
#pragma unroll 2
                        for (int jj = 0; jj < JL; jj++) {
                            const int j = j0 + jj;
                            if (j < N) {
                                const double aij = w.M[j * ld + i];
#pragma unroll
                                for (int q = 0; q < R; q++) acc[q] = fma(-aij, u.x[j * R + q], acc[q]);
                            }
                        }
                    }
#pragma unroll
                    for (int o = JB / 2; o > 0; o >>= 1)
#pragma unroll
                        for (int q = 0; q < R; q++) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
                    if (i < N && jb == 0)
#pragma unroll
                        for (int q = 0; q < R; q++) rbuf[i * R + q] = __double2float_rn(w.M[i * ld + N + q] + acc[q]);
                }
                __syncwarp();
#pragma unroll
                for (int s = 0; s < ROWS; s++) {
                    const int i = lane + 32 * s;
#pragma unroll
                    for (int q = 0; q < R; q++) rhs[s][q] = i < N ? rbuf[i * R + q] : 0.0f;
                }
                __syncwarp();
            };
            // the first solve leaves an error at the FP32 floor (about cond(A) * 2^-24
            // relative) from any start: a seed cannot beat it, so it costs no FP64 residual
            const float tolf = (float)P.tol;
            float dprev = 0.0f;
            for (int step = 0;; step++) {
                reglu_forward<N, R>(L, rhs, u.piv, lane);
                reglu_back<N, R>(L, rhs, u.piv, rcp, xs, lane);
                float dmaxf = 0.0f, xmaxf = 0.0f;
                for (int t = lane; t < N * R; t += 32) {
                    const float d = xs[t];
                    u.x[t] += widen(d);
                    if (t / R < P.k) {
                        dmaxf = fmaxf(dmaxf, fabsf(d));
                        xmaxf = fmaxf(xmaxf, fabsf(__double2float_rn(u.x[t])));
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    dmaxf = fmaxf(dmaxf, __shfl_xor_sync(0xffffffffu, dmaxf, o));
                    xmaxf = fmaxf(xmaxf, __shfl_xor_sync(0xffffffffu, xmaxf, o));
                }
                __syncwarp();
                if (step == 0) {
                    // the first solve reaches the same FP32 floor from any start, so |x| is
                    // the reference for the contraction estimate; with a seed, |d0|/|x| is
                    // the surrogate's error as judged by the solve
                    if (P.seed && lane == 0 && xmaxf > 0.0f) {
                        atomicAdd(&P.counters[5], (unsigned long long)(1e6f * fminf(1.0f, dmaxf / xmaxf)));
                        atomicAdd(&P.counters[6], 1ull);
                    }
                    dprev = xmaxf;
                } else {
                    // contraction of the refinement, |d1|/|d0|: about cond(A) * 2^-24; past
                    // 1e-3 (cond ~ 1e5) the double-float entries (~2^-44) could move the
                    // weights by more than 1e-9, so the stencil takes the FP64 path
                    if (step == 1 && !(dmaxf <= 1e-3f * dprev)) break;
                    // |d_s| estimates the error of x before this correction: accept once it is
                    // below tol and shrinking (a contraction estimate from one ratio is not
                    // safe: the error can lie along directions that contract far more slowly)
                    if (dmaxf <= tolf * xmaxf && dmaxf <= 0.5f * dprev) {
                        accepted = true;
                        est_final = xmaxf > 0.0f ? (double)(dmaxf / xmaxf) : 0.0;
                        break;
                    }
                    dprev = dmaxf;
                }
                if (step >= P.refine_steps || !isfinite(dmaxf)) break;
                residual();
            }
        }
        if (lane == 0 && ok) atomicAdd(&P.counters[4], (unsigned long long)nres);
        if (accepted) {
            scatter_row(P, e, w, lane, es, u.x, R, 1);
            if (lane == 0) {
                if (P.status) P.status[e] = 0;
                atomicMax(reinterpret_cast<unsigned long long *>(P.max_resid),
                          (unsigned long long)__double_as_longlong(est_final));
            }
        } else {
            if (eval_local == -2) assemble_fp64(P, w, lane, es, eval_local);
            const bool ok64 = lu_solve_fp64(w.M, N, R, lane);
            if (ok64) {
                scatter_row(P, e, w, lane, es, w.M + N, ld, 1);
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

template <int N, int R>
int launch_refined_reg(rbf_ctx *ctx, const StencilParams &P) {
    const size_t wb = reg_smem_bytes(P.n, P.k, P.nops);
    const int wpb = 4;
    const size_t smem = wb * wpb + sizeof(uint16_t) * (size_t)(P.k * (P.k + 1) / 2);
    RBF_CUDA(ctx, cudaFuncSetAttribute(build_refined_reg_kernel<N, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_refined_reg_kernel<N, R>, wpb * 32, smem));
    if (per_sm < 1) per_sm = 1;
    const int64_t blocks = std::min<int64_t>((P.ne + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
    build_refined_reg_kernel<N, R><<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P, wpb, wb);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

}  // namespace
