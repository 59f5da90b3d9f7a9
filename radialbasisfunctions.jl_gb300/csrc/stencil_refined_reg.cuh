// Templates of the register-resident refined build (instantiated in stencil_refined_*.cu).
#pragma once
#include <type_traits>

#include "stencil_device.cuh"

namespace {
// ---------------------------------------------------------------------------------------
// Register-resident FP32 factorisation for the system sizes of the standard workloads.
// Lane l owns rows l and l+32 of the system (N rows, fully in registers; N and the number R
// of right-hand sides are template parameters so every column index is static).  The FP32
// factorisation is a Gauss-Jordan inversion in place (reg_invert); the inverse stays in
// registers through all refinement solves, each one product with it (reg_apply_inverse).
// The residuals of the refinement are double-float dot products on the FP32 pipe, the final
// pass over the polynomial-reproduction rows is FP64.
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

// lower triangle by rows: A(i, j), j <= i, at tri(i) + j
__host__ __device__ constexpr int tri(int i) { return (i * (i + 1)) >> 1; }

// ---- double-float storage and residual arithmetic of the register kernels (FP32 pipe) ----
// The packed system, its right-hand sides and the refined solution are double-float values
// hi + lo (about 48 significant bits, the accuracy the double-float assembly gives the
// entries), each kept in one 64-bit shared-memory slot with hi in the low word.  On GB300 the
// FP64 pipe retires two lanes per SM and clock against 128 for FP32, so the residuals of the
// refinement run here in double-float arithmetic instead of FP64.
__device__ __forceinline__ double df_pack(float hi, float lo) {
    return __hiloint2double(__float_as_int(lo), __float_as_int(hi));
}
__device__ __forceinline__ float df_hi(double d) { return __int_as_float(__double2loint(d)); }
__device__ __forceinline__ float df_lo(double d) { return __int_as_float(__double2hiint(d)); }
// an FP64 value as the nearest float and the float nearest to the remainder
__device__ __forceinline__ double df_pack_double(double v) {
    const float h = d2f_rn_bits(v);
    return df_pack(h, d2f_rn_bits(v - widen(h)));
}
__device__ __forceinline__ double df_unpack_double(double d) { return widen(df_hi(d)) + widen(df_lo(d)); }
// x + d for a float d, renormalised
__device__ __forceinline__ double df_add_f(double x, float d) {
    const float xh = df_hi(x), xl = df_lo(x);
    const float s = xh + d, z = s - xh;
    const float q = ((xh - (s - z)) + (d - z)) + xl;
    const float h = s + q;
    return df_pack(h, q - (h - s));
}

// Dot-product accumulation after Sum2 of Ogita, Rump and Oishi ("Accurate sum and dot
// product", SIAM J. Sci. Comput. 26 (2005)): s is the running sum of the products' high
// parts, each addition's rounding error is recovered exactly (Knuth's TwoSum) and added to
// the compensation c, which also takes each product's rounding error (an FMA gives it
// exactly) and the cross terms hi*lo; the lo*lo terms (~2^-48 relative) are dropped.  The
// result is as accurate as if computed in about twice the working precision, whatever the
// cancellation between the terms.
struct DfSum {
    float s, c;
};
__device__ __forceinline__ DfSum dfsum_of(double b) { return {df_hi(b), df_lo(b)}; }
// acc -= a * x (a, x packed double-float)
__device__ __forceinline__ void dfsum_sub(DfSum &acc, double a, double x) {
    const float ah = df_hi(a), al = df_lo(a), xh = df_hi(x), xl = df_lo(x);
    const float p = (-ah) * xh;
    const float e = fmaf(-ah, xh, -p);  // -ah * xh = p + e exactly
    const float s = acc.s + p, z = s - acc.s;
    const float q = (acc.s - (s - z)) + (p - z);  // acc.s + p = s + q exactly
    acc.s = s;
    acc.c = fmaf(-al, xh, fmaf(-ah, xl, acc.c + (q + e)));
}
__device__ __forceinline__ DfSum dfsum_merge(DfSum a, DfSum b) {
    const float s = a.s + b.s, z = s - a.s;
    const float q = (a.s - (s - z)) + (b.s - z);
    return {s, (a.c + b.c) + q};
}
// a merged with lane (lane ^ o)'s accumulator; every lane of the warp must execute it
__device__ __forceinline__ DfSum dfsum_xor(DfSum a, int o) {
    return dfsum_merge(a, {__shfl_xor_sync(0xffffffffu, a.s, o), __shfl_xor_sync(0xffffffffu, a.c, o)});
}
__device__ __forceinline__ float dfsum_value(DfSum a) { return a.s + a.c; }

// Shared memory of one warp of the register kernels: packed system (lower triangle by rows)
// and its nops right-hand sides (n x nops), both double-float (df_pack), FP64 local
// coordinates and column indices, the double-float solution (n x nops; the weights are
// unpacked to FP64 in place before the scatter), FP32 increments (n x nops), split
// coordinates (hi and lo parts, four floats per point, 16-byte aligned: one vector load per
// point), pivots, reciprocal pivots and two pivot-row buffers (16-byte aligned,
// 4 * ceil(n/4) floats each), which the solves reuse for the right-hand sides in pivot order.
struct SplitSmem {
    double *Mp, *bv, *X, *x;
    int *cols, *piv;
    float *xs, *XH, *XL, *rcp, *rowbuf;
};

__host__ __device__ inline size_t split_smem_bytes(int n, int k, int nops = 1) {
    size_t b = sizeof(double) * ((size_t)tri(n) + 2 * (size_t)n * nops + 3 * (size_t)k);
    b += sizeof(int) * ((size_t)k + n) + sizeof(float) * (size_t)n * nops;
    b = (b + 15) & ~(size_t)15;
    b += sizeof(float) * (8 * (size_t)k + n);  // split coordinates (2 x 4 per point), reciprocal pivots
    b = (b + 15) & ~(size_t)15;
    // two pivot-row buffers, alternating by step; after the inversion the right-hand sides
    // in pivot order (n x nops)
    const size_t rb = 8 * (((size_t)n + 3) / 4), rr = (((size_t)n + 3) & ~(size_t)3) * nops;
    b += sizeof(float) * (rb > rr ? rb : rr);
    return (b + 15) & ~(size_t)15;
}

__device__ inline SplitSmem carve_split(char *base, int n, int k, int nops = 1) {
    SplitSmem s;
    double *d = reinterpret_cast<double *>(base);
    s.Mp = d;
    s.bv = s.Mp + tri(n);
    s.X = s.bv + (size_t)n * nops;
    s.x = s.X + 3 * k;
    s.cols = reinterpret_cast<int *>(s.x + (size_t)n * nops);
    s.piv = s.cols + k;
    s.xs = reinterpret_cast<float *>(s.piv + n);
    size_t o = (size_t)(reinterpret_cast<char *>(s.xs + (size_t)n * nops) - base);
    s.XH = reinterpret_cast<float *>(base + ((o + 15) & ~(size_t)15));
    s.XL = s.XH + 4 * k;
    s.rcp = s.XL + 4 * k;
    o = (size_t)(reinterpret_cast<char *>(s.rcp + n) - base);
    s.rowbuf = reinterpret_cast<float *>(base + ((o + 15) & ~(size_t)15));
    return s;
}

// Column indices and local coordinates (scaled by 2^-es, as load_stencil) of stencil e.
// Returns 1 without scaling when a boundary point is in the stencil: such stencils are
// deferred to the general kernel.
__device__ int load_interior(const StencilParams &P, int64_t e, const SplitSmem &s, int lane, int *es_out) {
    const int k = P.k, dim = P.dim;
    double x0[3] = {0, 0, 0};
    for (int d = 0; d < dim; d++) x0[d] = P.eval[e * dim + d];
    double r2max = 0.0;
    bool anyb = false;
    const int32_t *nbr = P.adj_ptr ? P.adjl + P.adj_ptr[e] : P.adjl + e * k;
    for (int i = lane; i < k; i += 32) {
        const int g = nbr[i];
        s.cols[i] = g;
        double r2 = 0.0;
        for (int d = 0; d < 3; d++) {
            const double dd = d < dim ? P.data[(int64_t)g * dim + d] - x0[d] : 0.0;
            s.X[i * 3 + d] = dd;
            r2 += dd * dd;
        }
        r2max = fmax(r2max, r2);
        if (P.isb) anyb |= (P.isb[g] != 0);
    }
    if (__any_sync(0xffffffffu, anyb)) return 1;
    {  // r2max >= 0: an integer max of its bit pattern
        long long m = __double_as_longlong(r2max);
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        r2max = __longlong_as_double(m);
    }
    int es = 0;
    if (r2max > 0.0) es = sqrt_frexp_exponent(r2max);
    *es_out = es;
    __syncwarp();
    for (int i = lane; i < k; i += 32)
        for (int d = 0; d < dim; d++) s.X[i * 3 + d] = scale2(s.X[i * 3 + d], -es);
    __syncwarp();
    return 0;
}

// [Phi P; P^T 0] of an interior stencil in double-float (the arithmetic of
// assemble_refined), stored as the packed lower triangle, and the right-hand sides (evaluated
// in FP64): packed double-float entries (DF, for double-float residuals) or FP64 ones.
template <bool DF>
__device__ void assemble_packed(const StencilParams &P, const SplitSmem &s, int lane, int es, const uint16_t *pairs) {
    const int k = P.k, n = P.n, dim = P.dim, nmon = P.nmon, nops = P.nops;
    for (int i = lane; i < k; i += 32)
        for (int d = 0; d < 3; d++) {
            const double xv = d < dim ? s.X[i * 3 + d] : 0.0;
            const float hi = d2f_rn_bits(xv);
            s.XH[i * 4 + d] = hi;
            s.XL[i * 4 + d] = d2f_rn_bits(xv - widen(hi));
        }
    for (int t = lane; t < tri(n) - tri(k); t += 32) s.Mp[tri(k) + t] = 0.0;  // rows k..n-1; the
    __syncwarp();                                                           // P^T part is set below
    // phi(0) = 0 on the diagonal; the strict pairs i < j from the block's table
    for (int i = lane; i < k; i += 32) s.Mp[tri(i) + i] = 0.0;
    const int npairs = k * (k - 1) / 2;
    for (int p = lane; p < npairs; p += 32) {
        const unsigned pk = pairs[p];
        const int i = (int)(pk & 0xffu), j = (int)(pk >> 8);  // i < j
        const float4 hi4 = reinterpret_cast<const float4 *>(s.XH)[i], hj4 = reinterpret_cast<const float4 *>(s.XH)[j];
        const float4 li4 = reinterpret_cast<const float4 *>(s.XL)[i], lj4 = reinterpret_cast<const float4 *>(s.XL)[j];
        const float hi[3] = {hi4.x, hi4.y, hi4.z}, hj[3] = {hj4.x, hj4.y, hj4.z};
        const float li[3] = {li4.x, li4.y, li4.z}, lj[3] = {lj4.x, lj4.y, lj4.z};
        dfl r2 = {0.0f, 0.0f};
#pragma unroll
        for (int d = 0; d < 3; d++)
            if (d < dim) {
                dfl dd = ts(hi[d], -hj[d]);
                dd = qts(dd.hi, dd.lo + (li[d] - lj[d]));
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
        s.Mp[tri(j) + i] = DF ? df_pack(phi.hi, phi.lo) : df_to_double(phi);
    }
    const AvoidInf<double> AI = avoid_inf_scaled<double>(es);
    for (int i = lane; i < k; i += 32) {
        dfl xd[3];
        for (int d = 0; d < 3; d++) xd[d] = {s.XH[i * 4 + d], s.XL[i * 4 + d]};
        for (int m = 0; m < nmon; m++) {
            dfl v = {1.0f, 0.0f};
            for (int d = 0; d < dim; d++)
                for (int t = 0; t < P.exps[m][d]; t++) v = df_mul(v, xd[d]);
            s.Mp[tri(k + m) + i] = DF ? df_pack(v.hi, v.lo) : df_to_double(v);
        }
        double D[3];
        for (int d = 0; d < dim; d++) D[d] = -s.X[i * 3 + d];
        for (int q = 0; q < nops; q++) {
            const double b = phs_op<double>(P.phs, P.op_code[q], P.op_dim[q], D, dim, AI);
            s.bv[i * nops + q] = DF ? df_pack_double(b) : b;
        }
    }
    for (int t = lane; t < nmon * nops; t += 32) {
        const int m = t / nops, q = t - (t / nops) * nops;
        const double b = mono_op_at_origin(P, m, P.op_code[q], P.op_dim[q]);
        s.bv[(k + m) * nops + q] = DF ? df_pack_double(b) : b;
    }
    __syncwarp();
}

// A(i, j) of the packed symmetric system (packed double-float)
__device__ __forceinline__ double pk_at(const double *Mp, int i, int j) {
    return Mp[i >= j ? tri(i) + j : tri(j) + i];
}

// Hands stencil e to the general refined kernel (its FP64 fallback included).
__device__ __forceinline__ void split_defer(const StencilParams &P, int64_t e, int lane) {
    if (lane == 0) {
        const unsigned long long t = atomicAdd(&P.counters[7], 1ull);
        P.defer[t] = (int32_t)e;
    }
}

template <int N, int R>
struct RegLU {
    static constexpr int ROWS = (N + 31) / 32;
    static constexpr int W = N;  // matrix only; right-hand sides go through reg_apply_inverse
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

// Gauss-Jordan inversion in place with partial pivoting (largest |a|, ties to the lower row;
// the rows not yet used as pivots evolve exactly as in an LU).  Each row slot is a window of
// N registers: before step c it holds columns c..N-1 of the row, then the row's entries of
// the c inverse columns formed so far.  Step c eliminates column c (window position 0) from
// every row but the pivot row, shifts each window left by one and appends the row's entry of
// the new inverse column (minus the multiplier; 1 in the pivot row, which stays unscaled and
// is multiplied by its reciprocal pivot at the end).  Every step runs the same code, so the
// loop stays rolled.  Afterwards the row pivoted at step c holds row c of the inverse, its
// window position t the column of the row pivoted at step t.  rowbuf: two buffers of
// 4 ceil(N/4) floats.  Returns false on a zero, subnormal or non-finite pivot (an entry of the
// inverse that is not finite).
template <int N, int R>
__device__ bool reg_invert(RegLU<N, R> &L, float *rowbuf2, int lane) {
    constexpr int ROWS = RegLU<N, R>::ROWS, W4 = (N + 3) / 4;
    float rsc[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; r++) rsc[r] = 1.0f;
#pragma unroll 1
    for (int c = 0; c < N; c++) {
        float *const rowbuf = rowbuf2 + (c & 1) * 4 * W4;  // alternating: one barrier per step
        unsigned key = 0u;
#pragma unroll
        for (int r = 0; r < ROWS; r++) {
            const unsigned kk = (__float_as_uint(fabsf(L.a[r][0])) & ~63u) | (unsigned)(63 - (lane + 32 * r));
            key = max(key, L.step[r] == N + 1 ? kk : 0u);
        }
        key = __reduce_max_sync(0xffffffffu, key);
        const int brow = 63 - (int)(key & 63u);
#pragma unroll
        for (int r = 0; r < ROWS; r++) {
            if (brow == lane + 32 * r) {
#pragma unroll
                for (int q4 = 0; q4 < W4; q4++) {
                    float4 v;
                    v.x = L.a[r][4 * q4];
                    v.y = 4 * q4 + 1 < N ? L.a[r][4 * q4 + 1 < N ? 4 * q4 + 1 : 0] : 0.0f;
                    v.z = 4 * q4 + 2 < N ? L.a[r][4 * q4 + 2 < N ? 4 * q4 + 2 : 0] : 0.0f;
                    v.w = 4 * q4 + 3 < N ? L.a[r][4 * q4 + 3 < N ? 4 * q4 + 3 : 0] : 0.0f;
                    reinterpret_cast<float4 *>(rowbuf)[q4] = v;
                }
            }
        }
        __syncwarp();
        const float pvt = rowbuf[0];
        // approximate reciprocal (the FP32 inverse only preconditions the refinement); a zero,
        // subnormal (flushed) or non-finite pivot gives an infinite or NaN reciprocal, which
        // reaches the inverse's entries: the check after the loop fails it
        float inv;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(pvt));
#pragma unroll
        for (int r = 0; r < ROWS; r++) {
            const bool pr = brow == lane + 32 * r;
            if (pr) {
                L.step[r] = c;
                rsc[r] = inv;
            }
            const float m = pr ? 0.0f : L.a[r][0] * inv;
#pragma unroll
            for (int q4 = 0; q4 < W4; q4++) {
                const float4 v = reinterpret_cast<const float4 *>(rowbuf)[q4];
                const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int j = 4 * q4 + t;
                    if (j >= 1 && j < N) L.a[r][j - 1 >= 0 ? j - 1 : 0] = fmaf(-m, vv[t], L.a[r][j < N ? j : 0]);
                }
            }
            L.a[r][N - 1] = pr ? 1.0f : -m;
        }
    }
    bool fin = true;
#pragma unroll
    for (int r = 0; r < ROWS; r++)
#pragma unroll
        for (int j = 0; j < N; j++) {
            L.a[r][j] *= rsc[r];
            fin &= isfinite(L.a[r][j]);
        }
    return __all_sync(0xffffffffu, fin);
}

// x = A32^{-1} rhs for the R right-hand sides held per row: every row puts its right-hand
// sides at its pivot step in rp (N x R floats, 16-byte aligned), then each row's dot products
// with the inverse's row are the unknowns at its pivot step, written to xs (N x R).
template <int N, int R>
__device__ void reg_apply_inverse(const RegLU<N, R> &L, const float (&rhs)[RegLU<N, R>::ROWS][R], float *rp,
                                  float *xs, int lane) {
    constexpr int ROWS = RegLU<N, R>::ROWS;
#pragma unroll
    for (int r = 0; r < ROWS; r++)
        if (L.step[r] >= 0)
#pragma unroll
            for (int q = 0; q < R; q++) rp[L.step[r] * R + q] = rhs[r][q];
    __syncwarp();
#pragma unroll
    for (int r = 0; r < ROWS; r++) {
        float acc[R];
#pragma unroll
        for (int q = 0; q < R; q++) acc[q] = 0.0f;
        if constexpr (R == 4) {
#pragma unroll
            for (int j = 0; j < N; j++) {
                const float4 v = reinterpret_cast<const float4 *>(rp)[j];
                acc[0] = fmaf(L.a[r][j], v.x, acc[0]);
                acc[1] = fmaf(L.a[r][j], v.y, acc[1]);
                acc[2] = fmaf(L.a[r][j], v.z, acc[2]);
                acc[3] = fmaf(L.a[r][j], v.w, acc[3]);
            }
        } else {
#pragma unroll
            for (int j = 0; j < N; j++)
#pragma unroll
                for (int q = 0; q < R; q++) acc[q] = fmaf(L.a[r][j], rp[j * R + q], acc[q]);
        }
        if (L.step[r] >= 0)
#pragma unroll
            for (int q = 0; q < R; q++) xs[L.step[r] * R + q] = acc[q];
    }
    __syncwarp();
}

// resident blocks of four warps per SM the register kernels are compiled for: one row slot
// (N <= 32) fits six blocks without spills (78 registers; n = 26 at 2M: 25.4 ms with three
// blocks, 23.4 ms with six), two row slots need three
__host__ __device__ constexpr int reg_kernel_blocks(int n) { return n <= 32 ? 6 : 3; }

template <int N, int R>
__global__ void __launch_bounds__(128, reg_kernel_blocks(N)) build_refined_reg_kernel(StencilParams P, int wpb,
                                                                                        size_t warp_bytes) {
    constexpr int ROWS = RegLU<N, R>::ROWS;
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const SplitSmem s = carve_split(smem + wib * warp_bytes, N, P.k, R);
    float *xs = s.xs;  // N x R floats
    // strict upper-triangle pair table of the RBF block (i < j), shared by the block's warps
    uint16_t *pairs = reinterpret_cast<uint16_t *>(smem + wpb * warp_bytes);
    for (int p = threadIdx.x; p < P.k * (P.k - 1) / 2; p += blockDim.x) {
        int j = 1;
        while ((j + 1) * j / 2 <= p) j++;
        pairs[p] = (uint16_t)((p - j * (j - 1) / 2) | (j << 8));
    }
    __syncthreads();
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P.ne; e += nwarps) {
        // a learned seed is read here, at the top of the stencil, so that its latency hides
        // behind the load and assembly (lane t holds entry t and t + 32; one operator)
        float seed_reg[ROWS];
#pragma unroll
        for (int r = 0; r < ROWS; r++) {
            const int i = lane + 32 * r;
            seed_reg[r] = (R == 1 && P.seed && i < P.k) ? __ldg(&P.seed[e * P.k + i]) : 0.0f;
        }
        // boundary stencils (Hermite rows) go to the general refined kernel
        int es = 0;
        if (load_interior(P, e, s, lane, &es) != 0) {
            split_defer(P, e, lane);
            __syncwarp();
            continue;
        }
        assemble_packed<true>(P, s, lane, es, pairs);
        RegLU<N, R> L;
#pragma unroll
        for (int r = 0; r < ROWS; r++) {
            const int i = lane + 32 * r;
            const bool act = i < N;
            L.step[r] = act ? N + 1 : -1;
#pragma unroll
            for (int cc = 0; cc < N; cc++) L.a[r][cc] = act ? df_hi(pk_at(s.Mp, act ? i : 0, cc)) : 0.0f;
        }
        // start of the refinement: x0 = 0 and rhs = b, or with a learned seed x0 = [w_pred; 0]
        // and rhs = b - A32 x0, formed here from the FP32 rows while they are still unfactored
        float rhs[ROWS][R];
        if (P.seed) {
            if constexpr (R == 1) {
#pragma unroll
                for (int r = 0; r < ROWS; r++) {
                    const int t = lane + 32 * r;
                    if (t < N) {
                        xs[t] = seed_reg[r];
                        s.x[t] = df_pack(seed_reg[r], 0.0f);
                    }
                }
            } else {
                for (int t = lane; t < N * R; t += 32) {
                    const int i = t / R;
                    const float sv = i < P.k ? __ldg(&P.seed[e * P.k + i]) : 0.0f;
                    xs[t] = sv;
                    s.x[t] = df_pack(sv, 0.0f);
                }
            }
            __syncwarp();
#pragma unroll
            for (int r = 0; r < ROWS; r++) {
                const int i = lane + 32 * r;
#pragma unroll
                for (int q = 0; q < R; q++) {
                    float acc = i < N ? df_hi(s.bv[(i < N ? i : 0) * R + q]) : 0.0f;
                    static_for<0, N, 1>([&](auto jI) {
                        constexpr int j = decltype(jI)::value;
                        acc = fmaf(-L.a[r][j], xs[j * R + q], acc);
                    });
                    rhs[r][q] = acc;
                }
            }
        } else {
            for (int t = lane; t < N * R; t += 32) s.x[t] = 0.0;
#pragma unroll
            for (int r = 0; r < ROWS; r++) {
                const int i = lane + 32 * r;
#pragma unroll
                for (int q = 0; q < R; q++) rhs[r][q] = i < N ? df_hi(s.bv[(i < N ? i : 0) * R + q]) : 0.0f;
            }
        }
        __syncwarp();
        const bool ok = reg_invert<N, R>(L, s.rowbuf, lane);
        bool accepted = false;
        double est_final = 0.0;
        int nres = 0;
        if (ok) {
            // double-float residual r = b - A x into rhs; rows k..N-1 are the polynomial
            // reproduction constraints.  The N x N products are spread evenly over the warp as
            // (row, block of JB columns) pairs; partial sums meet by shuffles and the row owner
            // picks its entry up from shared memory.
            auto residual = [&]() {
                nres++;
                constexpr int JB = residual_blocks(N);
                constexpr int JL = (N + JB - 1) / JB;
                float *rbuf = xs;  // N x R floats, free until the next solve
#pragma unroll 1
                for (int pass = 0; pass < (N * JB + 31) / 32; pass++) {
                    const int pr = pass * 32 + lane;
                    const int i = pr / JB, jb = pr % JB;
                    DfSum acc[R];
#pragma unroll
                    for (int q = 0; q < R; q++) acc[q] = {0.0f, 0.0f};
                    if (i < N) {
                        const int j0 = jb * JL;
                        const int ti = tri(i);
#pragma unroll 2
                        for (int jj = 0; jj < JL; jj++) {
                            const int j = j0 + jj;
                            if (j < N) {
                                const double aij = s.Mp[j <= i ? ti + j : tri(j) + i];
#pragma unroll
                                for (int q = 0; q < R; q++) dfsum_sub(acc[q], aij, s.x[j * R + q]);
                            }
                        }
                    }
#pragma unroll
                    for (int o = JB / 2; o > 0; o >>= 1)
#pragma unroll
                        for (int q = 0; q < R; q++) acc[q] = dfsum_xor(acc[q], o);
                    if (i < N && jb == 0)
#pragma unroll
                        for (int q = 0; q < R; q++)
                            rbuf[i * R + q] = dfsum_value(dfsum_merge(dfsum_of(s.bv[i * R + q]), acc[q]));
                }
                __syncwarp();
#pragma unroll
                for (int r = 0; r < ROWS; r++) {
                    const int i = lane + 32 * r;
#pragma unroll
                    for (int q = 0; q < R; q++) rhs[r][q] = i < N ? rbuf[(i < N ? i : 0) * R + q] : 0.0f;
                }
                __syncwarp();
            };
            // After acceptance: the polynomial-reproduction rows (k..N-1) once more, in FP64 on
            // the weights unpacked to FP64, and one correction through the inverse.  A product
            // with a Gauss-Jordan inverse is not backward stable: it leaves a residual of about
            // cond * 2^-24 of the last step, and in these rows that residual breaks the exact
            // reproduction of polynomials, which the apply of a smooth field amplifies by
            // sum |w|.  The double-float residuals leave ~2^-45 sum |a x| in these rows, which
            // the same amplification would make visible, so this pass is FP64 (ten rows of k
            // products).  Only the k columns of P enter (the rows' other block is zero); the
            // rows share the warp's lanes in one pass.
            auto polish_rhs = [&]() {
                const int k = P.k, nm = N - k;
                for (int t = lane; t < k * R; t += 32) s.x[t] = df_unpack_double(s.x[t]);  // the weights
                __syncwarp();
                // lane (t, h): row k + t, column block h of c3 blocks (c3 lanes per row)
                const int c3 = nm >= 32 ? 1 : 32 / nm, cw = (k + c3 - 1) / c3;
                const int t0 = lane / c3, h = lane - t0 * c3;
                float *rbuf = xs;
                for (int tb = 0; tb < nm; tb += 32 / c3) {
                    const int t = tb + t0;
                    double acc[R];
#pragma unroll
                    for (int q = 0; q < R; q++) acc[q] = 0.0;
                    if (t < nm && t0 < 32 / c3) {
                        const int ti2 = tri(k + t);
                        for (int jj = 0; jj < cw; jj++) {
                            const int j = h * cw + jj;
                            if (j < k) {
                                const double a = df_unpack_double(s.Mp[ti2 + j]);
#pragma unroll
                                for (int q = 0; q < R; q++) acc[q] = fma(-a, s.x[j * R + q], acc[q]);
                            }
                        }
                    }
                    for (int o = 1; o < c3; o++) {
#pragma unroll
                        for (int q = 0; q < R; q++) {
                            const double v = __shfl_down_sync(0xffffffffu, acc[q], o);
                            if (h == 0) acc[q] += v;
                        }
                    }
                    if (t < nm && t0 < 32 / c3 && h == 0)
#pragma unroll
                        for (int q = 0; q < R; q++)
                            rbuf[(k + t) * R + q] = __double2float_rn(df_unpack_double(s.bv[(k + t) * R + q]) + acc[q]);
                }
                __syncwarp();
#pragma unroll
                for (int r = 0; r < ROWS; r++) {
                    const int i = lane + 32 * r;
#pragma unroll
                    for (int q = 0; q < R; q++) rhs[r][q] = (i >= k && i < N) ? rbuf[(i < N ? i : 0) * R + q] : 0.0f;
                }
                __syncwarp();
            };  // the loop below applies the inverse to these right-hand sides and corrects the weights
            // the first solve leaves an error at the FP32 floor (about cond(A) * 2^-24
            // relative) from any start: a seed cannot beat it, so it costs no residual
            // One call site of the product with the inverse serves the refinement steps and the
            // polish (the kernel's code size sets its instruction-fetch stalls).
            const float tolf = (float)P.tol;
            float dprev = 0.0f;
            bool polishing = false;
            for (int step = 0;; step++) {
                reg_apply_inverse<N, R>(L, rhs, s.rowbuf, xs, lane);
                if (polishing) {
                    for (int t = lane; t < P.k * R; t += 32) s.x[t] += widen(xs[t]);  // the weights, FP64
                    __syncwarp();
                    break;
                }
                float dmaxf = 0.0f, xmaxf = 0.0f;
                for (int t = lane; t < N * R; t += 32) {
                    const float d = xs[t];
                    s.x[t] = df_add_f(s.x[t], d);
                    if (t / R < P.k) {
                        dmaxf = fmaxf(dmaxf, fabsf(d));
                        xmaxf = fmaxf(xmaxf, fabsf(df_hi(s.x[t])));
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
            WarpSmem w;  // the polish left the weights in FP64
            w.cols = s.cols;
            scatter_row(P, e, w, lane, es, s.x, R, 1);
            if (lane == 0) {
                if (P.status) P.status[e] = 0;
                atomicMax(reinterpret_cast<unsigned long long *>(P.max_resid),
                          (unsigned long long)__double_as_longlong(est_final));
            }
        } else {
            split_defer(P, e, lane);  // the general kernel's refinement, then its FP64 fallback
        }
        __syncwarp();
    }
}

// Launches the register kernel; the caller finishes the stencils it hands over (boundary
// stencils, failed refinements: P.defer, counted in P.counters[7]) with the general kernel.
template <int N, int R>
int launch_refined_reg(rbf_ctx *ctx, const StencilParams &P) {
    if (!P.defer) return rbf_fail(ctx, RBF_ERR_INTERNAL, "register kernel without a deferred list");
    const size_t wb = split_smem_bytes(N, P.k, R);
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
