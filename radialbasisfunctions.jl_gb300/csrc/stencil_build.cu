// Weight build kernels: one warp per stencil, the saddle-point system staged in shared
// memory, and the scatter of the solved row into its CSR slot with columns ascending.
//   plain FP64:        LU with partial pivoting in FP64.
//   FP32 + refinement: the same FP64 assembly is rounded to FP32 and factorised there;
//                      iterative refinement with FP64 residuals (including the polynomial
//                      reproduction rows P^T w = L(p)) recovers FP64 accuracy, and a stencil
//                      whose normwise backward error stays above tolerance is re-solved by
//                      the plain FP64 LU (status 3).
//
// Replaces the per-stencil loop of launch_kernel! (src/solve/execution.jl:186-265):
// classify_stencil (src/solve/types.jl:208-223), _build_stencil! /
// _build_collocation_matrix_impl! / _build_rhs! (src/solve/assembly.jl:95-217),
// _solve_system! (assembly.jl:220-222, rook Bunch-Kaufman on the raw-coordinate
// system), fill_entries! / fill_dirichlet_entry! (execution.jl:279-303) and the COO->CSC
// sort of _construct_sparse (execution.jl:105-115).  Assembly happens in scaled local
// coordinates (stencil_common.cuh), which gives the same weights to within rounding.
//
// Shared memory per warp: M[n][ld] (ld = n + nops: matrix | right-hand sides), local
// coordinates X[k][3], Hermite data (alpha, beta/s, normal, point type) and the k column
// indices.  Dominant cost: the LU update, n^3/3 FP64 FMA per stencil.
#include <algorithm>
#include <cmath>

#include "stencil_bk.cuh"
#include "stencil_solve.cuh"

#define RBF_LAUNCH_NO_VARIANT 1000
int rbf_launch_refined_reg_a(rbf_ctx *ctx, const StencilParams &P);
int rbf_launch_refined_reg_b(rbf_ctx *ctx, const StencilParams &P);
int rbf_launch_refined_split(rbf_ctx *ctx, const StencilParams &P);

namespace {

__global__ void build_fp64_kernel(StencilParams P, int wpb, size_t warp_bytes) {
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WarpSmem w = carve(smem + wib * warp_bytes, P.n, P.k, P.nops);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P.ne; e += nwarps) solve_fp64_warp(P, e, w, lane);
}

// The default plain FP64 build: symmetric indefinite factorisation of the packed system
// (stencil_bk.cuh), one warp per stencil.
__global__ void build_fp64_bk_kernel(StencilParams P, int wpb, size_t warp_bytes) {
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const BKSmem s = carve_bk(smem + wib * warp_bytes, P.n, P.k, P.nops);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P.ne; e += nwarps) solve_fp64_bk_warp(P, e, s, lane);
}

__global__ void build_fp32r_kernel(StencilParams P, int wpb, size_t warp_bytes) {
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    char *base = smem + wib * warp_bytes;
    WarpSmem w = carve(base, P.n, P.k, P.nops);
    Warp32 u = carve32(base, P.n, P.k, P.nops);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t e = (int64_t)blockIdx.x * wpb + wib; e < P.ne; e += nwarps) solve_fp32r_warp(P, e, w, u, lane);
}

// Stencils the split-row kernel handed over (boundary stencils, failed refinements): the
// general refined solve with its FP64 fallback.  The count is read on the device, so the
// launch needs no host synchronisation (and can be captured in a graph).
__global__ void build_deferred_kernel(StencilParams P, int wpb, size_t warp_bytes) {
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    char *base = smem + wib * warp_bytes;
    WarpSmem w = carve(base, P.n, P.k, P.nops);
    Warp32 u = carve32(base, P.n, P.k, P.nops);
    const int64_t count = (int64_t)*reinterpret_cast<volatile unsigned long long *>(&P.counters[7]);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t t = (int64_t)blockIdx.x * wpb + wib; t < count; t += nwarps) solve_fp32r_warp(P, P.defer[t], w, u, lane);
}

int launch_deferred(rbf_ctx *ctx, const StencilParams &P) {
    const size_t wb = warp_smem_bytes32(P.n, P.k, P.nops);
    int wpb = (int)std::max<size_t>(1, std::min<size_t>(8, (100 * 1024) / wb));
    size_t smem = wb * wpb;
    RBF_CUDA(ctx, cudaFuncSetAttribute(build_deferred_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_deferred_kernel, wpb * 32, smem));
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = std::min<int64_t>((P.ne + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
    build_deferred_kernel<<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P, wpb, wb);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

}  // namespace

size_t rbf_fp64_warp_smem(int n, int k, int nops) { return (warp_smem_bytes(n, k, nops) + 15) & ~(size_t)15; }

int rbf_build_fp64_launch(rbf_ctx *ctx, const StencilParams &P) {
    if (P.ne == 0) return RBF_OK;
    if (!(P.flags & RBF_FLAG_FP64_LU)) {
        const size_t wb = bk_warp_bytes(P.n, P.k, P.nops);
        const int wpb = 4;
        const size_t smem = wb * wpb;
        RBF_CUDA(ctx, cudaFuncSetAttribute(build_fp64_bk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
        int per_sm = 0;
        RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_fp64_bk_kernel, wpb * 32, smem));
        if (per_sm < 1) per_sm = 1;
        const int64_t blocks = std::min<int64_t>((P.ne + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
        build_fp64_bk_kernel<<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P, wpb, wb);
        RBF_CHECK_LAUNCH(ctx);
        return RBF_OK;
    }
    const size_t wb = rbf_fp64_warp_smem(P.n, P.k, P.nops);
    int wpb = (int)std::max<size_t>(1, std::min<size_t>(8, (100 * 1024) / wb));
    size_t smem = wb * wpb;
    RBF_CUDA(ctx, cudaFuncSetAttribute(build_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_fp64_kernel, wpb * 32, smem));
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = std::min<int64_t>((P.ne + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
    build_fp64_kernel<<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P, wpb, wb);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_build_fp32_launch(rbf_ctx *ctx, const StencilParams &P) {
    if (P.ne == 0) return RBF_OK;
    // 40-row single-operator systems: the split-row kernel on the interior stencils, then the
    // general kernel on the ones it deferred (every FP32 build passes a deferred list)
    if (P.defer) {
        const int st = rbf_launch_refined_split(ctx, P);
        if (st != RBF_LAUNCH_NO_VARIANT) {
            if (st != RBF_OK) return st;
            return launch_deferred(ctx, P);
        }
    }
    // register-resident kernels for the standard system sizes on the interior stencils, then
    // the general kernel on the ones they deferred
    if (P.defer) {
        int st = rbf_launch_refined_reg_a(ctx, P);
        if (st == RBF_LAUNCH_NO_VARIANT) st = rbf_launch_refined_reg_b(ctx, P);
        if (st != RBF_LAUNCH_NO_VARIANT) {
            if (st != RBF_OK) return st;
            return launch_deferred(ctx, P);
        }
    }
    const size_t wb = warp_smem_bytes32(P.n, P.k, P.nops);
    int wpb = (int)std::max<size_t>(1, std::min<size_t>(8, (100 * 1024) / wb));
    size_t smem = wb * wpb;
    RBF_CUDA(ctx, cudaFuncSetAttribute(build_fp32r_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_fp32r_kernel, wpb * 32, smem));
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = std::min<int64_t>((P.ne + wpb - 1) / wpb, (int64_t)ctx->num_sms * per_sm);
    build_fp32r_kernel<<<(unsigned)blocks, wpb * 32, smem, ctx->stream>>>(P, wpb, wb);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}
