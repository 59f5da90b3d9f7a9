// Locality reordering of a point cloud (replaces reorder_points!, src/utils.jl:45-55).
//
// The reference permutes the points by a symmetric reverse Cuthill-McKee ordering of the
// stencil graph so that the neighbours of a point have nearby indices; its test pins only
// the contract (a permutation p with x_new = x_old[p], test/utils.jl:61-78).  Here points
// are ordered along a Morton (Z-order) curve over a uniform grid of about two points per
// cell: a cell's neighbours are mostly a few cells away along the curve, so after the
// permutation the x values a stencil row gathers in the apply lie in a few cache lines and
// consecutive rows reuse them.  Counting sort on the Morton cell code (histogram, scan,
// scatter), then each cell's points in ascending original index, so the result is
// deterministic (for cells of up to 256 points: any non-degenerate cloud).
#include <algorithm>
#include <cmath>
#include <vector>

#include "rbf_internal.cuh"

namespace {

__global__ void bounds_kernel(const double *__restrict__ x, int64_t n, int dim, double *__restrict__ part) {
    __shared__ double s[6][256];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < dim; d++) {
            const double v = x[i * dim + d];
            mn[d] = fmin(mn[d], v);
            mx[d] = fmax(mx[d], v);
        }
    for (int d = 0; d < 3; d++) {
        s[d][threadIdx.x] = mn[d];
        s[3 + d][threadIdx.x] = mx[d];
    }
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int d = 0; d < 3; d++) {
                s[d][threadIdx.x] = fmin(s[d][threadIdx.x], s[d][threadIdx.x + h]);
                s[3 + d][threadIdx.x] = fmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + h]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
}

// spread the low 10 (3D) / 16 (2D) bits of v so that dim-1 zero bits separate them
__device__ __forceinline__ uint32_t spread(uint32_t v, int dim) {
    if (dim == 1) return v;
    if (dim == 2) {
        v &= 0xffffu;
        v = (v | (v << 8)) & 0x00ff00ffu;
        v = (v | (v << 4)) & 0x0f0f0f0fu;
        v = (v | (v << 2)) & 0x33333333u;
        v = (v | (v << 1)) & 0x55555555u;
        return v;
    }
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

struct MortonGrid {
    double lo[3], inv_h[3];
    int bits;  // bits per dimension; cells = 2^(bits*dim)
};

__global__ void morton_count_kernel(MortonGrid g, const double *__restrict__ x, int64_t n, int dim,
                                    uint32_t *__restrict__ code, int32_t *__restrict__ count) {
    const uint32_t top = (1u << g.bits) - 1u;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t c = 0;
        for (int d = 0; d < dim; d++) {
            const double f = floor((x[i * dim + d] - g.lo[d]) * g.inv_h[d]);
            uint32_t q = !(f >= 0.0) ? 0u : (f >= (double)top ? top : (uint32_t)f);
            c |= spread(q, dim) << d;
        }
        code[i] = c;
        atomicAdd(&count[c], 1);
    }
}

__global__ void morton_scatter_kernel(int64_t n, const uint32_t *__restrict__ code, const int32_t *__restrict__ start,
                                      int32_t *__restrict__ fill, int32_t *__restrict__ perm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = code[i];
        perm[start[c] + atomicAdd(&fill[c], 1)] = (int32_t)i;
    }
}

// insertion sort of each cell's (few) entries by original index; a cell of more than
// kMaxSorted points (only a degenerate cloud crowds one) keeps its scatter order, which
// bounds the work per thread
constexpr int kMaxSorted = 256;
__global__ void cell_sort_kernel(int64_t ncells, const int32_t *__restrict__ start, const int32_t *__restrict__ count,
                                 int32_t *__restrict__ perm) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
        const int32_t s = start[c], m = count[c];
        if (m > kMaxSorted) continue;
        for (int a = 1; a < m; a++) {
            const int32_t v = perm[s + a];
            int b = a - 1;
            while (b >= 0 && perm[s + b] > v) {
                perm[s + b + 1] = perm[s + b];
                b--;
            }
            perm[s + b + 1] = v;
        }
    }
}

__global__ void permute_points_kernel(int64_t n, int dim, const int32_t *__restrict__ perm,
                                      const double *__restrict__ x, double *__restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * dim; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = i / dim;
        y[i] = x[(int64_t)perm[p] * dim + (i - p * dim)];
    }
}

int nblocks(rbf_ctx *ctx, int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 16));
}

}  // namespace

// perm (device, n): x_new[i] = x[perm[i]]; data_out (device, optional): the permuted points
int rbf_reorder_device(rbf_ctx *ctx, const double *d_x, int64_t n, int dim, int32_t *d_perm, double *d_out) {
    if (n == 0) return RBF_OK;
    const int pb = (int)std::min<int64_t>((n + 255) / 256, 1024);
    DevBuf part;
    RBF_TRY(part.alloc(ctx, sizeof(double) * 6 * pb));
    bounds_kernel<<<pb, 256, 0, ctx->stream>>>(d_x, n, dim, part.as<double>());
    RBF_CHECK_LAUNCH(ctx);
    std::vector<double> hp(6 * (size_t)pb);
    RBF_CUDA(ctx, cudaMemcpyAsync(hp.data(), part.ptr, sizeof(double) * 6 * pb, cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    MortonGrid g{};
    // about two points per cell, at most 10 (3D) / 16 (2D) / 30 (1D) bits per dimension
    const int maxbits = dim == 3 ? 10 : (dim == 2 ? 16 : 30);
    int bits = (int)std::ceil(std::log2(std::max(2.0, std::pow((double)n / 2.0, 1.0 / dim))));
    bits = std::max(1, std::min(bits, maxbits));
    while (bits > 1 && bits * dim > 27) bits--;  // at most 2^27 cells
    g.bits = bits;
    for (int d = 0; d < 3; d++) {
        double lo = INFINITY, hi = -INFINITY;
        for (int b = 0; b < pb; b++) {
            lo = std::min(lo, hp[b * 6 + d]);
            hi = std::max(hi, hp[b * 6 + 3 + d]);
        }
        if (d < dim && (!std::isfinite(lo) || !std::isfinite(hi)))
            return rbf_fail(ctx, RBF_ERR_ARGUMENT, "data points contain non-finite coordinates");
        g.lo[d] = d < dim ? lo : 0.0;
        g.inv_h[d] = (d < dim && hi > lo) ? (double)(1u << bits) / (hi - lo) : 0.0;
    }
    const int64_t ncells = (int64_t)1 << (bits * dim);
    DevBuf code, count, start, fill;
    RBF_TRY(code.alloc(ctx, sizeof(uint32_t) * n));
    RBF_TRY(count.alloc(ctx, sizeof(int32_t) * (ncells + 1)));
    RBF_TRY(start.alloc(ctx, sizeof(int32_t) * (ncells + 1)));
    RBF_TRY(fill.alloc(ctx, sizeof(int32_t) * ncells));
    RBF_CUDA(ctx, cudaMemsetAsync(count.ptr, 0, sizeof(int32_t) * (ncells + 1), ctx->stream));
    RBF_CUDA(ctx, cudaMemsetAsync(fill.ptr, 0, sizeof(int32_t) * ncells, ctx->stream));
    morton_count_kernel<<<nblocks(ctx, n), 256, 0, ctx->stream>>>(g, d_x, n, dim, code.as<uint32_t>(),
                                                                  count.as<int32_t>());
    RBF_CHECK_LAUNCH(ctx);
    int64_t total = 0;
    RBF_TRY(rbf_exclusive_scan_i32(ctx, count.as<int32_t>(), start.as<int32_t>(), ncells + 1, &total));
    morton_scatter_kernel<<<nblocks(ctx, n), 256, 0, ctx->stream>>>(n, code.as<uint32_t>(), start.as<int32_t>(),
                                                                    fill.as<int32_t>(), d_perm);
    RBF_CHECK_LAUNCH(ctx);
    cell_sort_kernel<<<nblocks(ctx, ncells), 256, 0, ctx->stream>>>(ncells, start.as<int32_t>(), count.as<int32_t>(),
                                                                    d_perm);
    RBF_CHECK_LAUNCH(ctx);
    if (d_out) {
        permute_points_kernel<<<nblocks(ctx, n * dim), 256, 0, ctx->stream>>>(n, dim, d_perm, d_x, d_out);
        RBF_CHECK_LAUNCH(ctx);
    }
    return RBF_OK;
}

extern "C" int rbf_reorder_points(rbf_ctx *ctx, const double *data, int64_t n, int32_t dim, int32_t *perm_out,
                                  double *data_out) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    if (dim < 1 || dim > 3) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "dim must be 1, 2 or 3 (got %d)", dim);
    if (n < 0 || n >= INT32_MAX) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "point counts must be < 2^31");
    if (!data || !perm_out) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null array");
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != ctx->device) RBF_CUDA(ctx, cudaSetDevice(ctx->device));
    InArray d;
    RBF_TRY(d.bind(ctx, data, sizeof(double) * n * dim));
    OutArray p, o;
    RBF_TRY(p.bind(ctx, perm_out, sizeof(int32_t) * n));
    if (data_out) RBF_TRY(o.bind(ctx, data_out, sizeof(double) * n * dim));
    RBF_TRY(rbf_reorder_device(ctx, d.as<double>(), n, dim, p.as<int32_t>(), data_out ? o.as<double>() : nullptr));
    RBF_TRY(p.finish(ctx));
    if (data_out) RBF_TRY(o.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}
