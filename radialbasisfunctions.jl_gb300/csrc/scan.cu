// Device-wide exclusive prefix sums (row pointers, cell starts) and small
// bookkeeping kernels shared by the build and the neighbour search.
#include <algorithm>

#include "rbf_internal.cuh"

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <class T>
__device__ T block_exclusive_scan(T v, T *smem_warp, T *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = (lane < (int)(blockDim.x >> 5)) ? smem_warp[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        smem_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    T warp_off = warp > 0 ? smem_warp[warp - 1] : T(0);
    *total = smem_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_off + x - v;
}

template <class T>
__global__ void tile_sums_kernel(const T *__restrict__ in, int64_t n, T *__restrict__ sums) {
    __shared__ T sw[32];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    T acc = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        int64_t idx = base + (int64_t)threadIdx.x * SCAN_ITEMS + i;
        if (idx < n) acc += in[idx];
    }
    T tot;
    block_exclusive_scan<T>(acc, sw, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <class T>
__global__ void tile_scan_kernel(const T *__restrict__ in, int64_t n, const T *__restrict__ offs,
                                 T *__restrict__ out) {
    __shared__ T sw[32];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    T vals[SCAN_ITEMS];
    T acc = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        int64_t idx = base + (int64_t)threadIdx.x * SCAN_ITEMS + i;
        vals[i] = idx < n ? in[idx] : T(0);
        acc += vals[i];
    }
    T tot;
    T ex = block_exclusive_scan<T>(acc, sw, &tot);
    T run = ex + (offs ? offs[blockIdx.x] : T(0));
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        int64_t idx = base + (int64_t)threadIdx.x * SCAN_ITEMS + i;
        if (idx < n) out[idx] = run;
        run += vals[i];
    }
}

template <class T>
int exclusive_scan(rbf_ctx *ctx, const T *d_in, T *d_out, int64_t n, T *d_total_or_null,
                   int64_t *host_total) {
    if (n <= 0) {
        if (host_total) *host_total = 0;
        return RBF_OK;
    }
    int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    DevBuf sums, offs;
    RBF_TRY(sums.alloc(ctx, sizeof(T) * (tiles + 1)));
    RBF_TRY(offs.alloc(ctx, sizeof(T) * (tiles + 1)));
    tile_sums_kernel<T><<<(unsigned)tiles, SCAN_THREADS, 0, ctx->stream>>>(d_in, n, sums.as<T>());
    RBF_CHECK_LAUNCH(ctx);
    if (tiles > 1) {
        RBF_TRY(exclusive_scan<T>(ctx, sums.as<T>(), offs.as<T>(), tiles, nullptr, nullptr));
    } else {
        RBF_CUDA(ctx, cudaMemsetAsync(offs.as<T>(), 0, sizeof(T), ctx->stream));
    }
    tile_scan_kernel<T><<<(unsigned)tiles, SCAN_THREADS, 0, ctx->stream>>>(d_in, n, offs.as<T>(), d_out);
    RBF_CHECK_LAUNCH(ctx);
    if (host_total) {
        T last_in, last_out;
        RBF_CUDA(ctx, cudaMemcpyAsync(&last_in, d_in + (n - 1), sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
        RBF_CUDA(ctx, cudaMemcpyAsync(&last_out, d_out + (n - 1), sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
        RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        *host_total = (int64_t)last_in + (int64_t)last_out;
    }
    (void)d_total_or_null;
    return RBF_OK;
}

// rows: Dirichlet eval rows (boundary point with alpha == 1, beta == 0) hold one entry,
// every other row holds k (src/solve/execution.jl:39-69); with adj_idx (the normal-derivative
// formulation) k plus one du/dn entry per Neumann/Robin neighbour.
__global__ void row_counts_kernel(int64_t ne, int k, const uint8_t *__restrict__ isb,
                                  const int32_t *__restrict__ g2b, const double *__restrict__ alpha,
                                  const double *__restrict__ beta, int64_t *__restrict__ cnt,
                                  const int64_t *__restrict__ adj_ptr, const int32_t *__restrict__ adj_idx) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = adj_ptr ? adj_ptr[e + 1] - adj_ptr[e] : k;
        bool dirichlet_eval = false;
        if (isb && isb[e]) {
            int32_t b = g2b[e];
            dirichlet_eval = alpha[b] == 1.0 && beta[b] == 0.0;
        }
        if (dirichlet_eval) {
            c = 1;
        } else if (adj_idx && isb) {
            for (int64_t t = adj_ptr[e]; t < adj_ptr[e + 1]; t++) {
                const int32_t g = adj_idx[t];
                if (isb[g]) {
                    const int32_t b = g2b[g];
                    c += !(alpha[b] == 1.0 && beta[b] == 0.0);
                }
            }
        }
        cnt[e] = c;
    }
}

__global__ void flag_to_i32_kernel(int64_t n, const uint8_t *__restrict__ f, int32_t *__restrict__ o) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        o[i] = f[i] ? 1 : 0;
}

__global__ void g2b_finish_kernel(int64_t n, const uint8_t *__restrict__ f, int32_t *__restrict__ g) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (!f[i]) g[i] = -1;
}

__global__ void index_range_kernel(const int32_t *__restrict__ idx, int64_t n, int32_t hi, int *__restrict__ bad) {
    int local = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t v = idx[i];
        local |= (v < 0 || v >= hi);
    }
    if (__any_sync(0xffffffffu, local) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

}  // namespace

int rbf_check_indices(rbf_ctx *ctx, const int32_t *d_idx, int64_t n, int32_t hi, bool *ok) {
    DevBuf flag;
    RBF_TRY(flag.alloc(ctx, sizeof(int)));
    RBF_CUDA(ctx, cudaMemsetAsync(flag.ptr, 0, sizeof(int), ctx->stream));
    int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8);
    if (blocks < 1) blocks = 1;
    index_range_kernel<<<blocks, 256, 0, ctx->stream>>>(d_idx, n, hi, flag.as<int>());
    RBF_CHECK_LAUNCH(ctx);
    int h = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&h, flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *ok = (h == 0);
    return RBF_OK;
}

int rbf_exclusive_scan_i64(rbf_ctx *ctx, const int64_t *d_in, int64_t *d_out, int64_t n, int64_t *total) {
    return exclusive_scan<int64_t>(ctx, d_in, d_out, n, nullptr, total);
}

int rbf_exclusive_scan_i32(rbf_ctx *ctx, const int32_t *d_in, int32_t *d_out, int64_t n, int64_t *total) {
    return exclusive_scan<int32_t>(ctx, d_in, d_out, n, nullptr, total);
}

int rbf_boundary_map_device(rbf_ctx *ctx, int64_t n, const uint8_t *d_isb, int32_t *d_g2b,
                            int64_t *n_boundary) {
    DevBuf flags;
    RBF_TRY(flags.alloc(ctx, sizeof(int32_t) * (n + 1)));
    int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8);
    if (blocks < 1) blocks = 1;
    flag_to_i32_kernel<<<blocks, 256, 0, ctx->stream>>>(n, d_isb, flags.as<int32_t>());
    RBF_CHECK_LAUNCH(ctx);
    RBF_TRY(rbf_exclusive_scan_i32(ctx, flags.as<int32_t>(), d_g2b, n, n_boundary));
    g2b_finish_kernel<<<blocks, 256, 0, ctx->stream>>>(n, d_isb, d_g2b);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_count_rows_device(rbf_ctx *ctx, int64_t ne, int k, const uint8_t *d_isb, const int32_t *d_g2b,
                          const double *d_alpha, const double *d_beta, int64_t *d_row_ptr, int64_t *nnz,
                          const int64_t *d_adj_ptr, const int32_t *d_adj_idx) {
    DevBuf cnt;
    RBF_TRY(cnt.alloc(ctx, sizeof(int64_t) * (ne + 1)));
    int blocks = (int)std::min<int64_t>((ne + 255) / 256, (int64_t)ctx->num_sms * 8);
    if (blocks < 1) blocks = 1;
    row_counts_kernel<<<blocks, 256, 0, ctx->stream>>>(ne, k, d_isb, d_g2b, d_alpha, d_beta, cnt.as<int64_t>(),
                                                     d_adj_ptr, d_adj_idx);
    RBF_CHECK_LAUNCH(ctx);
    RBF_CUDA(ctx, cudaMemsetAsync(cnt.as<int64_t>() + ne, 0, sizeof(int64_t), ctx->stream));
    // scan over ne+1 entries so that row_ptr[ne] is the total
    RBF_TRY(rbf_exclusive_scan_i64(ctx, cnt.as<int64_t>(), d_row_ptr, ne + 1, nnz));
    return RBF_OK;
}
