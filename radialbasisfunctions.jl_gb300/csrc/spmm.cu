// Sparse apply Y = alpha * W X + beta * Y (replaces _eval_op / mul!,
// src/operators/operators.jl:217-218 and 529-542, a SparseMatrixCSC product) and the
// CSR -> CSC transpose (the layout _construct_sparse returns, src/solve/execution.jl:105-115).
//
// Single field: a group of TPR lanes per row; the groups of a warp cover consecutive rows,
// so val/col are streamed contiguously and each lane keeps several loads in flight.
// Several interleaved fields (X[i*ldx + f]): lanes are fields, a row's (val, col) pair is
// a broadcast load and each gather of x is one contiguous run of nf doubles.
// Column-major fields (a Julia Matrix) are transposed to interleaved scratch first.
// Roofline: HBM bandwidth; algorithmic bytes nnz*(8+4) + (ne+1)*8 + nf*(ns+ne)*8.
#include <algorithm>
#include <mutex>

#include "rbf_internal.cuh"

namespace {

template <int TPR, int U>
__global__ void __launch_bounds__(256) spmv_kernel(int64_t ne, const int64_t *__restrict__ rp,
                                                   const int32_t *__restrict__ col,
                                                   const double *__restrict__ val,
                                                   const double *__restrict__ x, double alpha, double beta,
                                                   double *__restrict__ y) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int sub = threadIdx.x % TPR;
    const int64_t groups = (int64_t)gridDim.x * blockDim.x / TPR;
    // warp-uniform trip count: every lane of a warp runs the same iterations
    const int64_t first = (tid / 32) * (32 / TPR);
    for (int64_t r0 = first; r0 < ne; r0 += groups) {
        const int64_t r = r0 + (threadIdx.x & 31) / TPR;
        const bool live = r < ne;
        const int64_t a = live ? __ldg(&rp[r]) : 0, b = live ? __ldg(&rp[r + 1]) : 0;
        double s = 0.0;
        // U entries per lane per chunk: all column and value loads issue first, then all
        // gathers, so each lane has U independent gathers in flight
        for (int64_t p0 = a + sub; p0 < b; p0 += (int64_t)U * TPR) {
            int32_t c[U];
            double v[U], xv[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int64_t p = p0 + (int64_t)u * TPR;
                c[u] = p < b ? __ldg(&col[p]) : -1;
                v[u] = p < b ? __ldg(&val[p]) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < U; u++) xv[u] = c[u] >= 0 ? __ldg(&x[c[u]]) : 0.0;
#pragma unroll
            for (int u = 0; u < U; u++) s = fma(v[u], xv[u], s);
        }
#pragma unroll
        for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
        if (sub == 0 && live) y[r] = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * y[r]);
    }
}

// Single field with paired loads: a row's entries are read two at a time (int2 columns,
// double2 values; an odd row start takes one scalar head entry first), which halves the
// load instructions per nonzero.  Lane sub of a row handles pairs sub, sub + TPR, ... (U per
// chunk), and each lane works on S rows at once (S independent load chains in flight).
// Rows are taken in contiguous ranges, so that in a locality order the x values an SM
// gathers stay in its L1: per warp (BLOCK_RANGE false), or per block with its warps
// interleaved in the range (BLOCK_RANGE true: all warps of a block share one window of x).
template <int TPR, int U, int S, bool BLOCK_RANGE>
__global__ void __launch_bounds__(256) spmv_pair_kernel(int64_t ne, const int64_t *__restrict__ rp,
                                                        const int32_t *__restrict__ col,
                                                        const double *__restrict__ val,
                                                        const double *__restrict__ x, double alpha, double beta,
                                                        double *__restrict__ y) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int sub = threadIdx.x % TPR;
    constexpr int RPW = 32 / TPR;
    const int64_t steps = (ne + RPW - 1) / RPW;
    int64_t st0, st_end, st_inc;
    if constexpr (BLOCK_RANGE) {
        const int64_t per = (steps + gridDim.x - 1) / gridDim.x;
        st0 = blockIdx.x * per + (threadIdx.x >> 5);
        st_end = min(steps, (int64_t)(blockIdx.x + 1) * per);
        st_inc = blockDim.x >> 5;
    } else {
        const int64_t warp = tid >> 5, nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
        const int64_t per = (steps + nwarps - 1) / nwarps;
        st0 = warp * per;
        st_end = min(steps, (warp + 1) * per);
        st_inc = 1;
    }
    for (int64_t st = st0; st < st_end; st += S * st_inc) {
        int64_t r[S], a[S], b[S];
        double acc[S];
#pragma unroll
        for (int t = 0; t < S; t++) {
            const int64_t stt = st + t * st_inc;
            r[t] = stt < st_end ? stt * RPW + (threadIdx.x & 31) / TPR : ne;
            const bool live = r[t] < ne;
            a[t] = live ? __ldg(&rp[r[t]]) : 0;
            b[t] = live ? __ldg(&rp[r[t] + 1]) : 0;
            acc[t] = 0.0;
            if ((a[t] & 1) && a[t] < b[t]) {  // odd start: one scalar entry so the pairs are aligned
                if (sub == 0) acc[t] = __ldg(&val[a[t]]) * __ldg(&x[__ldg(&col[a[t]])]);
                a[t]++;
            }
        }
        for (int64_t off = 2 * sub;; off += (int64_t)2 * TPR * U) {
            bool any = false;
#pragma unroll
            for (int t = 0; t < S; t++) any |= a[t] + off < b[t];
            if (!any) break;
            int2 c[S][U];
            double2 v[S][U];
#pragma unroll
            for (int t = 0; t < S; t++)
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int64_t q = a[t] + off + (int64_t)2 * TPR * u;
                    if (q + 1 < b[t]) {
                        c[t][u] = __ldg(reinterpret_cast<const int2 *>(col + q));
                        v[t][u] = __ldg(reinterpret_cast<const double2 *>(val + q));
                    } else if (q < b[t]) {
                        c[t][u] = make_int2(__ldg(&col[q]), -1);
                        v[t][u] = make_double2(__ldg(&val[q]), 0.0);
                    } else {
                        c[t][u] = make_int2(-1, -1);
                        v[t][u] = make_double2(0.0, 0.0);
                    }
                }
            double xa[S][U], xb[S][U];
#pragma unroll
            for (int t = 0; t < S; t++)
#pragma unroll
                for (int u = 0; u < U; u++) {
                    xa[t][u] = c[t][u].x >= 0 ? __ldg(&x[c[t][u].x]) : 0.0;
                    xb[t][u] = c[t][u].y >= 0 ? __ldg(&x[c[t][u].y]) : 0.0;
                }
#pragma unroll
            for (int t = 0; t < S; t++)
#pragma unroll
                for (int u = 0; u < U; u++) acc[t] = fma(v[t][u].y, xb[t][u], fma(v[t][u].x, xa[t][u], acc[t]));
        }
#pragma unroll
        for (int t = 0; t < S; t++) {
            double sm = acc[t];
#pragma unroll
            for (int o = TPR / 2; o > 0; o >>= 1) sm += __shfl_down_sync(0xffffffffu, sm, o, TPR);
            if (sub == 0 && r[t] < ne) y[r[t]] = (beta == 0.0) ? alpha * sm : fma(alpha, sm, beta * y[r[t]]);
        }
    }
}

// lanes = fields (nf <= 32), 32/nfp rows per warp, nfp = nf rounded up to a power of two
__global__ void __launch_bounds__(256) spmm_interleaved_kernel(int64_t ne, const int64_t *__restrict__ rp,
                                                               const int32_t *__restrict__ col,
                                                               const double *__restrict__ val, int nf, int nfp,
                                                               const double *__restrict__ X, int64_t ldx,
                                                               double alpha, double beta, double *__restrict__ Y,
                                                               int64_t ldy) {
    const int lane = threadIdx.x & 31;
    const int f = lane % nfp;
    const int rows_per_warp = 32 / nfp;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r0 = warp * rows_per_warp; r0 < ne; r0 += nwarps * rows_per_warp) {
        const int64_t r = r0 + lane / nfp;
        if (r >= ne || f >= nf) continue;
        const int64_t a = rp[r], b = rp[r + 1];
        // eight entries at a time: their indices and values first, then eight gathers in flight
        double s0 = 0.0, s1 = 0.0;
        int64_t p = a;
        for (; p + 7 < b; p += 8) {
            int c[8];
            double v[8], xg[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                c[u] = __ldg(&col[p + u]);
                v[u] = __ldg(&val[p + u]);
            }
#pragma unroll
            for (int u = 0; u < 8; u++) xg[u] = __ldg(&X[(int64_t)c[u] * ldx + f]);
#pragma unroll
            for (int u = 0; u < 8; u += 2) {
                s0 = fma(v[u], xg[u], s0);
                s1 = fma(v[u + 1], xg[u + 1], s1);
            }
        }
        for (; p < b; p++) s0 = fma(__ldg(&val[p]), __ldg(&X[(int64_t)__ldg(&col[p]) * ldx + f]), s0);
        const double s = s0 + s1;
        double *yp = &Y[r * ldy + f];
        *yp = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * *yp);
    }
}

// out[i*nf + f] = in[f*ld + i] (tiled through shared memory)
__global__ void to_interleaved_kernel(int64_t n, int nf, const double *__restrict__ in, int64_t ld,
                                      double *__restrict__ out) {
    __shared__ double tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32;
    const int f0 = blockIdx.y * 32;
    for (int fy = threadIdx.y; fy < 32; fy += blockDim.y) {
        int f = f0 + fy;
        int64_t i = i0 + threadIdx.x;
        tile[fy][threadIdx.x] = (f < nf && i < n) ? in[(int64_t)f * ld + i] : 0.0;
    }
    __syncthreads();
    for (int iy = threadIdx.y; iy < 32; iy += blockDim.y) {
        int64_t i = i0 + iy;
        int f = f0 + threadIdx.x;
        if (i < n && f < nf) out[i * nf + f] = tile[threadIdx.x][iy];
    }
}

// out[f*ld + i] = in[i*nf + f]
__global__ void from_interleaved_kernel(int64_t n, int nf, const double *__restrict__ in,
                                        double *__restrict__ out, int64_t ld) {
    __shared__ double tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32;
    const int f0 = blockIdx.y * 32;
    for (int iy = threadIdx.y; iy < 32; iy += blockDim.y) {
        int64_t i = i0 + iy;
        int f = f0 + threadIdx.x;
        tile[iy][threadIdx.x] = (i < n && f < nf) ? in[i * nf + f] : 0.0;
    }
    __syncthreads();
    for (int fy = threadIdx.y; fy < 32; fy += blockDim.y) {
        int f = f0 + fy;
        int64_t i = i0 + threadIdx.x;
        if (f < nf && i < n) out[(int64_t)f * ld + i] = tile[threadIdx.x][fy];
    }
}

__global__ void csc_count_kernel(int64_t nnz, const int32_t *__restrict__ col, int64_t *__restrict__ cnt) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x)
        atomicAdd((unsigned long long *)&cnt[col[p]], 1ull);
}

__global__ void csc_scatter_kernel(int64_t ne, const int64_t *__restrict__ rp, const int32_t *__restrict__ col,
                                   const double *__restrict__ val, const int64_t *__restrict__ cp,
                                   unsigned long long *__restrict__ fill, int32_t *__restrict__ row_out,
                                   double *__restrict__ val_out) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ne; r += (int64_t)gridDim.x * blockDim.x)
        for (int64_t p = rp[r]; p < rp[r + 1]; p++) {
            int32_t c = col[p];
            int64_t q = cp[c] + (int64_t)atomicAdd(&fill[c], 1ull);
            row_out[q] = (int32_t)r;
            val_out[q] = val[p];
        }
}

// rows within each column ascending (insertion sort; columns hold about k entries)
__global__ void csc_sort_kernel(int64_t ns, const int64_t *__restrict__ cp, int32_t *__restrict__ row,
                                double *__restrict__ v) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ns; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = cp[c], b = cp[c + 1];
        for (int64_t i = a + 1; i < b; i++) {
            int32_t rr = row[i];
            double vv = v[i];
            int64_t j = i - 1;
            while (j >= a && row[j] > rr) {
                row[j + 1] = row[j];
                v[j + 1] = v[j];
                j--;
            }
            row[j + 1] = rr;
            v[j + 1] = vv;
        }
    }
}

int blocks_for(rbf_ctx *ctx, int64_t work, int threads, int per_sm) {
    int64_t b = (work + threads - 1) / threads;
    b = std::min<int64_t>(b, (int64_t)ctx->num_sms * per_sm);
    return (int)std::max<int64_t>(b, 1);
}

}  // namespace

// One field: the paired-load kernel (4 lanes per row, 4 pairs per lane, block row ranges:
// the fastest of the shapes measured on GB300) when the arrays allow 8/16-byte loads.
static int spmv_launch(rbf_ctx *ctx, int64_t ne, const int64_t *d_rp, const int32_t *d_col, const double *d_val,
                const double *d_X, double alpha, double beta, double *d_Y) {
    if ((((uintptr_t)d_col) & 7) == 0 && (((uintptr_t)d_val) & 15) == 0)
        spmv_pair_kernel<4, 4, 1, true><<<blocks_for(ctx, ne * 4, 256, 8), 256, 0, ctx->stream>>>(
            ne, d_rp, d_col, d_val, d_X, alpha, beta, d_Y);
    else
        spmv_kernel<8, 4><<<blocks_for(ctx, ne * 8, 256, 16), 256, 0, ctx->stream>>>(ne, d_rp, d_col, d_val, d_X,
                                                                                    alpha, beta, d_Y);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

int rbf_spmm_device(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *d_rp, const int32_t *d_col,
                    const double *d_val, int nf, int layout, const double *d_X, int64_t ldx, double alpha,
                    double beta, double *d_Y, int64_t ldy) {
    if (ne == 0 || nf == 0) return RBF_OK;
    if (nf == 1) return spmv_launch(ctx, ne, d_rp, d_col, d_val, d_X, alpha, beta, d_Y);
    const double *Xi = d_X;
    double *Yi = d_Y;
    int64_t lx = ldx, ly = ldy;
    DevBuf xs, ys;
    if (layout == 0) {  // column-major: stage through interleaved scratch
        RBF_TRY(xs.alloc(ctx, sizeof(double) * ns * nf));
        RBF_TRY(ys.alloc(ctx, sizeof(double) * ne * nf));
        dim3 tb(32, 8);
        if (ns > 0) {  // with no data points every row is empty and X is never read
            to_interleaved_kernel<<<dim3((unsigned)((ns + 31) / 32), (unsigned)((nf + 31) / 32)), tb, 0,
                                    ctx->stream>>>(ns, nf, d_X, ldx, xs.as<double>());
            RBF_CHECK_LAUNCH(ctx);
        }
        if (beta != 0.0) {
            to_interleaved_kernel<<<dim3((unsigned)((ne + 31) / 32), (unsigned)((nf + 31) / 32)), tb, 0, ctx->stream>>>(
                ne, nf, d_Y, ldy, ys.as<double>());
            RBF_CHECK_LAUNCH(ctx);
        }
        Xi = xs.as<double>();
        Yi = ys.as<double>();
        lx = nf;
        ly = nf;
    }
    for (int f0 = 0; f0 < nf; f0 += 32) {
        int nfc = std::min(32, nf - f0);
        int nfp = 1;
        while (nfp < nfc) nfp <<= 1;
        int64_t warps = (ne + (32 / nfp) - 1) / (32 / nfp);
        spmm_interleaved_kernel<<<blocks_for(ctx, warps * 32, 256, 16), 256, 0, ctx->stream>>>(
            ne, d_rp, d_col, d_val, nfc, nfp, Xi + f0, lx, alpha, beta, Yi + f0, ly);
        RBF_CHECK_LAUNCH(ctx);
    }
    if (layout == 0) {
        dim3 tb(32, 8);
        from_interleaved_kernel<<<dim3((unsigned)((ne + 31) / 32), (unsigned)((nf + 31) / 32)), tb, 0, ctx->stream>>>(
            ne, nf, Yi, d_Y, ldy);
        RBF_CHECK_LAUNCH(ctx);
    }
    return RBF_OK;
}

int rbf_csr_to_csc_device(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *d_rp, const int32_t *d_col,
                          const double *d_val, int64_t *d_cp, int32_t *d_row, double *d_valc) {
    int64_t nnz = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&nnz, d_rp + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    DevBuf cnt, fill;
    RBF_TRY(cnt.alloc(ctx, sizeof(int64_t) * (ns + 1)));
    RBF_TRY(fill.alloc(ctx, sizeof(int64_t) * (ns + 1)));
    RBF_CUDA(ctx, cudaMemsetAsync(cnt.ptr, 0, sizeof(int64_t) * (ns + 1), ctx->stream));
    RBF_CUDA(ctx, cudaMemsetAsync(fill.ptr, 0, sizeof(int64_t) * (ns + 1), ctx->stream));
    csc_count_kernel<<<blocks_for(ctx, nnz, 256, 8), 256, 0, ctx->stream>>>(nnz, d_col, cnt.as<int64_t>());
    RBF_CHECK_LAUNCH(ctx);
    RBF_TRY(rbf_exclusive_scan_i64(ctx, cnt.as<int64_t>(), d_cp, ns + 1, nullptr));
    csc_scatter_kernel<<<blocks_for(ctx, ne, 256, 8), 256, 0, ctx->stream>>>(
        ne, d_rp, d_col, d_val, d_cp, fill.as<unsigned long long>(), d_row, d_valc);
    RBF_CHECK_LAUNCH(ctx);
    csc_sort_kernel<<<blocks_for(ctx, ns, 256, 8), 256, 0, ctx->stream>>>(ns, d_cp, d_row, d_valc);
    RBF_CHECK_LAUNCH(ctx);
    return RBF_OK;
}

// ---------------------------------------------------------------------------------------
// Allocation-free apply (rbf_spmm_noalloc)
//
// Some callers cannot allocate device memory while they apply an operator: code running
// inside another framework's memory pool that forbids foreign allocations, a time-stepping
// loop that must not touch the allocator between steps, or a host thread that may not
// synchronise with the device allocator.  For them the column-major multi-field apply,
// the one path of rbf_spmm that needs scratch (the interleaved copies of X and Y), stages
// through this fixed file-scope device array instead of stream-ordered allocations.
// Capacity: RBF_NOALLOC_SCRATCH_DOUBLES doubles (32 MiB) per GPU that loads the library,
// held until the process exits; a call needing nf*(ns+ne) doubles more than that is
// rejected.  Every call shares the array: calls that overlap on the GPU (different
// streams, or contexts on the same device) race on it.  Both halves are written in full
// before they are read, so nothing needs clearing between calls.
// ---------------------------------------------------------------------------------------
#define RBF_NOALLOC_SCRATCH_DOUBLES (4u << 20)
static __device__ __align__(256) double g_noalloc_scratch[RBF_NOALLOC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double *g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device with
// that device current.  The cached address belongs to the device's primary context: after a
// cudaDeviceReset every context of this library is invalid as well and the library must not
// be called again in that process.
int noalloc_scratch(rbf_ctx *ctx, double **out) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "device %d out of range for the no-alloc apply", ctx->device);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[ctx->device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return rbf_fail(ctx, RBF_ERR_CUDA, "cudaGetSymbolAddress(no-alloc scratch) failed: %s",
                            cudaGetErrorString(e));
        g_noalloc_ptr[ctx->device] = static_cast<double *>(p);
    }
    *out = g_noalloc_ptr[ctx->device];
    return RBF_OK;
}
}  // namespace

namespace {
// The device work of the allocation-free apply (arguments already checked).
int noalloc_apply(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *row_ptr, const int32_t *col,
                  const double *val, int32_t nf, int32_t layout, const double *X, int64_t ldx, double alpha,
                  double beta, double *Y, int64_t ldy) {
    const bool staged = (layout == 0 && nf > 1);
    if (!staged) {
        if (nf == 1) {
            RBF_TRY(spmv_launch(ctx, ne, row_ptr, col, val, X, alpha, beta, Y));
        } else {
            for (int f0 = 0; f0 < nf; f0 += 32) {
                int nfc = std::min(32, nf - f0), nfp = 1;
                while (nfp < nfc) nfp <<= 1;
                int64_t warps = (ne + (32 / nfp) - 1) / (32 / nfp);
                spmm_interleaved_kernel<<<blocks_for(ctx, warps * 32, 256, 16), 256, 0, ctx->stream>>>(
                    ne, row_ptr, col, val, nfc, nfp, X + f0, ldx, alpha, beta, Y + f0, ldy);
                RBF_CHECK_LAUNCH(ctx);
            }
        }
    } else {
        double *scratch = nullptr;
        RBF_TRY(noalloc_scratch(ctx, &scratch));
        double *xs = scratch, *ys = scratch + (size_t)nf * ns;
        dim3 tb(32, 8);
        if (ns > 0) {  // with no data points every row is empty and X is never read
            to_interleaved_kernel<<<dim3((unsigned)((ns + 31) / 32), (unsigned)((nf + 31) / 32)), tb, 0,
                                    ctx->stream>>>(ns, nf, X, ldx, xs);
            RBF_CHECK_LAUNCH(ctx);
        }
        if (beta != 0.0) {
            to_interleaved_kernel<<<dim3((unsigned)((ne + 31) / 32), (unsigned)((nf + 31) / 32)), tb, 0, ctx->stream>>>(
                ne, nf, Y, ldy, ys);
            RBF_CHECK_LAUNCH(ctx);
        }
        for (int f0 = 0; f0 < nf; f0 += 32) {
            int nfc = std::min(32, nf - f0), nfp = 1;
            while (nfp < nfc) nfp <<= 1;
            int64_t warps = (ne + (32 / nfp) - 1) / (32 / nfp);
            spmm_interleaved_kernel<<<blocks_for(ctx, warps * 32, 256, 16), 256, 0, ctx->stream>>>(
                ne, row_ptr, col, val, nfc, nfp, xs + f0, nf, alpha, beta, ys + f0, nf);
            RBF_CHECK_LAUNCH(ctx);
        }
        from_interleaved_kernel<<<dim3((unsigned)((ne + 31) / 32), (unsigned)((nf + 31) / 32)), tb, 0, ctx->stream>>>(
            ne, nf, ys, Y, ldy);
        RBF_CHECK_LAUNCH(ctx);
    }
    return RBF_OK;
}
}  // namespace

extern "C" int rbf_spmm_noalloc(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *row_ptr, const int32_t *col,
                                const double *val, int32_t nf, int32_t layout, const double *X, int64_t ldx,
                                double alpha, double beta, double *Y, int64_t ldy) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    RBF_CUDA(ctx, cudaSetDevice(ctx->device));
    if (nf < 1 || ne < 0 || ns < 0) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid sizes");
    if (layout != 0 && layout != 1) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "layout must be 0 or 1");
    if (layout == 0 && nf > 1 && (ldx < ns || ldy < ne)) return rbf_fail(ctx, RBF_ERR_DIMENSION, "leading dimension too small");
    if (layout == 1 && (ldx < nf || ldy < nf)) return rbf_fail(ctx, RBF_ERR_DIMENSION, "leading dimension too small");
    const bool staged = (layout == 0 && nf > 1);
    if (staged && (double)nf * (double)(ns + ne) > (double)RBF_NOALLOC_SCRATCH_DOUBLES)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT,
                        "no-alloc apply: nf*(ns+ne) = %lld doubles exceeds the fixed scratch of %u doubles (32 MiB); "
                        "use rbf_spmm or the interleaved layout",
                        (long long)nf * (long long)(ns + ne), RBF_NOALLOC_SCRATCH_DOUBLES);
    if (!rbf_is_device_ptr(row_ptr) || !rbf_is_device_ptr(col) || !rbf_is_device_ptr(val) || !rbf_is_device_ptr(X) ||
        !rbf_is_device_ptr(Y))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "no-alloc apply: every array must be a device pointer");
    if (ne == 0) return RBF_OK;
    // with timing on, CUDA events bracket the device work (as in rbf_spmm)
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (ctx->timing) {
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, ctx->stream);
    }
    const int st = noalloc_apply(ctx, ne, ns, row_ptr, col, val, nf, layout, X, ldx, alpha, beta, Y, ldy);
    if (ctx->timing) {
        cudaEventRecord(t1, ctx->stream);
        cudaEventSynchronize(t1);
        cudaEventElapsedTime(&ctx->last_ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    RBF_TRY(st);
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}
