// Grid-bucketed exact k-nearest-neighbour search (replaces find_neighbors,
// src/utils.jl:12-18, which builds a KDTree and calls knn(tree, eval, k, true)).
//
// Layout in HBM
//   source points are counting-sorted into a uniform grid: sp[] (AoS doubles, cell order),
//   sidx[] (original index per sorted slot), cstart[ncells+1] (first slot of each cell).
//   Queries are visited in cell order (qorder[]) so that neighbouring warps touch the same
//   cells and the candidate reads hit L1/L2.
// Search (one warp per query)
//   The warp scans the block of cells within Chebyshev radius R0 of the query's cell, then
//   shells R0+1, R0+2, ... until the k-th best squared distance is below the squared
//   distance from the query to the outside of the scanned block.  Candidates are read as
//   one flattened list of contiguous cell runs (each x-row of cells is contiguous in the
//   sorted order), 32 per step, so all lanes stay busy.
// Ordering
//   Keys are (squared distance, point index): the squared distance is accumulated in
//   dimension order without FMA contraction, exactly as the reference's Euclidean
//   reduction does, and exact ties go to the smaller index.  The running top-k list is a
//   sorted array spread over the warp (slot j at lane j%32, register j/32) and candidates
//   that beat the current k-th key are inserted with warp shuffles.  In the first block of
//   cells (up to 256 candidates) the keys are held in registers first and a bisection finds
//   a key bound with at least k + 8 keys below it; only those are offered to the list, which
//   cuts the insertions (74 % of the search time before) from ~2.8 (k + 8) to ~(k + 8);
//   when the offered keys fit the list they become it by one warp bitonic sort instead.
#include <algorithm>
#include <cmath>
#include <vector>

#include "rbf_internal.cuh"

namespace {

constexpr int KNN_WARPS = 8;     // warps per block
constexpr int KNN_RANGES = 64;   // cell runs buffered per warp step

struct GridDesc {
    double lo[3];
    double h[3];
    double inv_h[3];
    float lof[3], hf[3], inv_hf[3];  // FP32 copies (rounded on the host) for the FP32 search
    int nc[3];
    int64_t ncells;
};

// A non-negative double rounded up to a float, on the integer pipe (as __double2float_ru).
__device__ __forceinline__ float d2f_ru_nonneg_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    if (e <= 0 || e >= 255) return __double2float_ru(x);
    unsigned r = ((unsigned)e << 23) | (unsigned)((b & 0xfffffffffffffull) >> 29);
    if (b & 0x1fffffffull) r += 1u;
    return __uint_as_float(r);
}

__device__ __forceinline__ double sqdist(const double *a, const double *b, int dim) {
    double t = __dsub_rn(a[0], b[0]);
    double s = __dmul_rn(t, t);
    for (int d = 1; d < dim; d++) {
        t = __dsub_rn(a[d], b[d]);
        s = __dadd_rn(s, __dmul_rn(t, t));
    }
    return s;
}

template <int DIM>
__device__ __forceinline__ int64_t cell_of(const GridDesc &g, const double *x, int *c) {
    int64_t id = 0;
#pragma unroll
    for (int d = DIM - 1; d >= 0; d--) {
        double f = floor((x[d] - g.lo[d]) * g.inv_h[d]);
        int cd;
        if (!(f >= 0.0)) cd = 0;  // also catches NaN
        else if (f >= (double)(g.nc[d] - 1)) cd = g.nc[d] - 1;
        else cd = (int)f;
        c[d] = cd;
        id = id * g.nc[d] + cd;
    }
    return id;
}

__global__ void bbox_partial_kernel(const double *__restrict__ x, int64_t n, int dim, double *__restrict__ part) {
    __shared__ double smin[3][256], smax[3][256];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < dim; d++) {
            double v = x[i * dim + d];
            mn[d] = fmin(mn[d], v);
            mx[d] = fmax(mx[d], v);
        }
    for (int d = 0; d < 3; d++) {
        smin[d][threadIdx.x] = mn[d];
        smax[d][threadIdx.x] = mx[d];
    }
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int d = 0; d < 3; d++) {
                smin[d][threadIdx.x] = fmin(smin[d][threadIdx.x], smin[d][threadIdx.x + s]);
                smax[d][threadIdx.x] = fmax(smax[d][threadIdx.x], smax[d][threadIdx.x + s]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; d++) {
            part[blockIdx.x * 6 + d] = smin[d][0];
            part[blockIdx.x * 6 + 3 + d] = smax[d][0];
        }
}

template <int DIM>
__global__ void cell_count_kernel(GridDesc g, const double *__restrict__ x, int64_t n,
                                  int32_t *__restrict__ cell, int32_t *__restrict__ count) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double p[DIM];
#pragma unroll
        for (int d = 0; d < DIM; d++) p[d] = x[i * DIM + d];
        int c[DIM];
        int64_t id = cell_of<DIM>(g, p, c);
        cell[i] = (int32_t)id;
        atomicAdd(&count[id], 1);
    }
}

template <int DIM>
__global__ void cell_scatter_kernel(const double *__restrict__ x, int64_t n, const int32_t *__restrict__ cell,
                                    const int32_t *__restrict__ start, int32_t *__restrict__ fill,
                                    double *__restrict__ sp, float4 *__restrict__ sp32, int32_t *__restrict__ sidx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t c = cell[i];
        int32_t pos = start[c] + atomicAdd(&fill[c], 1);
        if (sp) {
            double v[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int d = 0; d < DIM; d++) {
                v[d] = x[i * DIM + d];
                sp[(int64_t)pos * DIM + d] = v[d];
            }
            sp32[pos] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.0f);
        }
        sidx[pos] = (int32_t)i;
    }
}

__device__ __forceinline__ bool key_less(double d1, int32_t i1, double d2, int32_t i2) {
    return d1 < d2 || (d1 == d2 && i1 < i2);
}

template <int DIM, int SLOTS>
__global__ void __launch_bounds__(KNN_WARPS * 32)
knn_query_kernel(GridDesc g, const double *__restrict__ sp, const int32_t *__restrict__ sidx,
                 const int32_t *__restrict__ cstart, const double *__restrict__ q,
                 const int32_t *__restrict__ qorder, int64_t nq, int k, int R0,
                 int32_t *__restrict__ out) {
    __shared__ int32_t s_start[KNN_WARPS][KNN_RANGES];
    __shared__ int32_t s_off[KNN_WARPS][KNN_RANGES + 1];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t warp0 = (int64_t)blockIdx.x * KNN_WARPS + wib;
    const int64_t nwarps = (int64_t)gridDim.x * KNN_WARPS;
    int32_t *my_start = s_start[wib];
    int32_t *my_off = s_off[wib];

    for (int64_t t = warp0; t < nq; t += nwarps) {
        const int32_t qi = qorder[t];
        double qp[DIM];
#pragma unroll
        for (int d = 0; d < DIM; d++) qp[d] = q[(int64_t)qi * DIM + d];
        int qc[3] = {0, 0, 0};
        cell_of<DIM>(g, qp, qc);

        double key[SLOTS];
        int32_t kid[SLOTS];
#pragma unroll
        for (int s = 0; s < SLOTS; s++) {
            key[s] = INFINITY;
            kid[s] = 0x7fffffff;
        }
        double kth = INFINITY;
        int32_t kth_id = 0x7fffffff;
        const int kl = (k - 1) & 31, ks = (k - 1) >> 5;

        int r_in = -1;
        for (int R = R0;; R++) {
            // rows of cells: (dy, dz) in [-R, R]^(DIM-1)
            const int side = 2 * R + 1;
            const int nrows = DIM == 1 ? 1 : (DIM == 2 ? side : side * side);
            for (int row0 = 0; row0 < nrows; row0 += 32) {
                // each lane describes up to two runs of cells of one row
                int row = row0 + lane;
                int32_t a0 = 0, l0 = 0, a1 = 0, l1 = 0;
                if (row < nrows) {
                    int dy = 0, dz = 0;
                    if (DIM >= 2) dy = (row % side) - R;
                    if (DIM == 3) dz = (row / side) - R;
                    int cy = qc[1] + dy, cz = qc[2] + dz;
                    bool inside = (DIM < 2 || (cy >= 0 && cy < g.nc[1])) && (DIM < 3 || (cz >= 0 && cz < g.nc[2]));
                    if (inside) {
                        int m = max(abs(dy), abs(dz));
                        int64_t rowbase = ((int64_t)cz * g.nc[1] + cy) * g.nc[0];
                        if (m > r_in) {
                            int x0 = max(qc[0] - R, 0), x1 = min(qc[0] + R, g.nc[0] - 1);
                            if (x0 <= x1) {
                                a0 = cstart[rowbase + x0];
                                l0 = cstart[rowbase + x1 + 1] - a0;
                            }
                        } else {
                            int x0 = max(qc[0] - R, 0), x1 = min(qc[0] - r_in - 1, g.nc[0] - 1);
                            if (x0 <= x1) {
                                a0 = cstart[rowbase + x0];
                                l0 = cstart[rowbase + x1 + 1] - a0;
                            }
                            x0 = max(qc[0] + r_in + 1, 0);
                            x1 = min(qc[0] + R, g.nc[0] - 1);
                            if (x0 <= x1) {
                                a1 = cstart[rowbase + x0];
                                l1 = cstart[rowbase + x1 + 1] - a1;
                            }
                        }
                    }
                }
                // exclusive offsets of the 64 runs (run 2*lane and 2*lane+1)
                int32_t pair = l0 + l1, incl = pair;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                int32_t excl = incl - pair;
                my_start[2 * lane] = a0;
                my_start[2 * lane + 1] = a1;
                my_off[2 * lane] = excl;
                my_off[2 * lane + 1] = excl + l0;
                const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
                if (lane == 31) my_off[KNN_RANGES] = total;
                __syncwarp();
                for (int32_t f0 = 0; f0 < total; f0 += 32) {
                    int32_t f = f0 + lane;
                    double dd = INFINITY;
                    int32_t id = 0x7fffffff;
                    if (f < total) {
                        // last run whose offset <= f (runs of length 0 are skipped by <=)
                        int lo = 0, hi = KNN_RANGES - 1;
                        while (lo < hi) {
                            int mid = (lo + hi + 1) >> 1;
                            if (my_off[mid] <= f) lo = mid;
                            else hi = mid - 1;
                        }
                        int32_t p = my_start[lo] + (f - my_off[lo]);
                        double xp[DIM];
#pragma unroll
                        for (int d = 0; d < DIM; d++) xp[d] = sp[(int64_t)p * DIM + d];
                        dd = sqdist(qp, xp, DIM);
                        id = sidx[p];
                    }
                    bool pass = (f < total) && key_less(dd, id, kth, kth_id);
                    unsigned m = __ballot_sync(0xffffffffu, pass);
                    while (m) {
                        const int src = __ffs(m) - 1;
                        m &= m - 1;
                        const double cd = __shfl_sync(0xffffffffu, dd, src);
                        const int32_t ci = __shfl_sync(0xffffffffu, id, src);
                        if (!key_less(cd, ci, kth, kth_id)) continue;  // uniform across the warp
                        int pos = 0;
#pragma unroll
                        for (int s = 0; s < SLOTS; s++)
                            pos += __popc(__ballot_sync(0xffffffffu, key_less(key[s], kid[s], cd, ci)));
                        // shift right by one from pos, insert at pos
                        double pk[SLOTS];
                        int32_t pi[SLOTS];
#pragma unroll
                        for (int s = 0; s < SLOTS; s++) {
                            pk[s] = __shfl_up_sync(0xffffffffu, key[s], 1);
                            pi[s] = __shfl_up_sync(0xffffffffu, kid[s], 1);
                            const int sp = s > 0 ? s - 1 : 0;
                            double wk = __shfl_sync(0xffffffffu, key[sp], 31);
                            int32_t wi = __shfl_sync(0xffffffffu, kid[sp], 31);
                            if (lane == 0) {
                                pk[s] = wk;
                                pi[s] = wi;
                            }
                        }
#pragma unroll
                        for (int s = 0; s < SLOTS; s++) {
                            int j = lane + 32 * s;
                            if (j == pos) {
                                key[s] = cd;
                                kid[s] = ci;
                            } else if (j > pos) {
                                key[s] = pk[s];
                                kid[s] = pi[s];
                            }
                        }
                        double kv = key[0];
                        int32_t ki = kid[0];
#pragma unroll
                        for (int s = 1; s < SLOTS; s++)
                            if (s == ks) {
                                kv = key[s];
                                ki = kid[s];
                            }
                        kth = __shfl_sync(0xffffffffu, kv, kl);
                        kth_id = __shfl_sync(0xffffffffu, ki, kl);
                    }
                }
                __syncwarp();
            }
            // distance from the query to the outside of the scanned block
            double cover = INFINITY;
            bool all_covered = true;
#pragma unroll
            for (int d = 0; d < DIM; d++) {
                if (qc[d] - R > 0) {
                    all_covered = false;
                    cover = fmin(cover, qp[d] - (g.lo[d] + (double)(qc[d] - R) * g.h[d]));
                }
                if (qc[d] + R < g.nc[d] - 1) {
                    all_covered = false;
                    cover = fmin(cover, (g.lo[d] + (double)(qc[d] + R + 1) * g.h[d]) - qp[d]);
                }
            }
            if (all_covered) break;
            if (kth < INFINITY) {
                // slack for the rounding of cell assignment vs. face positions
                double mag = 0.0;
#pragma unroll
                for (int d = 0; d < DIM; d++) mag = fmax(mag, fabs(qp[d]) + fabs(g.lo[d]) + g.h[d] * g.nc[d]);
                double c = cover * (1.0 - 1e-9) - 4e-15 * mag;
                if (c > 0.0 && kth < c * c) break;
            }
            r_in = R;
        }
        // write the sorted row
#pragma unroll
        for (int s = 0; s < SLOTS; s++) {
            int j = lane + 32 * s;
            if (j < k) out[(int64_t)qi * k + j] = kid[s];
        }
    }
}


__device__ __forceinline__ bool fkey_less(float d1, int32_t i1, float d2, int32_t i2) {
    return d1 < d2 || (d1 == d2 && i1 < i2);
}

__device__ __forceinline__ bool xkey_less(unsigned long long d1, int32_t i1, unsigned long long d2, int32_t i2) {
    return d1 < d2 || (d1 == d2 && i1 < i2);
}

// Bitonic sort of the 32 * SLOTS (FP32 key, index) pairs of a warp, ascending (element
// j = lane + 32 s): strides below 32 by shuffles, stride 32 between a lane's registers.  A
// pair is packed as (key bits << 32) | index: the keys are squared distances (+0 or positive,
// never NaN), whose bit patterns order as unsigned integers, so the packed order is the
// (key, index) order of fkey_less and every compare-exchange is one 64-bit shuffle, one
// unsigned comparison and one select.
template <int SLOTS>
__device__ __forceinline__ void warp_sort_packed(unsigned long long (&v)[SLOTS], int lane) {
#pragma unroll
    for (int size = 2; size <= 32 * SLOTS; size <<= 1) {
#pragma unroll
        for (int stride = size / 2; stride > 0; stride >>= 1) {
            if (stride >= 32) {
                if constexpr (SLOTS > 1) {
                    const bool sw = v[SLOTS - 1] < v[0];
                    const unsigned long long lo = sw ? v[SLOTS - 1] : v[0], hi = sw ? v[0] : v[SLOTS - 1];
                    v[0] = lo;
                    v[SLOTS - 1] = hi;
                }
            } else {
#pragma unroll
                for (int s = 0; s < SLOTS; s++) {
                    const int e = lane + 32 * s;
                    const unsigned long long o = __shfl_xor_sync(0xffffffffu, v[s], stride);
                    const bool keep_min = ((e & size) == 0) == ((e & stride) == 0);
                    v[s] = (keep_min == (o < v[s])) ? o : v[s];
                }
            }
        }
    }
}

// FP32-key search.  Candidate keys are squared distances from the FP32 copy of the points;
// the warp keeps the kp = k + 8 best (FP32 key, index) pairs.  The search stops once the
// kp-th FP32 distance plus its error bound is inside the covered ball, so the kp listed
// points are the kp nearest up to rounding.  Then the exact FP64 squared distances (dimension
// order, no FMA) of the kp candidates are sorted with the index tie-break, and the result is
// accepted only if the exact k-th distance is below the smallest exact distance any unlisted
// point can have (the kp-th FP32 distance minus its error bound); otherwise the query is
// appended to the fallback list for the exact FP64 search.
// Error bound of an FP32 distance (u = 2^-24, M the largest coordinate magnitude):
// |d32 - d| <= 8u (M + d).
// SLOTS: registers per lane of the sorted candidate list (32 SLOTS entries, room for the first
// block's offered keys, kp .. 1.25 kp); XSLOTS: registers per lane of the exact re-rank of the
// kp listed candidates (kp <= 32 XSLOTS).
template <int DIM, int SLOTS, int XSLOTS>
__global__ void __launch_bounds__(KNN_WARPS * 32, 4)  // 32 warps/SM: 64 registers
knn_fast_kernel(GridDesc g, const float4 *__restrict__ sp32, const int32_t *__restrict__ sidx,
                const int32_t *__restrict__ cstart, const double *__restrict__ data, const double *__restrict__ q,
                const int32_t *__restrict__ qorder, int64_t nq, int k, int kp, int R0, float mag, int64_t ns,
                int32_t *__restrict__ out, int32_t *__restrict__ fb_list, int32_t *__restrict__ fb_count) {
    __shared__ int32_t s_start[KNN_WARPS][KNN_RANGES];
    __shared__ int32_t s_off[KNN_WARPS][KNN_RANGES + 1];
    __shared__ int32_t s_cid[KNN_WARPS][256];
    __shared__ unsigned long long s_lv[KNN_WARPS][32 * SLOTS];  // offered (key, index), packed
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t warp0 = (int64_t)blockIdx.x * KNN_WARPS + wib;
    const int64_t nwarps = (int64_t)gridDim.x * KNN_WARPS;
    int32_t *my_start = s_start[wib];
    int32_t *my_off = s_off[wib];
    int32_t *my_cid = s_cid[wib];
    const float u8 = 8.0f * 5.9604645e-08f;
    const int tl = (kp - 1) & 31, ts = (kp - 1) >> 5;

    for (int64_t t = warp0; t < nq; t += nwarps) {
        const int32_t qi = qorder[t];
        double qp[DIM];
        float qf[3] = {0.f, 0.f, 0.f};
        float qmag = mag;
#pragma unroll
        for (int d = 0; d < DIM; d++) {
            qp[d] = q[(int64_t)qi * DIM + d];
            qf[d] = d2f_rn_bits(qp[d]);
            qmag = fmaxf(qmag, fabsf(qf[d]));
        }
        const float errc = u8 * qmag * 1.0001f;
        // the search starts in the query's cell, found in FP32: it only centres the search
        // (the covered ball below is measured from the FP32 face positions with slack), so a
        // neighbouring cell at a face changes nothing in the result
        int qc[3] = {0, 0, 0};
        float lof[3], hf[3];
        float gmag = qmag;
#pragma unroll
        for (int d = 0; d < DIM; d++) {
            lof[d] = g.lof[d];
            hf[d] = g.hf[d];
            gmag = fmaxf(gmag, fabsf(lof[d]) + hf[d] * (float)g.nc[d]);
            const float f = floorf((qf[d] - lof[d]) * g.inv_hf[d]);
            qc[d] = !(f >= 0.0f) ? 0 : (f >= (float)(g.nc[d] - 1) ? g.nc[d] - 1 : (int)f);
        }
        const float slackf = 16.0f * 5.9604645e-08f * gmag + 1e-30f;

        float key[SLOTS];
        int32_t kid[SLOTS];
#pragma unroll
        for (int s = 0; s < SLOTS; s++) {
            key[s] = INFINITY;
            kid[s] = 0x7fffffff;
        }
        float kth = INFINITY;
        int32_t kth_id = 0x7fffffff;

        int r_in = -1;
        for (int R = R0;; R++) {
            const int side = 2 * R + 1;
            const int nrows = DIM == 1 ? 1 : (DIM == 2 ? side : side * side);
            for (int row0 = 0; row0 < nrows; row0 += 32) {
                int row = row0 + lane;
                int32_t a0 = 0, l0 = 0, a1 = 0, l1 = 0;
                if (row < nrows) {
                    int dy = 0, dz = 0;
                    if (DIM == 2) dy = row - R;  // row < nrows = side
                    if (DIM == 3) {
                        // row / side without an integer division: (row + 1/2) / side is at least
                        // 1/(2 side) from an integer, the FP32 quotient (2 ulp) within 2e-4 of it
                        // for side <= 512
                        const int zq = side <= 512 ? (int)__fdividef((float)row + 0.5f, (float)side) : row / side;
                        dy = row - zq * side - R;
                        dz = zq - R;
                    }
                    int cy = qc[1] + dy, cz = qc[2] + dz;
                    bool inside = (DIM < 2 || (cy >= 0 && cy < g.nc[1])) && (DIM < 3 || (cz >= 0 && cz < g.nc[2]));
                    if (inside) {
                        int m = max(abs(dy), abs(dz));
                        int64_t rowbase = ((int64_t)cz * g.nc[1] + cy) * g.nc[0];
                        if (m > r_in) {
                            int x0 = max(qc[0] - R, 0), x1 = min(qc[0] + R, g.nc[0] - 1);
                            if (x0 <= x1) {
                                a0 = cstart[rowbase + x0];
                                l0 = cstart[rowbase + x1 + 1] - a0;
                            }
                        } else {
                            int x0 = max(qc[0] - R, 0), x1 = min(qc[0] - r_in - 1, g.nc[0] - 1);
                            if (x0 <= x1) {
                                a0 = cstart[rowbase + x0];
                                l0 = cstart[rowbase + x1 + 1] - a0;
                            }
                            x0 = max(qc[0] + r_in + 1, 0);
                            x1 = min(qc[0] + R, g.nc[0] - 1);
                            if (x0 <= x1) {
                                a1 = cstart[rowbase + x0];
                                l1 = cstart[rowbase + x1 + 1] - a1;
                            }
                        }
                    }
                }
                int32_t pair = l0 + l1, incl = pair;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                int32_t excl = incl - pair;
                my_start[2 * lane] = a0;
                my_start[2 * lane + 1] = a1;
                my_off[2 * lane] = excl;
                my_off[2 * lane + 1] = excl + l0;
                const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
                __syncwarp();
                // FP32 key and point index of flattened candidate f < total
                // FP32 key of the candidate in point slot p
                auto key_at = [&](int32_t p, float &dd) {
                    float4 c4 = __ldg(&sp32[p]);
                    float dx = c4.x - qf[0];
                    dd = dx * dx;
                    if (DIM > 1) {
                        float dy = c4.y - qf[1];
                        dd = fmaf(dy, dy, dd);
                    }
                    if (DIM > 2) {
                        float dz = c4.z - qf[2];
                        dd = fmaf(dz, dz, dd);
                    }
                };
                // ... and its point index
                auto cand_at = [&](int32_t p, float &dd, int32_t &id) {
                    key_at(p, dd);
                    id = __ldg(&sidx[p]);
                };
                // ... of flattened candidate f < total: its cell run by bisection over the offsets
                auto cand = [&](int32_t f, float &dd, int32_t &id) {
                    int lo = 0, hi = KNN_RANGES - 1;
                    while (lo < hi) {
                        int mid = (lo + hi + 1) >> 1;
                        if (my_off[mid] <= f) lo = mid;
                        else hi = mid - 1;
                    }
                    cand_at(my_start[lo] + (f - my_off[lo]), dd, id);
                };
                // the passing candidates of the warp, one at a time, into the sorted list
                auto insert_passing = [&](float dd, int32_t id, bool pass) {
                    unsigned m = __ballot_sync(0xffffffffu, pass);
                    while (m) {
                        const int src = __ffs(m) - 1;
                        m &= m - 1;
                        const float cd = __shfl_sync(0xffffffffu, dd, src);
                        const int32_t ci = __shfl_sync(0xffffffffu, id, src);
                        if (!fkey_less(cd, ci, kth, kth_id)) continue;  // warp-uniform
                        int pos = 0;
#pragma unroll
                        for (int s = 0; s < SLOTS; s++)
                            pos += __popc(__ballot_sync(0xffffffffu, fkey_less(key[s], kid[s], cd, ci)));
                        float pk[SLOTS];
                        int32_t pi[SLOTS];
#pragma unroll
                        for (int s = 0; s < SLOTS; s++) {
                            pk[s] = __shfl_up_sync(0xffffffffu, key[s], 1);
                            pi[s] = __shfl_up_sync(0xffffffffu, kid[s], 1);
                            const int sp = s > 0 ? s - 1 : 0;
                            float wk = __shfl_sync(0xffffffffu, key[sp], 31);
                            int32_t wi = __shfl_sync(0xffffffffu, kid[sp], 31);
                            if (lane == 0) {
                                pk[s] = wk;
                                pi[s] = wi;
                            }
                        }
#pragma unroll
                        for (int s = 0; s < SLOTS; s++) {
                            int j = lane + 32 * s;
                            if (j == pos) {
                                key[s] = cd;
                                kid[s] = ci;
                            } else if (j > pos) {
                                key[s] = pk[s];
                                kid[s] = pi[s];
                            }
                        }
                        float kv = key[0];
                        int32_t ki = kid[0];
#pragma unroll
                        for (int s = 1; s < SLOTS; s++)
                            if (s == ts) {
                                kv = key[s];
                                ki = kid[s];
                            }
                        kth = __shfl_sync(0xffffffffu, kv, tl);
                        kth_id = __shfl_sync(0xffffffffu, ki, tl);
                    }
                };
                if (r_in < 0 && nrows <= 32 && total <= 256 && total > kp) {
                    // first block: keys in registers, indices in shared memory, and a key
                    // threshold t with at least kp keys <= t (found by bisection, aiming at
                    // kp .. 1.25 kp): only keys <= t can be among the kp best, so only they
                    // are offered to the list (about kp insertions instead of ~2.8 kp)
                    // every lane owns one row's run here (nrows <= 32, r_in < 0: no second run):
                    // it writes the point slots of its candidates, so that each candidate is
                    // one shared load away instead of a bisection over the run offsets; only
                    // the offered candidates' point indices are read
                    for (int32_t t = 0; t < l0; t++) my_cid[excl + t] = a0 + t;
                    __syncwarp();
                    float bk[8];
                    float kmax = 0.0f;
#pragma unroll
                    for (int r = 0; r < 8; r++) {
                        const int32_t f = r * 32 + lane;
                        bk[r] = INFINITY;
                        if (f < total) {
                            key_at(my_cid[f], bk[r]);
                            kmax = fmaxf(kmax, bk[r]);
                        }
                    }
                    kmax = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(kmax)));  // keys >= 0
                    __syncwarp();
                    float lo_t = 0.0f, hi_t = kmax;  // all total >= kp keys are <= kmax
                    float t = kmax * exp2f(0.6667f * log2f(1.15f * (float)kp / (float)total));
                    for (int it = 0; it < 8; it++) {
                        int c = 0;
#pragma unroll
                        for (int r = 0; r < 8; r++) c += bk[r] <= t;
                        c = __reduce_add_sync(0xffffffffu, c);
                        if (c >= kp) {
                            hi_t = t;
                            if (c <= kp + (kp >> 2)) break;
                        } else {
                            lo_t = t;
                        }
                        t = 0.5f * (lo_t + hi_t);
                    }
                    // the offered keys, compacted; when they fit the list (the usual case) they
                    // become the list by one bitonic sort, else they are inserted one by one
                    int32_t nof = 0;
#pragma unroll
                    for (int r = 0; r < 8; r++) {
                        const int32_t f = r * 32 + lane;
                        const bool offer = f < total && bk[r] <= hi_t;
                        const unsigned m = __ballot_sync(0xffffffffu, offer);
                        const int32_t pos = nof + __popc(m & ((1u << lane) - 1u));
                        if (offer && pos < 32 * SLOTS)
                            s_lv[wib][pos] = ((unsigned long long)__float_as_uint(bk[r]) << 32) |
                                             (unsigned)__ldg(&sidx[my_cid[f]]);
                        nof += __popc(m);
                    }
                    __syncwarp();
                    if (nof <= 32 * SLOTS) {
                        unsigned long long pv[SLOTS];
#pragma unroll
                        for (int s = 0; s < SLOTS; s++) {
                            const int j = lane + 32 * s;
                            pv[s] = j < nof ? s_lv[wib][j] : 0x7f8000007fffffffull;  // (+inf, 0x7fffffff)
                        }
                        warp_sort_packed<SLOTS>(pv, lane);
#pragma unroll
                        for (int s = 0; s < SLOTS; s++) {
                            key[s] = __uint_as_float((unsigned)(pv[s] >> 32));
                            kid[s] = (int32_t)(unsigned)pv[s];
                        }
                        float kv = key[0];
                        int32_t ki = kid[0];
#pragma unroll
                        for (int s = 1; s < SLOTS; s++)
                            if (s == ts) {
                                kv = key[s];
                                ki = kid[s];
                            }
                        kth = __shfl_sync(0xffffffffu, kv, tl);
                        kth_id = __shfl_sync(0xffffffffu, ki, tl);
                    } else {
#pragma unroll
                        for (int r = 0; r < 8; r++) {
                            const int32_t f = r * 32 + lane;
                            const bool offer = f < total && bk[r] <= hi_t;
                            const int32_t id = offer ? __ldg(&sidx[my_cid[f]]) : 0x7fffffff;
                            insert_passing(bk[r], id, offer && fkey_less(bk[r], id, kth, kth_id));
                        }
                    }
                    __syncwarp();
                    continue;
                }
                for (int32_t f0 = 0; f0 < total; f0 += 32) {
                    int32_t f = f0 + lane;
                    float dd = INFINITY;
                    int32_t id = 0x7fffffff;
                    if (f < total) cand(f, dd, id);
                    insert_passing(dd, id, (f < total) && fkey_less(dd, id, kth, kth_id));
                }
                __syncwarp();
            }
            // distance to the outside of the scanned block, in FP32: every face position and
            // the query carry a rounding error below u*mag, covered by the slack below
            float cover = INFINITY;
            bool all_covered = true;
#pragma unroll
            for (int d = 0; d < DIM; d++) {
                if (qc[d] - R > 0) {
                    all_covered = false;
                    cover = fminf(cover, qf[d] - fmaf((float)(qc[d] - R), hf[d], lof[d]));
                }
                if (qc[d] + R < g.nc[d] - 1) {
                    all_covered = false;
                    cover = fminf(cover, fmaf((float)(qc[d] + R + 1), hf[d], lof[d]) - qf[d]);
                }
            }
            if (all_covered) break;
            if (kth < INFINITY) {
                const float dk = sqrtf(kth);
                const float reach = dk + errc + u8 * dk;
                if (reach < cover * (1.0f - 1e-5f) - slackf) break;
            }
            r_in = R;
        }

        // exact keys of the kp candidates, then a transposition sort (they are nearly sorted)
        unsigned long long xk[XSLOTS];
        int32_t xi[XSLOTS];
#pragma unroll
        for (int s = 0; s < XSLOTS; s++) {
            const int j = lane + 32 * s;
            xk[s] = ~0ull;
            xi[s] = 0x7fffffff;
            if (j < kp && kid[s] != 0x7fffffff) {
                const double *pp = data + (int64_t)kid[s] * DIM;
                double tt = __dsub_rn(qp[0], pp[0]);
                double d2 = __dmul_rn(tt, tt);
#pragma unroll
                for (int d = 1; d < DIM; d++) {
                    tt = __dsub_rn(qp[d], pp[d]);
                    d2 = __dadd_rn(d2, __dmul_rn(tt, tt));
                }
                xk[s] = (unsigned long long)__double_as_longlong(d2);
                xi[s] = kid[s];
            }
        }
        for (int iter = 0; iter < 32 * XSLOTS; iter++) {
            bool swapped = false;
#pragma unroll
            for (int phase = 0; phase < 2; phase++) {
                // neighbours of every position, read before any position of this phase changes
                unsigned long long up_k[XSLOTS], dn_k[XSLOTS];
                int32_t up_i[XSLOTS], dn_i[XSLOTS];
#pragma unroll
                for (int s = 0; s < XSLOTS; s++) {
                    up_k[s] = __shfl_down_sync(0xffffffffu, xk[s], 1);
                    up_i[s] = __shfl_down_sync(0xffffffffu, xi[s], 1);
                    dn_k[s] = __shfl_up_sync(0xffffffffu, xk[s], 1);
                    dn_i[s] = __shfl_up_sync(0xffffffffu, xi[s], 1);
                    if constexpr (XSLOTS > 1) {  // neighbours across the slots' boundary
                        const int sn = s + 1 < XSLOTS ? s + 1 : s;
                        const int spv = s > 0 ? s - 1 : 0;
                        unsigned long long nx_k = __shfl_sync(0xffffffffu, xk[sn], 0);
                        int32_t nx_i = __shfl_sync(0xffffffffu, xi[sn], 0);
                        unsigned long long pv_k = __shfl_sync(0xffffffffu, xk[spv], 31);
                        int32_t pv_i = __shfl_sync(0xffffffffu, xi[spv], 31);
                        if (lane == 31) {
                            up_k[s] = nx_k;
                            up_i[s] = nx_i;
                        }
                        if (lane == 0) {
                            dn_k[s] = pv_k;
                            dn_i[s] = pv_i;
                        }
                    }
                }
#pragma unroll
                for (int s = 0; s < XSLOTS; s++) {
                    const int j = lane + 32 * s;
                    const bool low = ((j & 1) == phase);  // j pairs with j+1, else with j-1
                    if (low && j < 32 * XSLOTS - 1) {
                        if (xkey_less(up_k[s], up_i[s], xk[s], xi[s])) {
                            xk[s] = up_k[s];
                            xi[s] = up_i[s];
                            swapped = true;
                        }
                    } else if (!low && j > 0) {
                        if (xkey_less(xk[s], xi[s], dn_k[s], dn_i[s])) {
                            xk[s] = dn_k[s];
                            xi[s] = dn_i[s];
                            swapped = true;
                        }
                    }
                }
            }
            if (!__any_sync(0xffffffffu, swapped)) break;
        }
        // certify: exact k-th distance below the smallest exact distance of unlisted points
        bool certified = true;
        if ((int64_t)kp < ns) {
            unsigned long long kk = xk[0];
#pragma unroll
            for (int s = 1; s < XSLOTS; s++)
                if (s == ((k - 1) >> 5)) kk = xk[s];
            kk = __shfl_sync(0xffffffffu, kk, (k - 1) & 31);
            // exact k-th squared distance rounded up vs the squared lower bound of any unlisted
            // point's distance rounded down (no FP64 square roots)
            const float dk2_up = d2f_ru_nonneg_bits(__longlong_as_double((long long)kk));
            const float dt = sqrtf(kth);
            const float floor_unlisted = dt - (errc + u8 * dt) * 1.0001f;
            certified = (kth < INFINITY) && (floor_unlisted > 0.0f) &&
                        (dk2_up < __fmul_rd(floor_unlisted, floor_unlisted) * (1.0f - 1e-6f));
        }
        if (certified) {
#pragma unroll
            for (int s = 0; s < XSLOTS; s++) {
                const int j = lane + 32 * s;
                if (j < k) out[(int64_t)qi * k + j] = xi[s];
            }
        } else if (lane == 0) {
            int slot = atomicAdd(fb_count, 1);
            fb_list[slot] = qi;
        }
    }
}

int grid_blocks(rbf_ctx *ctx, int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    int64_t cap = (int64_t)ctx->num_sms * 16;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

template <int DIM>
int knn_dim(rbf_ctx *ctx, const double *d_data, int64_t ns, const double *d_eval, int64_t ne, int k,
            int32_t *d_idx) {
    // bounding box of the sources
    const int pb = std::min<int64_t>((ns + 255) / 256, 1024);
    DevBuf part;
    RBF_TRY(part.alloc(ctx, sizeof(double) * 6 * pb));
    bbox_partial_kernel<<<pb, 256, 0, ctx->stream>>>(d_data, ns, DIM, part.as<double>());
    RBF_CHECK_LAUNCH(ctx);
    std::vector<double> hp(6 * (size_t)pb);
    RBF_CUDA(ctx, cudaMemcpyAsync(hp.data(), part.ptr, sizeof(double) * 6 * pb, cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int b = 0; b < pb; b++)
        for (int d = 0; d < DIM; d++) {
            lo[d] = std::min(lo[d], hp[b * 6 + d]);
            hi[d] = std::max(hi[d], hp[b * 6 + 3 + d]);
        }
    for (int d = 0; d < DIM; d++)
        if (!std::isfinite(lo[d]) || !std::isfinite(hi[d]))
            return rbf_fail(ctx, RBF_ERR_ARGUMENT, "data points contain non-finite coordinates");

    // cell size: about 1.5 k points expected inside the ball of radius R0 cells
    const int R0 = 2;
    const double unit_ball = DIM == 1 ? 2.0 : (DIM == 2 ? M_PI : 4.0 * M_PI / 3.0);
    double ppc = 1.5 * k / (unit_ball * std::pow((double)R0, DIM));
    if (ppc < 0.5) ppc = 0.5;
    double vol = 1.0;
    int eff = 0;
    for (int d = 0; d < DIM; d++)
        if (hi[d] > lo[d]) {
            vol *= hi[d] - lo[d];
            eff++;
        }
    double target_cells = std::max(1.0, (double)ns / ppc);
    double h = eff > 0 ? std::pow(vol / target_cells, 1.0 / eff) : 1.0;
    GridDesc g{};
    int64_t ncells = 1;
    for (int d = 0; d < 3; d++) {
        if (d >= DIM) {
            g.nc[d] = 1;
            g.lo[d] = 0;
            g.h[d] = 1;
            g.inv_h[d] = 1;
            continue;
        }
        double ext = hi[d] - lo[d];
        int64_t m = ext > 0 ? (int64_t)std::floor(ext / h) : 1;
        m = std::max<int64_t>(1, std::min<int64_t>(m, 1 << 20));
        g.nc[d] = (int)m;
        g.lo[d] = lo[d];
        g.h[d] = ext > 0 ? ext / (double)m : 1.0;
        g.inv_h[d] = 1.0 / g.h[d];
        ncells *= m;
    }
    while (ncells > (int64_t)1 << 27) {  // keep cell starts in int32 and memory modest
        ncells = 1;
        for (int d = 0; d < DIM; d++) {
            g.nc[d] = std::max(1, g.nc[d] / 2);
            g.h[d] = (hi[d] > lo[d]) ? (hi[d] - lo[d]) / g.nc[d] : 1.0;
            g.inv_h[d] = 1.0 / g.h[d];
            ncells *= g.nc[d];
        }
    }
    g.ncells = ncells;
    for (int d = 0; d < 3; d++) {
        g.lof[d] = (float)g.lo[d];
        g.hf[d] = (float)g.h[d];
        g.inv_hf[d] = (float)g.inv_h[d];
    }

    DevBuf cell, count, start, fill, sp, sp32, sidx, qcell, qcount, qstart, qfill, qorder, fb;
    RBF_TRY(cell.alloc(ctx, sizeof(int32_t) * ns));
    RBF_TRY(count.alloc(ctx, sizeof(int32_t) * (ncells + 1)));
    RBF_TRY(start.alloc(ctx, sizeof(int32_t) * (ncells + 1)));
    RBF_TRY(fill.alloc(ctx, sizeof(int32_t) * (ncells + 1)));
    RBF_TRY(sp.alloc(ctx, sizeof(double) * DIM * ns));
    RBF_TRY(sp32.alloc(ctx, sizeof(float4) * ns));
    RBF_TRY(sidx.alloc(ctx, sizeof(int32_t) * ns));
    RBF_CUDA(ctx, cudaMemsetAsync(count.ptr, 0, sizeof(int32_t) * (ncells + 1), ctx->stream));
    RBF_CUDA(ctx, cudaMemsetAsync(fill.ptr, 0, sizeof(int32_t) * (ncells + 1), ctx->stream));
    cell_count_kernel<DIM><<<grid_blocks(ctx, ns, 256), 256, 0, ctx->stream>>>(g, d_data, ns, cell.as<int32_t>(), count.as<int32_t>());
    RBF_CHECK_LAUNCH(ctx);
    RBF_TRY(rbf_exclusive_scan_i32(ctx, count.as<int32_t>(), start.as<int32_t>(), ncells + 1, nullptr));
    cell_scatter_kernel<DIM><<<grid_blocks(ctx, ns, 256), 256, 0, ctx->stream>>>(
        d_data, ns, cell.as<int32_t>(), start.as<int32_t>(), fill.as<int32_t>(), sp.as<double>(), sp32.as<float4>(),
        sidx.as<int32_t>());
    RBF_CHECK_LAUNCH(ctx);

    // visit queries in cell order
    RBF_TRY(qcell.alloc(ctx, sizeof(int32_t) * ne));
    RBF_TRY(qcount.alloc(ctx, sizeof(int32_t) * (ncells + 1)));
    RBF_TRY(qstart.alloc(ctx, sizeof(int32_t) * (ncells + 1)));
    RBF_TRY(qfill.alloc(ctx, sizeof(int32_t) * (ncells + 1)));
    RBF_TRY(qorder.alloc(ctx, sizeof(int32_t) * ne));
    RBF_CUDA(ctx, cudaMemsetAsync(qcount.ptr, 0, sizeof(int32_t) * (ncells + 1), ctx->stream));
    RBF_CUDA(ctx, cudaMemsetAsync(qfill.ptr, 0, sizeof(int32_t) * (ncells + 1), ctx->stream));
    cell_count_kernel<DIM><<<grid_blocks(ctx, ne, 256), 256, 0, ctx->stream>>>(g, d_eval, ne, qcell.as<int32_t>(), qcount.as<int32_t>());
    RBF_CHECK_LAUNCH(ctx);
    RBF_TRY(rbf_exclusive_scan_i32(ctx, qcount.as<int32_t>(), qstart.as<int32_t>(), ncells + 1, nullptr));
    cell_scatter_kernel<DIM><<<grid_blocks(ctx, ne, 256), 256, 0, ctx->stream>>>(
        d_eval, ne, qcell.as<int32_t>(), qstart.as<int32_t>(), qfill.as<int32_t>(), nullptr, nullptr,
        qorder.as<int32_t>());
    RBF_CHECK_LAUNCH(ctx);

    int64_t blocks = (ne + KNN_WARPS - 1) / KNN_WARPS;
    int64_t cap = (int64_t)ctx->num_sms * 32;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    // FP32 search with an exact FP64 re-sort of kp candidates: k + 8, or 32 for 25 <= k <= 30 so
    // that the re-rank fits one register per lane (a margin of at least two neighbours, whose
    // distances differ by far more than the FP32 error bound except at near-ties); queries
    // whose FP32 margins do not certify the exact order go to the FP64 search below
    const int kp = (k >= 25 && k <= 30) ? 32 : std::min(k + 8, 64);
    float mag = 0.f;
    for (int d = 0; d < DIM; d++) mag = std::max(mag, (float)std::max(std::fabs(lo[d]), std::fabs(hi[d])));
    RBF_TRY(fb.alloc(ctx, sizeof(int32_t) * (ne + 1)));
    RBF_CUDA(ctx, cudaMemsetAsync(fb.as<int32_t>() + ne, 0, sizeof(int32_t), ctx->stream));
    // list of 32 SLOTS entries, re-rank of kp in 32 XSLOTS (k + 8 <= 32: one register each)
    if (k + 8 <= 32)
        knn_fast_kernel<DIM, 1, 1><<<(unsigned)blocks, KNN_WARPS * 32, 0, ctx->stream>>>(
            g, sp32.as<float4>(), sidx.as<int32_t>(), start.as<int32_t>(), d_data, d_eval, qorder.as<int32_t>(), ne,
            k, kp, R0, mag, ns, d_idx, fb.as<int32_t>(), fb.as<int32_t>() + ne);
    else if (kp <= 32)
        knn_fast_kernel<DIM, 2, 1><<<(unsigned)blocks, KNN_WARPS * 32, 0, ctx->stream>>>(
            g, sp32.as<float4>(), sidx.as<int32_t>(), start.as<int32_t>(), d_data, d_eval, qorder.as<int32_t>(), ne,
            k, kp, R0, mag, ns, d_idx, fb.as<int32_t>(), fb.as<int32_t>() + ne);
    else
        knn_fast_kernel<DIM, 2, 2><<<(unsigned)blocks, KNN_WARPS * 32, 0, ctx->stream>>>(
            g, sp32.as<float4>(), sidx.as<int32_t>(), start.as<int32_t>(), d_data, d_eval, qorder.as<int32_t>(), ne,
            k, kp, R0, mag, ns, d_idx, fb.as<int32_t>(), fb.as<int32_t>() + ne);
    RBF_CHECK_LAUNCH(ctx);
    int32_t nfb = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&nfb, fb.as<int32_t>() + ne, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->knn_fallback += nfb;
    if (nfb > 0) {
        int64_t fblocks = std::min<int64_t>((nfb + KNN_WARPS - 1) / KNN_WARPS, cap);
        if (k <= 32)
            knn_query_kernel<DIM, 1><<<(unsigned)fblocks, KNN_WARPS * 32, 0, ctx->stream>>>(
                g, sp.as<double>(), sidx.as<int32_t>(), start.as<int32_t>(), d_eval, fb.as<int32_t>(), nfb, k, R0, d_idx);
        else
            knn_query_kernel<DIM, 2><<<(unsigned)fblocks, KNN_WARPS * 32, 0, ctx->stream>>>(
                g, sp.as<double>(), sidx.as<int32_t>(), start.as<int32_t>(), d_eval, fb.as<int32_t>(), nfb, k, R0, d_idx);
        RBF_CHECK_LAUNCH(ctx);
    }
    return RBF_OK;
}

}  // namespace

int rbf_knn_device(rbf_ctx *ctx, const double *d_data, int64_t ns, const double *d_eval, int64_t ne, int dim,
                   int k, int32_t *d_idx) {
    if (ne == 0) return RBF_OK;
    switch (dim) {
    case 1: return knn_dim<1>(ctx, d_data, ns, d_eval, ne, k, d_idx);
    case 2: return knn_dim<2>(ctx, d_data, ns, d_eval, ne, k, d_idx);
    case 3: return knn_dim<3>(ctx, d_data, ns, d_eval, ne, k, d_idx);
    default: return rbf_fail(ctx, RBF_ERR_ARGUMENT, "dim must be 1, 2 or 3 (got %d)", dim);
    }
}
