// Batched build of uneven stencils: one persistent kernel over size classes.
//
// A batched build takes ragged stencils (the neighbours of eval point e are
// adj_idx[adj_ptr[e] .. adj_ptr[e+1])) with a polynomial degree per stencil, and Hermite
// boundary stencils in the reference formulation.  Stencils are binned by size class
// (stencil size k, degree: the system size n = k + nmon) with a counting sort on the
// device; every class has its own StencilParams (k, n, monomial table) in a BinDesc.
// One persistent launch then drains a global work queue (one atomic per item): an item is
// four stencils of a class on the block's four warps (warp tile) or one stencil on the
// whole block (block tile, the O(n^3) factorisations shared by 128 threads).  Classes are
// queued largest system first so the long items start early.  Which tile each class
// uses is decided by an autotuner that times both tiles on a sample of the class and
// caches the choice in the context (rbf_tuning_report prints the table).
//
// The per-stencil work is that of the one-size kernels: FP64 warp tiles run the
// Bunch-Kaufman solve of the default plain build (stencil_bk.cuh); FP64 block tiles run a
// block-cooperative LU, bit-identical to the one-warp LU that the one-size build uses under
// RBF_FLAG_FP64_LU; the refined tiles' FP32 factorisations are bit-identical between the two
// tile shapes (stencil_solve.cuh).
#include <algorithm>
#include <cstring>
#include <vector>

#include "stencil_bk.cuh"
#include "stencil_solve.cuh"

namespace {

constexpr int kKeys = kRbfBatchKeys;  // (m * 65 + k) * 8 + (degree + 1)

__device__ int nmon_of(int dim, int deg) {
    if (deg < 0) return 0;
    // binomial(dim + deg, dim)
    int r = 1;
    for (int i = 1; i <= dim; i++) r = r * (deg + i) / i;
    return r;
}

// Class key of every stencil and the class histogram; err: bit 0 stencil size out of
// range, bit 1 system too large, bit 2 degree out of range, bit 3 adj_ptr not monotone.
// nd (RBF_FLAG_NORMAL_DOF builds, else null adj_idx): m, the stencil's Neumann/Robin
// neighbours, enters the key; Dirichlet eval stencils (identity rows) count none.
struct NormalDofView {
    const int32_t *adj_idx;
    const uint8_t *isb;
    const int32_t *g2b;
    const double *alpha, *beta;
};

__global__ void classify_kernel(int64_t ne, int dim, const int64_t *__restrict__ adj_ptr,
                                const int8_t *__restrict__ degs, int def_deg, NormalDofView nd,
                                int32_t *__restrict__ key, unsigned long long *__restrict__ hist,
                                int *__restrict__ err) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t len = adj_ptr[e + 1] - adj_ptr[e];
        const int deg = degs ? (int)degs[e] : def_deg;
        int bad = 0;
        if (len < 0) bad |= 8;
        if (len < 1 || len > RBF_MAX_STENCIL) bad |= 1;
        if (deg < -1 || deg > 6) bad |= 4;
        int m = 0;
        if (!bad && nd.adj_idx && nd.isb &&
            !(nd.isb[e] && nd.alpha[nd.g2b[e]] == 1.0 && nd.beta[nd.g2b[e]] == 0.0)) {
            for (int64_t t = adj_ptr[e]; t < adj_ptr[e + 1]; t++) {
                const int32_t g = nd.adj_idx[t];
                if (nd.isb[g]) m += !(nd.alpha[nd.g2b[g]] == 1.0 && nd.beta[nd.g2b[g]] == 0.0);
            }
        }
        if (!bad && len + m + nmon_of(dim, deg) > RBF_MAX_SYSTEM) bad |= 2;
        if (bad) {
            atomicOr(err, bad);
            key[e] = -1;
            continue;
        }
        const int kk = (m * 65 + (int)len) * 8 + deg + 1;
        key[e] = kk;
        atomicAdd(&hist[kk], 1ull);
    }
}

// Counting-sort scatter of the stencils into their class's slot range.
__global__ void scatter_slots_kernel(int64_t ne, const int32_t *__restrict__ key, const int *__restrict__ class_of_key,
                                     unsigned long long *__restrict__ cursor, int32_t *__restrict__ slots) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        const int kk = key[e];
        if (kk < 0) continue;
        const int c = class_of_key[kk];
        const unsigned long long pos = atomicAdd(&cursor[c], 1ull);
        slots[pos] = (int32_t)e;
    }
}

struct BlockScratch {
    double redv[4];
    float redvf[4];
    int redi[4];
    int flag, es, accepted;
};

// One stencil on the whole block, plain FP64: warp 0 loads, assembles and scatters, every
// thread factorises.
template <bool ND>
__device__ void solve_fp64_block(const StencilParams &P, int64_t e, const WarpSmem &w, int tid, int G,
                                 BlockScratch &bs) {
    const int lane = tid & 31;
    if (tid < 32) {
        int es = 0, eval_local = -2;
        const int st = load_stencil(P, e, w, lane, &es, &eval_local);
        if (st == 0) assemble_fp64<ND>(P, w, lane, es, eval_local);
        if (lane == 0) {
            bs.flag = st;
            bs.es = es;
        }
    }
    __syncthreads();
    if (bs.flag != 0) return;
    const bool ok = lu_solve_fp64_block(w.M, P.n, P.nops, tid, G, bs.redv, bs.redi);
    if (tid < 32) {
        if (!ok) {
            if (lane == 0) {
                if (P.status) P.status[e] = 1;
                atomicAdd(&P.counters[0], 1ull);
            }
        } else {
            scatter_row(P, e, w, lane, bs.es, w.M + P.n, mat_ld(P.n, P.nops), 1);
            if (lane == 0 && P.status) P.status[e] = 0;
        }
    }
}

// One stencil on the whole block, FP32 factor + FP64 refinement: every thread factorises,
// warp 0 refines (O(n^2) per step); the FP64 fallback is factorised by the block again.
template <bool ND>
__device__ void solve_fp32r_block(const StencilParams &P, int64_t e, const WarpSmem &w, const Warp32 &u, int tid,
                                  int G, BlockScratch &bs) {
    const int lane = tid & 31;
    int es = 0, eval_local = -2;
    if (tid < 32) {
        const int st = load_stencil(P, e, w, lane, &es, &eval_local);
        if (st == 0) assemble_refined<ND>(P, w, u, lane, es, eval_local);
        if (lane == 0) {
            bs.flag = st;
            bs.es = es;
        }
    }
    __syncthreads();
    if (bs.flag != 0) return;
    const bool ok = lu_factor_fp32_block(u.F, u.piv, P.n, tid, G, bs.redvf, bs.redi);
    if (tid < 32) {
        double est = 0.0;
        const bool acc = ok && refine_fp32_warp(P, w, u, lane, &est);
        if (acc) {
            scatter_row(P, e, w, lane, es, u.x, P.nops, 1);
            if (lane == 0) {
                if (P.status) P.status[e] = 0;
                atomicMax(reinterpret_cast<unsigned long long *>(P.max_resid),
                          (unsigned long long)__double_as_longlong(est));
            }
        } else if (eval_local == -2) {
            assemble_fp64(P, w, lane, es, eval_local);
        }
        if (lane == 0) bs.accepted = acc ? 1 : 0;
    }
    __syncthreads();
    if (bs.accepted) return;
    const bool ok64 = lu_solve_fp64_block(w.M, P.n, P.nops, tid, G, bs.redv, bs.redi);
    if (tid < 32) {
        if (ok64) {
            scatter_row(P, e, w, lane, bs.es, w.M + P.n, mat_ld(P.n, P.nops), 1);
            if (lane == 0) {
                if (P.status) P.status[e] = 3;
                atomicAdd(&P.counters[2], 1ull);
            }
        } else if (lane == 0) {
            if (P.status) P.status[e] = 1;
            atomicAdd(&P.counters[0], 1ull);
        }
    }
}

constexpr int kBatchedThreads = 128;

// The persistent kernel: blocks take items from the queue until it is drained.  The
// current class's descriptor is kept in shared memory (reloaded when the class changes).
__global__ void __launch_bounds__(kBatchedThreads) build_batched_kernel(const BinDesc *__restrict__ bins, int nbins,
                                                                        int64_t n_items,
                                                                        unsigned long long *__restrict__ queue,
                                                                        size_t region) {
    extern __shared__ __align__(16) char smem[];
    __shared__ long long s_item;
    __shared__ __align__(16) BinDesc s_bin;
    __shared__ BlockScratch bs;
    const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
    int cur = -1;
    for (;;) {
        if (tid == 0) s_item = (long long)atomicAdd(queue, 1ull);
        __syncthreads();
        const long long item = s_item;
        if (item >= n_items) break;
        int b = 0;
        while (b + 1 < nbins && bins[b + 1].item_start <= item) b++;
        if (b != cur) {
            const int *src = reinterpret_cast<const int *>(&bins[b]);
            int *dst = reinterpret_cast<int *>(&s_bin);
            for (int t = tid; t < (int)(sizeof(BinDesc) / sizeof(int)); t += blockDim.x) dst[t] = src[t];
            cur = b;
            __syncthreads();
        }
        const StencilParams &P = s_bin.P;
        const bool nd = P.nnr > 0;  // classes with du/dn unknowns take the ND instantiations
        if (s_bin.tile == 0) {
            const int64_t slot = (item - s_bin.item_start) * 4 + wib;
            if (slot < s_bin.count) {
                char *base = smem + wib * region;
                const WarpSmem w = carve(base, P.n, P.k, P.nops);
                const int64_t e = s_bin.slots[slot];
                if (s_bin.precision == RBF_PREC_FP64) {
                    const BKSmem bk = carve_bk(base, P.n, P.k, P.nops);
                    if (nd)
                        solve_fp64_bk_warp<true>(P, e, bk, lane);
                    else
                        solve_fp64_bk_warp<false>(P, e, bk, lane);
                } else {
                    const Warp32 u = carve32(base, P.n, P.k, P.nops);
                    if (nd)
                        solve_fp32r_warp<true>(P, e, w, u, lane);
                    else
                        solve_fp32r_warp<false>(P, e, w, u, lane);
                }
            }
        } else {
            const int64_t e = s_bin.slots[item - s_bin.item_start];
            const WarpSmem w = carve(smem, P.n, P.k, P.nops);
            if (s_bin.precision == RBF_PREC_FP64) {
                if (nd)
                    solve_fp64_block<true>(P, e, w, tid, blockDim.x, bs);
                else
                    solve_fp64_block<false>(P, e, w, tid, blockDim.x, bs);
            } else {
                const Warp32 u = carve32(smem, P.n, P.k, P.nops);
                if (nd)
                    solve_fp32r_block<true>(P, e, w, u, tid, blockDim.x, bs);
                else
                    solve_fp32r_block<false>(P, e, w, u, tid, blockDim.x, bs);
            }
        }
        __syncthreads();
    }
}

int grid_for(rbf_ctx *ctx, int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
}

}  // namespace

int rbf_build_fp32_launch(rbf_ctx *ctx, const StencilParams &P);

// Classes the split tile serves: FP32-refined 40-row systems with one operator and no
// normal-derivative unknowns, the sizes of the split-row register kernel (stencil_refined_c.cu).
static bool split_tile_serves(const BinDesc &b) {
    return b.precision == RBF_PREC_FP32_REFINED && b.P.n == 40 && b.P.nops == 1 && b.P.nnr == 0;
}

size_t rbf_batched_region(int n, int k, int nops, int precision) {
    // FP64 warp tiles solve by Bunch-Kaufman on the packed system, block tiles by the LU on the
    // full one: room for either
    const size_t b = precision == RBF_PREC_FP64 ? std::max(warp_smem_bytes(n, k, nops), bk_warp_bytes(n, k, nops))
                                                : warp_smem_bytes32(n, k, nops);
    return (b + 15) & ~(size_t)15;
}

int rbf_batched_classify(rbf_ctx *ctx, int64_t ne, int dim, const int64_t *d_adj_ptr, const int8_t *d_degs,
                         int def_deg, const StencilParams *nd, int32_t *d_key, std::vector<unsigned long long> &hist,
                         int *err) {
    NormalDofView v{nullptr, nullptr, nullptr, nullptr, nullptr};
    if (nd && nd->isb) v = NormalDofView{nd->adjl, nd->isb, nd->g2b, nd->alpha, nd->beta};
    hist.assign(kKeys, 0ull);
    DevBuf dh, de;
    RBF_TRY(dh.alloc(ctx, sizeof(unsigned long long) * kKeys));
    RBF_TRY(de.alloc(ctx, sizeof(int)));
    RBF_CUDA(ctx, cudaMemsetAsync(dh.ptr, 0, sizeof(unsigned long long) * kKeys, ctx->stream));
    RBF_CUDA(ctx, cudaMemsetAsync(de.ptr, 0, sizeof(int), ctx->stream));
    if (ne > 0) {
        classify_kernel<<<grid_for(ctx, ne), 256, 0, ctx->stream>>>(ne, dim, d_adj_ptr, d_degs, def_deg, v, d_key,
                                                                    dh.as<unsigned long long>(), de.as<int>());
        RBF_CHECK_LAUNCH(ctx);
    }
    RBF_CUDA(ctx, cudaMemcpyAsync(hist.data(), dh.ptr, sizeof(unsigned long long) * kKeys, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    RBF_CUDA(ctx, cudaMemcpyAsync(err, de.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

int rbf_batched_scatter(rbf_ctx *ctx, int64_t ne, const int32_t *d_key, const std::vector<int> &class_of_key,
                        const std::vector<unsigned long long> &class_start, int32_t *d_slots) {
    DevBuf dmap, dcur;
    RBF_TRY(dmap.alloc(ctx, sizeof(int) * kKeys));
    RBF_TRY(dcur.alloc(ctx, sizeof(unsigned long long) * class_start.size()));
    RBF_CUDA(ctx, cudaMemcpyAsync(dmap.ptr, class_of_key.data(), sizeof(int) * kKeys, cudaMemcpyHostToDevice,
                                  ctx->stream));
    RBF_CUDA(ctx, cudaMemcpyAsync(dcur.ptr, class_start.data(), sizeof(unsigned long long) * class_start.size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
    if (ne > 0) {
        scatter_slots_kernel<<<grid_for(ctx, ne), 256, 0, ctx->stream>>>(ne, d_key, dmap.as<int>(),
                                                                         dcur.as<unsigned long long>(), d_slots);
        RBF_CHECK_LAUNCH(ctx);
    }
    // the host vectors are read by the copies above: wait before they go out of scope
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

// One persistent launch over the warp- and block-tile classes in `bins` (their item_start
// fields are filled here), with room for the largest of their systems.
static int run_persistent(rbf_ctx *ctx, std::vector<BinDesc> &bins) {
    int64_t items = 0;
    size_t region = 16;
    for (auto &b : bins) {
        b.item_start = items;
        items += b.tile == 0 ? (b.count + 3) / 4 : b.count;
        region = std::max(region, rbf_batched_region(b.P.n, b.P.k, b.P.nops, b.precision));
    }
    if (items == 0) return RBF_OK;
    const size_t smem = 4 * region;
    if (smem > 227 * 1024) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "batched build: system too large for shared memory");
    DevBuf dbins, dq;
    RBF_TRY(dbins.alloc(ctx, sizeof(BinDesc) * bins.size()));
    RBF_TRY(dq.alloc(ctx, sizeof(unsigned long long)));
    RBF_CUDA(ctx, cudaMemcpyAsync(dbins.ptr, bins.data(), sizeof(BinDesc) * bins.size(), cudaMemcpyHostToDevice,
                                  ctx->stream));
    RBF_CUDA(ctx, cudaMemsetAsync(dq.ptr, 0, sizeof(unsigned long long), ctx->stream));
    RBF_CUDA(ctx, cudaFuncSetAttribute(build_batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_batched_kernel, kBatchedThreads, smem));
    if (per_sm < 1) per_sm = 1;
    const int64_t grid = std::min<int64_t>(items, (int64_t)ctx->num_sms * per_sm);
    build_batched_kernel<<<(unsigned)grid, kBatchedThreads, smem, ctx->stream>>>(
        dbins.as<BinDesc>(), (int)bins.size(), items, dq.as<unsigned long long>(), region);
    RBF_CHECK_LAUNCH(ctx);
    // the descriptor copy reads host memory: complete it before the vector can change
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

// Runs each split-tile class on the split-row register kernel (the general refined kernel
// finishing what it hands over; defer: room for the largest such class's stencil count),
// then the warp- and block-tile classes in persistent launches grouped by occupancy: the
// shared memory of a launch is set by its largest system, so classes whose systems allow
// more resident blocks per SM (the common interior class beside a few larger boundary
// classes) get a launch of their own instead of running at the larger classes' occupancy.
int rbf_batched_run(rbf_ctx *ctx, std::vector<BinDesc> &bins, int32_t *defer) {
    if (bins.empty()) return RBF_OK;
    for (auto &b : bins) b.item_start = 0;
    for (const auto &b : bins) {
        if (b.tile != kTileSplit || b.count == 0) continue;
        if (!defer) return rbf_fail(ctx, RBF_ERR_INTERNAL, "split tile without a deferred list");
        StencilParams Ps = b.P;
        Ps.slots = b.slots;
        Ps.nslots = b.count;
        Ps.defer = defer;
        RBF_CUDA(ctx, cudaMemsetAsync(&Ps.counters[7], 0, sizeof(unsigned long long), ctx->stream));
        RBF_TRY(rbf_build_fp32_launch(ctx, Ps));
    }
    // resident blocks per SM of each remaining class at its own shared memory
    std::vector<std::pair<int, size_t>> occ;  // (blocks per SM, index into bins)
    for (size_t i = 0; i < bins.size(); i++) {
        const BinDesc &b = bins[i];
        if (b.tile == kTileSplit || b.count == 0) continue;
        const size_t smem = 4 * rbf_batched_region(b.P.n, b.P.k, b.P.nops, b.precision);
        if (smem > 227 * 1024) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "batched build: system too large for shared memory");
        RBF_CUDA(ctx, cudaFuncSetAttribute(build_batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        RBF_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_batched_kernel, kBatchedThreads, smem));
        occ.push_back({per_sm, i});
    }
    // one launch per occupancy level, the highest first (classes keep their largest-system-
    // first order within a launch)
    std::stable_sort(occ.begin(), occ.end(), [](const std::pair<int, size_t> &a, const std::pair<int, size_t> &c) {
        return a.first > c.first;
    });
    for (size_t g = 0; g < occ.size();) {
        size_t h = g;
        std::vector<BinDesc> group;
        while (h < occ.size() && occ[h].first == occ[g].first) group.push_back(bins[occ[h++].second]);
        RBF_TRY(run_persistent(ctx, group));
        g = h;
    }
    return RBF_OK;
}

// Key of a size class in the tuning cache.
unsigned long long rbf_tune_key(const BinDesc &b, bool boundary) {
    const StencilParams &P = b.P;
    return (unsigned long long)b.precision | ((unsigned long long)P.dim << 4) | ((unsigned long long)P.phs << 8) |
           ((unsigned long long)P.nops << 12) | ((unsigned long long)P.k << 16) |
           ((unsigned long long)(P.poly_deg + 1) << 24) | ((unsigned long long)boundary << 28) |
           ((unsigned long long)P.op_code[0] << 32) | ((unsigned long long)P.nnr << 40);
}

// Chooses each class's tile: a cached choice, or (tune >= 1) the faster of the two tiles
// on a sample of up to 16384 stencils of the class, timed on the context's stream; the
// trial runs write the real outputs of the sampled stencils (the final run rewrites
// them) and count into scratch counters.  Classes too small to time get the warp tile
// below n = 64 and the block tile above.
int rbf_batched_tune(rbf_ctx *ctx, std::vector<BinDesc> &bins, bool boundary, int tune, int32_t *defer) {
    DevBuf scratch;
    RBF_TRY(scratch.alloc(ctx, sizeof(unsigned long long) * 8 + sizeof(double)));
    for (auto &b : bins) {
        const unsigned long long key = rbf_tune_key(b, boundary);
        auto it = ctx->tune.find(key);
        if (it != ctx->tune.end() && tune < 2) {
            b.tile = it->second.tile;
            continue;
        }
        const bool split_ok = split_tile_serves(b) && defer;
        if (tune == 0 || b.count < 1024) {
            b.tile = split_ok ? kTileSplit : (b.P.n > 64 ? 1 : 0);
            continue;
        }
        rbf_tune_entry ent;
        ent.sample = std::min<int64_t>(b.count, 16384);
        float ms[3] = {0.f, 0.f, 0.f};
        for (int tile = 0; tile < (split_ok ? 3 : 2); tile++) {
            std::vector<BinDesc> one(1, b);
            one[0].count = ent.sample;
            one[0].tile = tile;
            one[0].P.counters = scratch.as<unsigned long long>();
            one[0].P.max_resid = reinterpret_cast<double *>(scratch.as<unsigned long long>() + 8);
            RBF_TRY(rbf_batched_run(ctx, one, defer));  // warm-up (module load, caches)
            cudaEvent_t e0, e1;
            RBF_CUDA(ctx, cudaEventCreate(&e0));
            RBF_CUDA(ctx, cudaEventCreate(&e1));
            cudaEventRecord(e0, ctx->stream);
            int st = rbf_batched_run(ctx, one, defer);
            cudaEventRecord(e1, ctx->stream);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms[tile], e0, e1);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            RBF_TRY(st);
        }
        ent.ms_warp = ms[0];
        ent.ms_block = ms[1];
        ent.ms_split = split_ok ? ms[2] : 0.f;
        ent.tile = ms[1] < ms[0] ? 1 : 0;
        if (split_ok && ms[2] < ms[ent.tile]) ent.tile = kTileSplit;
        ctx->tune[key] = ent;
        b.tile = ent.tile;
    }
    return RBF_OK;
}
