// C ABI of librbffd_gb300.so: contexts, argument checks (with the reference's error
// classes), host/device pointer staging and the orchestration of the kernels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "rbf_internal.cuh"
#include "stencil_common.cuh"

int rbf_build_fp64_launch(rbf_ctx *ctx, const StencilParams &P);
int rbf_build_fp32_launch(rbf_ctx *ctx, const StencilParams &P);
int rbf_batched_classify(rbf_ctx *ctx, int64_t ne, int dim, const int64_t *d_adj_ptr, const int8_t *d_degs,
                         int def_deg, const StencilParams *nd, int32_t *d_key, std::vector<unsigned long long> &hist,
                         int *err);
int rbf_batched_scatter(rbf_ctx *ctx, int64_t ne, const int32_t *d_key, const std::vector<int> &class_of_key,
                        const std::vector<unsigned long long> &class_start, int32_t *d_slots);
int rbf_batched_tune(rbf_ctx *ctx, std::vector<BinDesc> &bins, bool boundary, int tune, int32_t *defer);
int rbf_batched_run(rbf_ctx *ctx, std::vector<BinDesc> &bins, int32_t *defer);

int rbf_fail(rbf_ctx *ctx, int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (ctx) ctx->last_error = buf;
    return code;
}

bool rbf_is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int InArray::bind(rbf_ctx *ctx, const void *p, size_t bytes) {
    if (!p || bytes == 0 || rbf_is_device_ptr(p)) {
        dptr = p;
        return RBF_OK;
    }
    RBF_TRY(staged.alloc(ctx, bytes));
    RBF_CUDA(ctx, cudaMemcpyAsync(staged.ptr, p, bytes, cudaMemcpyHostToDevice, ctx->stream));
    dptr = staged.ptr;
    return RBF_OK;
}

int OutArray::bind(rbf_ctx *ctx, void *p, size_t bytes_) {
    user = p;
    bytes = bytes_;
    if (!p || bytes == 0 || rbf_is_device_ptr(p)) {
        dptr = p;
        host = false;
        return RBF_OK;
    }
    host = true;
    RBF_TRY(staged.alloc(ctx, bytes));
    dptr = staged.ptr;
    return RBF_OK;
}

int OutArray::finish(rbf_ctx *ctx) {
    if (host && bytes) RBF_CUDA(ctx, cudaMemcpyAsync(user, dptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return RBF_OK;
}

namespace {

int binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    long r = 1;
    for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
    return (int)r;
}

void multiexp(int slots, int remaining, int pos, int *cur, std::vector<std::vector<int>> &out) {
    if (pos == slots) {
        out.emplace_back(cur, cur + slots);
        return;
    }
    for (int e = remaining; e >= 0; e--) {
        if (pos == slots - 1 && e != remaining) break;
        cur[pos] = e;
        multiexp(slots, remaining - e, pos + 1, cur, out);
    }
}

// Monomial exponents in the reference's order (src/basis/monomial.jl:27-123): hand-coded
// evaluators for 1D and for 2D/3D up to degree 2, Combinatorics.multiexponents(dim+1, deg)
// (reverse lexicographic, last entry the slack) otherwise.
int monomial_exponents(int dim, int deg, int8_t (*ex)[3]) {
    if (deg < 0) return 0;
    int nmon = binom(dim + deg, dim);
    for (int m = 0; m < nmon; m++) ex[m][0] = ex[m][1] = ex[m][2] = 0;
    if (deg == 0) return 1;
    if (dim == 1) {
        for (int j = 0; j <= deg; j++) ex[j][0] = (int8_t)j;
        return nmon;
    }
    static const int t21[3][2] = {{0, 0}, {1, 0}, {0, 1}};
    static const int t22[6][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}, {2, 0}, {0, 2}};
    static const int t31[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    static const int t32[10][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0},
                                   {1, 0, 1}, {0, 1, 1}, {2, 0, 0}, {0, 2, 0}, {0, 0, 2}};
    if (dim == 2 && deg == 1) {
        for (int m = 0; m < 3; m++) ex[m][0] = t21[m][0], ex[m][1] = t21[m][1];
        return nmon;
    }
    if (dim == 2 && deg == 2) {
        for (int m = 0; m < 6; m++) ex[m][0] = t22[m][0], ex[m][1] = t22[m][1];
        return nmon;
    }
    if (dim == 3 && deg == 1) {
        for (int m = 0; m < 4; m++) ex[m][0] = t31[m][0], ex[m][1] = t31[m][1], ex[m][2] = t31[m][2];
        return nmon;
    }
    if (dim == 3 && deg == 2) {
        for (int m = 0; m < 10; m++) ex[m][0] = t32[m][0], ex[m][1] = t32[m][1], ex[m][2] = t32[m][2];
        return nmon;
    }
    std::vector<std::vector<int>> all;
    int cur[8];
    multiexp(dim + 1, deg, 0, cur, all);
    for (int m = 0; m < nmon; m++)
        for (int d = 0; d < dim; d++) ex[m][d] = (int8_t)all[m][d];
    return nmon;
}

int op_order(int code) {
    switch (code) {
    case RBF_OP_IDENTITY: return 0;
    case RBF_OP_PARTIAL1: return 1;
    default: return 2;
    }
}

// Operator codes of a build configuration into P (op_code, op_dim, op_order).
int set_operators(rbf_ctx *ctx, const rbf_build_cfg *cfg, StencilParams &P) {
    const int dim = cfg->dim;
    for (int r = 0; r < cfg->nops; r++) {
        int c = cfg->op_code[r];
        if (c < RBF_OP_IDENTITY || c > RBF_OP_LAPLACIAN) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "unknown operator code %d", c);
        if ((c == RBF_OP_PARTIAL1 || c == RBF_OP_PARTIAL2) && (cfg->op_dim[r] < 0 || cfg->op_dim[r] >= dim))
            return rbf_fail(ctx, RBF_ERR_ARGUMENT, "partial derivative dimension %d out of range", cfg->op_dim[r]);
        P.op_code[r] = c;
        P.op_dim[r] = (c == RBF_OP_PARTIAL1 || c == RBF_OP_PARTIAL2) ? cfg->op_dim[r] : 0;
        P.op_order[r] = op_order(c);
    }
    return RBF_OK;
}

int check_ctx(rbf_ctx *ctx) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != ctx->device) RBF_CUDA(ctx, cudaSetDevice(ctx->device));
    return RBF_OK;
}

// Boundary bookkeeping shared by rbf_build_count and rbf_build.
struct BoundaryDev {
    InArray isb, alpha, beta, normals;
    DevBuf g2b;
    int64_t nb = 0;
    bool any = false;
    bool any_nr = false;
};

int bind_boundary(rbf_ctx *ctx, const rbf_hermite *h, int64_t ns, int dim, BoundaryDev &b) {
    if (!h || !h->is_boundary) return RBF_OK;
    b.any = true;
    if (h->n_boundary < 0) return rbf_fail(ctx, RBF_ERR_DIMENSION, "n_boundary must be >= 0");
    RBF_TRY(b.isb.bind(ctx, h->is_boundary, (size_t)ns));
    RBF_TRY(b.alpha.bind(ctx, h->alpha, sizeof(double) * h->n_boundary));
    RBF_TRY(b.beta.bind(ctx, h->beta, sizeof(double) * h->n_boundary));
    RBF_TRY(b.normals.bind(ctx, h->normals, sizeof(double) * h->n_boundary * dim));
    RBF_TRY(b.g2b.alloc(ctx, sizeof(int32_t) * (ns + 1)));
    RBF_TRY(rbf_boundary_map_device(ctx, ns, b.isb.as<uint8_t>(), b.g2b.as<int32_t>(), &b.nb));
    // _validate_boundary_inputs (src/solve/api.jl:96-116)
    if (b.nb != h->n_boundary)
        return rbf_fail(ctx, RBF_ERR_DIMENSION,
                        "boundary_conditions (%lld) and normals (%lld) must each have one entry per boundary "
                        "point (count(is_boundary) = %lld)",
                        (long long)h->n_boundary, (long long)h->n_boundary, (long long)b.nb);
    if (b.nb > 0) {
        std::vector<double> a(b.nb), be(b.nb);
        RBF_CUDA(ctx, cudaMemcpyAsync(a.data(), b.alpha.dptr, sizeof(double) * b.nb, cudaMemcpyDeviceToHost, ctx->stream));
        RBF_CUDA(ctx, cudaMemcpyAsync(be.data(), b.beta.dptr, sizeof(double) * b.nb, cudaMemcpyDeviceToHost, ctx->stream));
        RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int64_t i = 0; i < b.nb; i++)
            if (!(a[i] == 1.0 && be[i] == 0.0)) b.any_nr = true;
    }
    return RBF_OK;
}

}  // namespace

// Basis, operator and precision fields of P for a plan (P.k set by the caller).
int rbf_plan_params(rbf_ctx *ctx, const rbf_build_cfg *cfg, StencilParams &P) {
    const int dim = cfg->dim;
    if (cfg->flags & RBF_FLAG_NORMAL_DOF)
        return rbf_fail(ctx, RBF_ERR_UNSUPPORTED, "normal-derivative unknowns are built by rbf_build_batched");
    if (dim < 1 || dim > 3) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "dim must be 1, 2 or 3 (got %d)", dim);
    if (!(cfg->phs == 1 || cfg->phs == 3 || cfg->phs == 5 || cfg->phs == 7))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "n must be 1, 3, 5, or 7 (got n=%d)", cfg->phs);
    if (cfg->poly_deg < -1) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "poly_deg must be >= -1 (got %d)", cfg->poly_deg);
    if (cfg->nops < 1 || cfg->nops > RBF_MAX_OPS) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "nops must be in 1..%d", RBF_MAX_OPS);
    RBF_TRY(set_operators(ctx, cfg, P));
    P.nmon = monomial_exponents(dim, cfg->poly_deg, P.exps);
    if (P.k + P.nmon > RBF_MAX_SYSTEM)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "k + number of monomials (%d) exceeds %d", P.k + P.nmon, RBF_MAX_SYSTEM);
    P.dim = dim;
    P.phs = cfg->phs;
    P.poly_deg = cfg->poly_deg;
    P.n = P.k + P.nmon;
    P.nops = cfg->nops;
    P.refine_steps = cfg->refine_steps > 0 ? cfg->refine_steps : 6;
    P.tol = cfg->tol > 0 ? cfg->tol : 1e-9;
    P.flags = cfg->flags;
    return RBF_OK;
}

extern "C" {

const char *rbf_version(void) { return "rbffd-gb300 0.1.0 (sm_103a)"; }

int rbf_ctx_create(int device, rbf_ctx **out) {
    if (!out) return RBF_ERR_ARGUMENT;
    *out = nullptr;
    rbf_ctx *ctx = new rbf_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        delete ctx;
        cudaGetLastError();
        return RBF_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
    return RBF_OK;
}

int rbf_ctx_destroy(rbf_ctx *ctx) {
    if (!ctx) return RBF_OK;
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->own_stream);
        cudaStreamDestroy(ctx->own_stream);
    }
    delete ctx;
    return RBF_OK;
}

int rbf_ctx_set_timing(rbf_ctx *ctx, int32_t on) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    ctx->timing = on != 0;
    return RBF_OK;
}

int rbf_ctx_last_ms(rbf_ctx *ctx, float *ms) {
    if (!ctx || !ms) return RBF_ERR_ARGUMENT;
    *ms = ctx->last_ms;
    return RBF_OK;
}

int rbf_ctx_set_stream(rbf_ctx *ctx, void *s) {
    if (!ctx) return RBF_ERR_ARGUMENT;
    ctx->stream = s ? static_cast<cudaStream_t>(s) : ctx->own_stream;
    return RBF_OK;
}

const char *rbf_last_error(const rbf_ctx *ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int rbf_knn(rbf_ctx *ctx, const double *data, int64_t ns, const double *eval, int64_t ne, int32_t dim, int32_t k,
            int32_t *idx_out) {
    RBF_TRY(check_ctx(ctx));
    if (dim < 1 || dim > 3) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "dim must be 1, 2 or 3 (got %d)", dim);
    if (k < 1 || k > 64) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "k must be in 1..64 (got %d)", k);
    if (ns < 1 || ns >= INT32_MAX || ne < 0 || ne >= INT32_MAX)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "point counts must be in [1, 2^31)");
    if (k > ns) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "k = %d exceeds the number of data points (%lld)", k, (long long)ns);
    if (!data || (!eval && ne > 0) || (!idx_out && ne > 0)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null array");
    InArray d, q;
    OutArray o;
    RBF_TRY(d.bind(ctx, data, sizeof(double) * ns * dim));
    RBF_TRY(q.bind(ctx, eval, sizeof(double) * ne * dim));
    RBF_TRY(o.bind(ctx, idx_out, sizeof(int32_t) * ne * k));
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (ctx->timing) {
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, ctx->stream);
    }
    const int kst = rbf_knn_device(ctx, d.as<double>(), ns, q.as<double>(), ne, dim, k, o.as<int32_t>());
    if (ctx->timing) {
        cudaEventRecord(t1, ctx->stream);
        cudaEventSynchronize(t1);
        cudaEventElapsedTime(&ctx->last_ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    RBF_TRY(kst);
    RBF_TRY(o.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

int rbf_build_count(rbf_ctx *ctx, int64_t ns, int64_t ne, int32_t k, const rbf_hermite *herm,
                    int64_t *row_ptr_out, int64_t *nnz_out) {
    RBF_TRY(check_ctx(ctx));
    if (k < 1 || ne < 0 || ns < 1) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid sizes");
    if (herm && herm->is_boundary && ne > ns)
        return rbf_fail(ctx, RBF_ERR_DIMENSION, "Hermite builds evaluate at the data points (ne <= ns)");
    BoundaryDev b;
    RBF_TRY(bind_boundary(ctx, herm, ns, 1, b));
    OutArray rp;
    RBF_TRY(rp.bind(ctx, row_ptr_out, sizeof(int64_t) * (ne + 1)));
    int64_t nnz = 0;
    RBF_TRY(rbf_count_rows_device(ctx, ne, k, b.any ? b.isb.as<uint8_t>() : nullptr, b.any ? b.g2b.as<int32_t>() : nullptr,
                                  b.any ? b.alpha.as<double>() : nullptr, b.any ? b.beta.as<double>() : nullptr,
                                  rp.as<int64_t>(), &nnz));
    RBF_TRY(rp.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nnz_out) *nnz_out = nnz;
    return RBF_OK;
}

int rbf_build(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns, const double *eval,
              int64_t ne, const int32_t *adjl, int32_t k, const rbf_hermite *herm, const int64_t *row_ptr,
              int32_t *col, double *val, int8_t *status_out, rbf_build_stats *stats) {
    RBF_TRY(check_ctx(ctx));
    if (!cfg) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null configuration");
    if (cfg->flags & RBF_FLAG_NORMAL_DOF)
        return rbf_fail(ctx, RBF_ERR_UNSUPPORTED, "normal-derivative unknowns are built by rbf_build_batched");
    const int dim = cfg->dim;
    if (dim < 1 || dim > 3) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "dim must be 1, 2 or 3 (got %d)", dim);
    if (!(cfg->phs == 1 || cfg->phs == 3 || cfg->phs == 5 || cfg->phs == 7))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "n must be 1, 3, 5, or 7 (got n=%d)", cfg->phs);
    if (cfg->poly_deg < -1)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "poly_deg must be >= -1 (got %d)", cfg->poly_deg);
    if (cfg->nops < 1 || cfg->nops > RBF_MAX_OPS)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "nops must be in 1..%d", RBF_MAX_OPS);
    if (k < 1 || k > RBF_MAX_STENCIL) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "k must be in 1..%d", RBF_MAX_STENCIL);
    if (k > ns) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "k exceeds the number of data points");
    if (ns >= INT32_MAX || ne >= INT32_MAX || ne < 0) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "point counts must be < 2^31");
    StencilParams P;
    memset(&P, 0, sizeof P);
    P.nmon = monomial_exponents(dim, cfg->poly_deg, P.exps);
    if (k + P.nmon > RBF_MAX_SYSTEM)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "k + number of monomials (%d) exceeds %d", k + P.nmon, RBF_MAX_SYSTEM);
    RBF_TRY(set_operators(ctx, cfg, P));
    if (herm && herm->is_boundary && ne > ns)
        return rbf_fail(ctx, RBF_ERR_DIMENSION, "Hermite builds evaluate at the data points (ne <= ns)");
    BoundaryDev b;
    RBF_TRY(bind_boundary(ctx, herm, ns, dim, b));
    if (b.any_nr)
        for (int r = 0; r < cfg->nops; r++)
            if (P.op_code[r] == RBF_OP_IDENTITY)  // _check_normal_form_support, src/solve/api.jl:79-94
                return rbf_fail(ctx, RBF_ERR_UNSUPPORTED,
                                "Neumann/Robin boundary conditions require the operator's basis action to support "
                                "the normal-derivative form; the identity (regrid) has none");
    InArray d, q, a, rp;
    RBF_TRY(d.bind(ctx, data, sizeof(double) * ns * dim));
    RBF_TRY(q.bind(ctx, eval, sizeof(double) * ne * dim));
    RBF_TRY(a.bind(ctx, adjl, sizeof(int32_t) * ne * k));
    RBF_TRY(rp.bind(ctx, row_ptr, sizeof(int64_t) * (ne + 1)));
    bool idx_ok = true;
    RBF_TRY(rbf_check_indices(ctx, a.as<int32_t>(), ne * (int64_t)k, (int32_t)ns, &idx_ok));
    if (!idx_ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "adjl holds indices outside [0, %lld)", (long long)ns);
    int64_t nnz = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&nnz, rp.as<int64_t>() + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nnz < 0 || nnz > ne * (int64_t)k) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "row_ptr is not the layout of this build");
    OutArray oc, ov, os;
    RBF_TRY(oc.bind(ctx, col, sizeof(int32_t) * nnz));
    RBF_TRY(ov.bind(ctx, val, sizeof(double) * nnz * cfg->nops));
    RBF_TRY(os.bind(ctx, status_out, (size_t)ne));
    DevBuf counters;
    RBF_TRY(counters.alloc(ctx, sizeof(unsigned long long) * 8 + sizeof(double)));
    RBF_CUDA(ctx, cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long) * 8 + sizeof(double), ctx->stream));

    P.dim = dim;
    P.phs = cfg->phs;
    P.poly_deg = cfg->poly_deg;
    P.k = k;
    P.n = k + P.nmon;
    P.nops = cfg->nops;
    P.ne = ne;
    P.ns = ns;
    P.nnz = nnz;
    P.data = d.as<double>();
    P.eval = q.as<double>();
    P.adjl = a.as<int32_t>();
    P.isb = b.any ? b.isb.as<uint8_t>() : nullptr;
    P.g2b = b.any ? b.g2b.as<int32_t>() : nullptr;
    P.alpha = b.any ? b.alpha.as<double>() : nullptr;
    P.beta = b.any ? b.beta.as<double>() : nullptr;
    P.normals = b.any ? b.normals.as<double>() : nullptr;
    P.row_ptr = rp.as<int64_t>();
    P.col = oc.as<int32_t>();
    P.val = ov.as<double>();
    P.status = os.as<int8_t>();
    P.counters = counters.as<unsigned long long>();
    P.max_resid = reinterpret_cast<double *>(counters.as<unsigned long long>() + 8);
    P.refine_steps = cfg->refine_steps > 0 ? cfg->refine_steps : 6;
    P.tol = cfg->tol > 0 ? cfg->tol : 1e-9;
    P.flags = cfg->flags;
    P.seed = cfg->seed;
    if (cfg->sell_col || cfg->sell_val || cfg->sell_slice_off) {
        if (!cfg->sell_col || !cfg->sell_val || !cfg->sell_slice_off || !rbf_is_device_ptr(cfg->sell_col) ||
            !rbf_is_device_ptr(cfg->sell_val) || !rbf_is_device_ptr(cfg->sell_slice_off))
            return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the sliced copy needs device pointers for offsets, columns and values");
        if (cfg->sell_nnz < nnz) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "sell_nnz is below the CSR entry count");
        if (cfg->sell_nnz > nnz) {  // uneven rows: padding entries are column 0, value 0
            RBF_CUDA(ctx, cudaMemsetAsync(cfg->sell_col, 0, sizeof(int32_t) * cfg->sell_nnz, ctx->stream));
            RBF_CUDA(ctx, cudaMemsetAsync(cfg->sell_val, 0, sizeof(double) * cfg->sell_nnz * cfg->nops, ctx->stream));
        }
        P.sell_off = cfg->sell_slice_off;
        P.sell_col = cfg->sell_col;
        P.sell_val = cfg->sell_val;
        P.sell_nnz = cfg->sell_nnz;
    }
    DevBuf defer;
    if (cfg->precision != RBF_PREC_FP64) {
        RBF_TRY(defer.alloc(ctx, sizeof(int32_t) * (size_t)ne));
        P.defer = defer.as<int32_t>();
    }
    if (cfg->precision == RBF_PREC_LEARNED) {
        if (!cfg->seed || !rbf_is_device_ptr(cfg->seed))
            return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the learned build needs a device pointer to the predicted weights");
        if (cfg->nops != 1) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the learned build predicts one operator");
    } else {
        P.seed = nullptr;
    }

    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    cudaEventRecord(ev0, ctx->stream);
    int st;
    if (cfg->precision == RBF_PREC_FP64)
        st = rbf_build_fp64_launch(ctx, P);
    else if (cfg->precision == RBF_PREC_FP32_REFINED || cfg->precision == RBF_PREC_LEARNED)
        st = rbf_build_fp32_launch(ctx, P);
    else
        st = rbf_fail(ctx, RBF_ERR_ARGUMENT, "unknown precision mode %d", cfg->precision);
    cudaEventRecord(ev1, ctx->stream);
    if (st != RBF_OK) {
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        return st;
    }
    unsigned long long hc[8];
    double hres = 0.0;
    RBF_CUDA(ctx, cudaMemcpyAsync(hc, counters.ptr, sizeof hc, cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaMemcpyAsync(&hres, P.max_resid, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_TRY(oc.finish(ctx));
    RBF_TRY(ov.finish(ctx));
    RBF_TRY(os.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    if (stats) {
        stats->n_identity_rows = (int64_t)hc[3];
        stats->n_stencils = ne - (int64_t)hc[3];
        stats->n_singular = (int64_t)hc[0];
        stats->n_fallback = (int64_t)hc[2];
        stats->max_residual = hres;
        stats->ms_build = ms;
        stats->ms_knn = 0.f;
        stats->ms_total = ms;
        stats->n_residuals = (int64_t)hc[4];
        stats->seed_rel_err_mean = hc[6] ? (double)hc[5] * 1e-6 / (double)hc[6] : 0.0;
    }
    if (hc[1]) return rbf_fail(ctx, RBF_ERR_NOT_FOUND, "evaluation point not found in stencil data (%llu stencils)", hc[1]);
    if (hc[0]) return rbf_fail(ctx, RBF_ERR_SINGULAR, "%llu stencil system(s) are singular", hc[0]);
    return RBF_OK;
}

int rbf_csr_free(rbf_ctx *ctx, rbf_csr *csr) {
    RBF_TRY(check_ctx(ctx));
    if (!csr) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null csr");
    RBF_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaError_t e = cudaSuccess;
    for (void *p : {(void *)csr->row_ptr, (void *)csr->col, (void *)csr->val})
        if (p) {
            const cudaError_t f = cudaFree(p);
            if (e == cudaSuccess) e = f;
        }
    *csr = rbf_csr{};
    if (e != cudaSuccess) return rbf_fail(ctx, RBF_ERR_CUDA, "cudaFree: %s", cudaGetErrorString(e));
    return RBF_OK;
}

int rbf_build_csr(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns, const double *eval,
                  int64_t ne, const int32_t *adjl, int32_t k, const rbf_hermite *herm, int8_t *status_out,
                  rbf_build_stats *stats, rbf_csr *out) {
    RBF_TRY(check_ctx(ctx));
    if (!cfg || !out) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null configuration or output");
    *out = rbf_csr{};
    if (cfg->nops < 1 || cfg->nops > RBF_MAX_OPS)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "nops must be in 1..%d (got %d)", RBF_MAX_OPS, cfg->nops);
    if (ne < 0) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid sizes");
    RBF_CUDA(ctx, cudaSetDevice(ctx->device));
    rbf_csr c{};
    c.ne = ne;
    c.ns = ns;
    c.nops = cfg->nops;
    int st = RBF_OK;
    // a failed allocation's error is cleared (cudaGetLastError), so that the next launch check
    // does not report it as its own
    if (cudaMalloc(&c.row_ptr, sizeof(int64_t) * (size_t)(ne + 1)) != cudaSuccess) {
        c.row_ptr = nullptr;
        cudaGetLastError();
        st = rbf_fail(ctx, RBF_ERR_CUDA, "cudaMalloc of %lld row offsets failed", (long long)(ne + 1));
    }
    if (st == RBF_OK) st = rbf_build_count(ctx, ns, ne, k, herm, c.row_ptr, &c.nnz);
    if (st == RBF_OK) {
        const size_t nz = c.nnz > 0 ? (size_t)c.nnz : 1;
        if (cudaMalloc(&c.col, sizeof(int32_t) * nz) != cudaSuccess) c.col = nullptr;
        if (cudaMalloc(&c.val, sizeof(double) * nz * (size_t)cfg->nops) != cudaSuccess) c.val = nullptr;
        if (!c.col || !c.val) {
            cudaGetLastError();
            st = rbf_fail(ctx, RBF_ERR_CUDA, "cudaMalloc of %lld entries x %d operators failed", (long long)c.nnz,
                          cfg->nops);
        }
    }
    if (st == RBF_OK) st = rbf_build(ctx, cfg, data, ns, eval, ne, adjl, k, herm, c.row_ptr, c.col, c.val, status_out, stats);
    if (st != RBF_OK) {
        const std::string msg = ctx->last_error;  // the build's error, not the free's
        rbf_csr_free(ctx, &c);
        ctx->last_error = msg;
        return st;
    }
    *out = c;
    return RBF_OK;
}

int rbf_spmm(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *row_ptr, const int32_t *col, const double *val,
             int32_t nf, int32_t layout, const double *X, int64_t ldx, double alpha, double beta, double *Y,
             int64_t ldy) {
    RBF_TRY(check_ctx(ctx));
    if (nf < 1 || ne < 0 || ns < 0) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid sizes");
    if (layout != 0 && layout != 1) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "layout must be 0 or 1");
    if (layout == 0 && nf > 1 && (ldx < ns || ldy < ne)) return rbf_fail(ctx, RBF_ERR_DIMENSION, "leading dimension too small");
    if (layout == 1 && (ldx < nf || ldy < nf)) return rbf_fail(ctx, RBF_ERR_DIMENSION, "leading dimension too small");
    InArray rp, c, v, x;
    RBF_TRY(rp.bind(ctx, row_ptr, sizeof(int64_t) * (ne + 1)));
    if (rbf_is_device_ptr(col) && rbf_is_device_ptr(val)) {  // no staging: nnz not needed
        c.dptr = col;
        v.dptr = val;
    } else {
        int64_t nnz = 0;
        RBF_CUDA(ctx, cudaMemcpyAsync(&nnz, rp.as<int64_t>() + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
        RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        RBF_TRY(c.bind(ctx, col, sizeof(int32_t) * nnz));
        RBF_TRY(v.bind(ctx, val, sizeof(double) * nnz));
    }
    size_t xbytes = sizeof(double) * (size_t)(layout == 0 ? (nf > 1 ? ldx * (nf - 1) + ns : ns) : ns * ldx);
    size_t ybytes = sizeof(double) * (size_t)(layout == 0 ? (nf > 1 ? ldy * (nf - 1) + ne : ne) : ne * ldy);
    RBF_TRY(x.bind(ctx, X, xbytes));
    OutArray y;
    RBF_TRY(y.bind(ctx, Y, ybytes));
    if (y.host && beta != 0.0) RBF_CUDA(ctx, cudaMemcpyAsync(y.dptr, Y, ybytes, cudaMemcpyHostToDevice, ctx->stream));
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (ctx->timing) {
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, ctx->stream);
    }
    const int sst = rbf_spmm_device(ctx, ne, ns, rp.as<int64_t>(), c.as<int32_t>(), v.as<double>(), nf, layout,
                                    x.as<double>(), nf == 1 ? 1 : ldx, alpha, beta, y.as<double>(), nf == 1 ? 1 : ldy);
    if (ctx->timing) {
        cudaEventRecord(t1, ctx->stream);
        cudaEventSynchronize(t1);
        cudaEventElapsedTime(&ctx->last_ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    RBF_TRY(sst);
    RBF_TRY(y.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

int rbf_csr_to_csc(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *row_ptr, const int32_t *col,
                   const double *val, int64_t *col_ptr_out, int32_t *row_out, double *val_out) {
    RBF_TRY(check_ctx(ctx));
    InArray rp, c, v;
    RBF_TRY(rp.bind(ctx, row_ptr, sizeof(int64_t) * (ne + 1)));
    int64_t nnz = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&nnz, rp.as<int64_t>() + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    RBF_TRY(c.bind(ctx, col, sizeof(int32_t) * nnz));
    RBF_TRY(v.bind(ctx, val, sizeof(double) * nnz));
    OutArray cp, ro, vo;
    RBF_TRY(cp.bind(ctx, col_ptr_out, sizeof(int64_t) * (ns + 1)));
    RBF_TRY(ro.bind(ctx, row_out, sizeof(int32_t) * nnz));
    RBF_TRY(vo.bind(ctx, val_out, sizeof(double) * nnz));
    RBF_TRY(rbf_csr_to_csc_device(ctx, ne, ns, rp.as<int64_t>(), c.as<int32_t>(), v.as<double>(), cp.as<int64_t>(),
                                  ro.as<int32_t>(), vo.as<double>()));
    RBF_TRY(cp.finish(ctx));
    RBF_TRY(ro.finish(ctx));
    RBF_TRY(vo.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

int rbf_build_backward(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns, const double *eval,
                       int64_t ne, const int32_t *adjl, int32_t k, const int64_t *row_ptr, const double *dW,
                       double *ddata, double *deval) {
    RBF_TRY(check_ctx(ctx));
    if (!cfg) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null configuration");
    if (k < 1 || k > RBF_MAX_STENCIL) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "k must be in 1..%d", RBF_MAX_STENCIL);
    if (k > ns) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "k exceeds the number of data points");
    if (ns >= INT32_MAX || ne >= INT32_MAX || ne < 0) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "point counts must be < 2^31");
    if (!data || !adjl || !row_ptr || !dW || !ddata || (ne > 0 && !deval))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null array");
    StencilParams P;
    memset(&P, 0, sizeof P);
    P.k = k;
    RBF_TRY(rbf_plan_params(ctx, cfg, P));
    for (int r = 0; r < P.nops; r++)
        if (P.op_code[r] == RBF_OP_PARTIAL2)
            return rbf_fail(ctx, RBF_ERR_UNSUPPORTED, "the weight adjoint supports the identity, first partials and "
                                                      "the Laplacian");
    const int dim = P.dim;
    if (!eval) {
        eval = data;
        if (ne != ns) return rbf_fail(ctx, RBF_ERR_DIMENSION, "without eval points ne must equal ns");
    }
    InArray d, q, a, rp, gw;
    RBF_TRY(d.bind(ctx, data, sizeof(double) * ns * dim));
    RBF_TRY(q.bind(ctx, eval, sizeof(double) * ne * dim));
    RBF_TRY(a.bind(ctx, adjl, sizeof(int32_t) * ne * k));
    RBF_TRY(rp.bind(ctx, row_ptr, sizeof(int64_t) * (ne + 1)));
    bool idx_ok = true;
    RBF_TRY(rbf_check_indices(ctx, a.as<int32_t>(), ne * (int64_t)k, (int32_t)ns, &idx_ok));
    if (!idx_ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "adjl holds indices outside [0, %lld)", (long long)ns);
    int64_t nnz = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&nnz, rp.as<int64_t>() + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nnz != ne * (int64_t)k)
        return rbf_fail(ctx, RBF_ERR_UNSUPPORTED, "the weight adjoint takes interior builds (k entries per row)");
    RBF_TRY(gw.bind(ctx, dW, sizeof(double) * nnz * P.nops));
    OutArray od, oe;
    RBF_TRY(od.bind(ctx, ddata, sizeof(double) * ns * dim));
    RBF_TRY(oe.bind(ctx, deval, sizeof(double) * ne * dim));
    RBF_CUDA(ctx, cudaMemsetAsync(od.as<double>(), 0, sizeof(double) * ns * dim, ctx->stream));
    if (ne > 0) RBF_CUDA(ctx, cudaMemsetAsync(oe.as<double>(), 0, sizeof(double) * ne * dim, ctx->stream));
    DevBuf counters;
    RBF_TRY(counters.alloc(ctx, sizeof(unsigned long long) * 8 + sizeof(double)));
    RBF_CUDA(ctx, cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long) * 8 + sizeof(double), ctx->stream));
    P.ne = ne;
    P.ns = ns;
    P.nnz = nnz;
    P.data = d.as<double>();
    P.eval = q.as<double>();
    P.adjl = a.as<int32_t>();
    P.row_ptr = rp.as<int64_t>();
    P.counters = counters.as<unsigned long long>();
    P.max_resid = reinterpret_cast<double *>(counters.as<unsigned long long>() + 8);
    // the adjoint's refinement aims below the forward's default tolerance: the gradients
    // combine the weights and the adjoint, and are checked against FP64 to 1e-9
    P.tol = cfg->tol > 0 ? cfg->tol : 1e-11;
    RBF_TRY(rbf_backward_launch(ctx, P, cfg->precision != RBF_PREC_FP64, gw.as<double>(), od.as<double>(),
                                oe.as<double>()));
    unsigned long long nsing = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&nsing, counters.ptr, sizeof nsing, cudaMemcpyDeviceToHost, ctx->stream));
    RBF_TRY(od.finish(ctx));
    RBF_TRY(oe.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nsing) return rbf_fail(ctx, RBF_ERR_SINGULAR, "%llu stencil system(s) are singular", nsing);
    return RBF_OK;
}

int rbf_sytrf_rook(rbf_ctx *ctx, int64_t n, double *A, int64_t lda, int32_t *ipiv, int64_t *info) {
    RBF_TRY(check_ctx(ctx));
    if (n < 0 || n >= INT32_MAX || lda < std::max<int64_t>(1, n)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "bad n / lda");
    if ((n > 0 && (!A || !ipiv)) || !info) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null array");
    *info = 0;
    if (n == 0) return RBF_OK;
    const size_t abytes = sizeof(double) * (size_t)lda * (size_t)n;
    OutArray ao, po;
    RBF_TRY(ao.bind(ctx, A, abytes));
    if (ao.host) RBF_CUDA(ctx, cudaMemcpyAsync(ao.dptr, A, abytes, cudaMemcpyHostToDevice, ctx->stream));
    RBF_TRY(po.bind(ctx, ipiv, sizeof(int32_t) * n));
    DevBuf perm;
    RBF_TRY(perm.alloc(ctx, sizeof(int32_t) * n));
    RBF_TRY(rbf_sytrf_rook_device(ctx, (int)n, ao.as<double>(), lda, po.as<int32_t>(), perm.as<int32_t>(), info));
    RBF_TRY(ao.finish(ctx));
    RBF_TRY(po.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

int rbf_sytrs_rook(rbf_ctx *ctx, int64_t n, int32_t nrhs, const double *A, int64_t lda, const int32_t *ipiv,
                   double *B, int64_t ldb) {
    RBF_TRY(check_ctx(ctx));
    if (n < 0 || n >= INT32_MAX || nrhs < 0 || lda < std::max<int64_t>(1, n) || ldb < std::max<int64_t>(1, n))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "bad n / nrhs / lda / ldb");
    if (n == 0 || nrhs == 0) return RBF_OK;
    if (!A || !ipiv || !B) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null array");
    const size_t bbytes = sizeof(double) * (size_t)ldb * (size_t)nrhs;
    InArray ai, pi;
    OutArray bo;
    RBF_TRY(ai.bind(ctx, A, sizeof(double) * (size_t)lda * (size_t)n));
    RBF_TRY(pi.bind(ctx, ipiv, sizeof(int32_t) * n));
    RBF_TRY(bo.bind(ctx, B, bbytes));
    bool ok = true;
    RBF_TRY(rbf_check_ipiv_device(ctx, (int)n, pi.as<int32_t>(), &ok));
    if (!ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "ipiv holds entries outside +-[1, n]");
    if (bo.host) RBF_CUDA(ctx, cudaMemcpyAsync(bo.dptr, B, bbytes, cudaMemcpyHostToDevice, ctx->stream));
    DevBuf tmp;
    RBF_TRY(tmp.alloc(ctx, sizeof(double) * n));
    for (int r = 0; r < nrhs; r++) {
        double *col = bo.as<double>() + (size_t)r * ldb;
        RBF_TRY(rbf_sytrs_rook_device(ctx, (int)n, ai.as<double>(), lda, pi.as<int32_t>(), nullptr, col,
                                      tmp.as<double>()));
        RBF_CUDA(ctx, cudaMemcpyAsync(col, tmp.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    RBF_TRY(bo.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

}  // extern "C"

namespace {
int interp_args(rbf_ctx *ctx, int32_t dim, int32_t phs, int32_t poly_deg, int64_t n, int8_t (*ex)[3], int *nmon) {
    if (dim < 1 || dim > 3) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "dim must be 1, 2 or 3 (got %d)", dim);
    if (!(phs == 1 || phs == 3 || phs == 5 || phs == 7))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "n must be 1, 3, 5, or 7 (got n=%d)", phs);
    if (poly_deg < -1) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "poly_deg must be >= -1 (got %d)", poly_deg);
    if (poly_deg >= 0 && binom(dim + poly_deg, dim) > RBF_MAX_SYSTEM)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "more than %d monomials", RBF_MAX_SYSTEM);
    *nmon = monomial_exponents(dim, poly_deg, ex);
    if (n < 1 || n + *nmon >= 2000000000LL) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "bad number of points");
    return RBF_OK;
}
}  // namespace

extern "C" {

int rbf_interp_fit(rbf_ctx *ctx, int32_t dim, int32_t phs, int32_t poly_deg, const double *x, int64_t n,
                   const double *y, double *coef) {
    RBF_TRY(check_ctx(ctx));
    int8_t ex[RBF_MAX_SYSTEM][3];
    int nmon = 0;
    RBF_TRY(interp_args(ctx, dim, phs, poly_deg, n, ex, &nmon));
    if (!x || !y || !coef) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null array");
    const int64_t nt = n + nmon;
    const size_t abytes = sizeof(double) * (size_t)nt * (size_t)nt;
    size_t free_b = 0, total_b = 0;
    RBF_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
    if (abytes + (size_t)nt * 64 > free_b / 10 * 9)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the %lld x %lld collocation matrix (%.1f GB) does not fit in device memory",
                        (long long)nt, (long long)nt, abytes / 1e9);
    InArray xi, yi;
    OutArray co;
    RBF_TRY(xi.bind(ctx, x, sizeof(double) * n * dim));
    RBF_TRY(yi.bind(ctx, y, sizeof(double) * n));
    RBF_TRY(co.bind(ctx, coef, sizeof(double) * nt));
    DevBuf A, piv, perm, rhs;
    RBF_TRY(A.alloc(ctx, abytes));
    RBF_TRY(piv.alloc(ctx, sizeof(int32_t) * nt));
    RBF_TRY(perm.alloc(ctx, sizeof(int32_t) * nt));
    RBF_TRY(rhs.alloc(ctx, sizeof(double) * nt));
    RBF_TRY(rbf_interp_assemble_device(ctx, dim, phs, nmon, ex, xi.as<double>(), (int)n, A.as<double>(), nt));
    int64_t info = 0;
    RBF_TRY(rbf_sytrf_rook_device(ctx, (int)nt, A.as<double>(), nt, piv.as<int32_t>(), perm.as<int32_t>(), &info));
    if (info) return rbf_fail(ctx, RBF_ERR_SINGULAR, "the collocation matrix is singular (D(%lld,%lld) = 0)",
                              (long long)info, (long long)info);
    RBF_CUDA(ctx, cudaMemcpyAsync(rhs.ptr, yi.dptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    if (nmon) RBF_CUDA(ctx, cudaMemsetAsync(rhs.as<double>() + n, 0, sizeof(double) * nmon, ctx->stream));
    RBF_TRY(rbf_sytrs_rook_device(ctx, (int)nt, A.as<double>(), nt, piv.as<int32_t>(), perm.as<int32_t>(),
                                  rhs.as<double>(), co.as<double>()));
    RBF_TRY(co.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

int rbf_interp_eval(rbf_ctx *ctx, int32_t dim, int32_t phs, int32_t poly_deg, const double *x, int64_t n,
                    const double *coef, const double *xe, int64_t m, double *out) {
    RBF_TRY(check_ctx(ctx));
    int8_t ex[RBF_MAX_SYSTEM][3];
    int nmon = 0;
    RBF_TRY(interp_args(ctx, dim, phs, poly_deg, n, ex, &nmon));
    if (m < 0) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "m must be >= 0");
    if (m == 0) return RBF_OK;
    if (!x || !coef || !xe || !out) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null array");
    InArray xi, ci, ei;
    OutArray oo;
    RBF_TRY(xi.bind(ctx, x, sizeof(double) * n * dim));
    RBF_TRY(ci.bind(ctx, coef, sizeof(double) * (n + nmon)));
    RBF_TRY(ei.bind(ctx, xe, sizeof(double) * m * dim));
    RBF_TRY(oo.bind(ctx, out, sizeof(double) * m));
    RBF_TRY(rbf_interp_eval_device(ctx, dim, phs, nmon, ex, xi.as<double>(), (int)n, ci.as<double>(), ei.as<double>(), m,
                                   oo.as<double>()));
    RBF_TRY(oo.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

int rbf_weights_axpby(rbf_ctx *ctx, int64_t nnz, double alpha, const double *a, double beta, const double *b,
                      double *out) {
    RBF_TRY(check_ctx(ctx));
    if (nnz < 0) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid entry count");
    if (!rbf_is_device_ptr(a) || !rbf_is_device_ptr(out) || (b && !rbf_is_device_ptr(b)))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "operator algebra takes device pointers only");
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (ctx->timing) {
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, ctx->stream);
    }
    const int st = rbf_weights_axpby_device(ctx, nnz, alpha, a, beta, b, out);
    if (ctx->timing) {
        cudaEventRecord(t1, ctx->stream);
        cudaEventSynchronize(t1);
        cudaEventElapsedTime(&ctx->last_ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    return st;
}

int rbf_weights_directional(rbf_ctx *ctx, int64_t ne, const int64_t *row_ptr, int32_t nd, const double *val,
                            int64_t nnz, const double *v, int32_t per_row, double *out) {
    RBF_TRY(check_ctx(ctx));
    if (ne < 0 || nnz < 0 || nd < 1 || nd > RBF_MAX_OPS) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid sizes");
    const void *ptrs[] = {row_ptr, val, v, out};
    for (const void *p : ptrs)
        if (!rbf_is_device_ptr(p)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "operator algebra takes device pointers only");
    return rbf_weights_directional_device(ctx, ne, row_ptr, nd, val, nnz, v, per_row != 0, out);
}

int rbf_sell_offsets(rbf_ctx *ctx, int64_t ne, const int64_t *row_ptr, int64_t *slice_off, int64_t *sell_nnz) {
    RBF_TRY(check_ctx(ctx));
    if (ne < 0 || ne >= INT32_MAX) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid row count");
    if (!rbf_is_device_ptr(row_ptr) || !rbf_is_device_ptr(slice_off))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the sliced layout takes device pointers only");
    int64_t total = 0;
    RBF_TRY(rbf_sell_offsets_device(ctx, ne, row_ptr, slice_off, &total));
    if (sell_nnz) *sell_nnz = total;
    return RBF_OK;
}

int rbf_sell_from_csr(rbf_ctx *ctx, int64_t ne, const int64_t *row_ptr, const int32_t *col, const double *val,
                      const int64_t *slice_off, int32_t *sell_col, double *sell_val) {
    RBF_TRY(check_ctx(ctx));
    if (ne < 0 || ne >= INT32_MAX) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid row count");
    const void *ptrs[] = {row_ptr, col, val, slice_off, sell_col, sell_val};
    for (const void *p : ptrs)
        if (!rbf_is_device_ptr(p)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the sliced layout takes device pointers only");
    return rbf_sell_fill_device(ctx, ne, row_ptr, col, val, slice_off, sell_col, sell_val);
}

int rbf_spmv_sell(rbf_ctx *ctx, int64_t ne, const int64_t *slice_off, const int32_t *sell_col,
                  const double *sell_val, const double *x, double alpha, double beta, double *y) {
    RBF_TRY(check_ctx(ctx));
    if (ne < 0 || ne >= INT32_MAX) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid row count");
    const void *ptrs[] = {slice_off, sell_col, sell_val, x, y};
    for (const void *p : ptrs)
        if (!rbf_is_device_ptr(p)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the sliced apply takes device pointers only");
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (ctx->timing) {
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, ctx->stream);
    }
    const int st = rbf_spmv_sell_device(ctx, ne, slice_off, sell_col, sell_val, x, alpha, beta, y);
    if (ctx->timing) {
        cudaEventRecord(t1, ctx->stream);
        cudaEventSynchronize(t1);
        cudaEventElapsedTime(&ctx->last_ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    return st;
}

int rbf_sell_offsets_perm(rbf_ctx *ctx, int64_t ne, const int64_t *row_ptr, const int32_t *row_at, int64_t *slice_off,
                          int64_t *sell_nnz) {
    RBF_TRY(check_ctx(ctx));
    if (ne < 0 || ne >= INT32_MAX) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid row count");
    if (!sell_nnz) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null sell_nnz");
    const void *ptrs[] = {row_ptr, row_at, slice_off};
    for (const void *p : ptrs)
        if (!rbf_is_device_ptr(p)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the sliced layout takes device pointers only");
    bool ok = true;
    RBF_TRY(rbf_check_indices(ctx, row_at, ne, (int32_t)ne, &ok));
    if (!ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "row_at holds a row index outside [0, ne)");
    RBF_TRY(rbf_sell_offsets_perm_device(ctx, ne, row_ptr, row_at, slice_off, sell_nnz));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

int rbf_sell_from_csr_perm(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *row_ptr, const int32_t *col,
                           const double *val, const int32_t *row_at, const int32_t *col_at, const int64_t *slice_off,
                           int32_t *sell_col, double *sell_val) {
    RBF_TRY(check_ctx(ctx));
    if (ne < 0 || ne >= INT32_MAX || ns < 0 || ns >= INT32_MAX)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid row or column count");
    const void *ptrs[] = {row_ptr, col, val, row_at, col_at, slice_off, sell_col, sell_val};
    for (const void *p : ptrs)
        if (!rbf_is_device_ptr(p)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the sliced layout takes device pointers only");
    bool ok = true;
    RBF_TRY(rbf_check_indices(ctx, row_at, ne, (int32_t)ne, &ok));
    if (!ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "row_at holds a row index outside [0, ne)");
    RBF_TRY(rbf_check_indices(ctx, col_at, ns, (int32_t)ns, &ok));
    if (!ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "col_at holds a column index outside [0, ns)");
    RBF_TRY(rbf_sell_fill_perm_device(ctx, ne, ns, row_ptr, col, val, row_at, col_at, slice_off, sell_col, sell_val));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RBF_OK;
}

int rbf_spmv_sell_perm(rbf_ctx *ctx, int64_t ne, int64_t ns, const int64_t *slice_off, const int32_t *sell_col,
                       const double *sell_val, const int32_t *row_at, const int32_t *col_at, const double *x,
                       double *x_work, double alpha, double beta, double *y) {
    RBF_TRY(check_ctx(ctx));
    if (ne < 0 || ne >= INT32_MAX || ns < 0 || ns >= INT32_MAX)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid row or column count");
    const void *ptrs[] = {slice_off, sell_col, sell_val, row_at, col_at, x, x_work, y};
    for (const void *p : ptrs)
        if (!rbf_is_device_ptr(p)) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "the sliced apply takes device pointers only");
    if (x_work == x) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "x_work must not alias x");
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (ctx->timing) {
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, ctx->stream);
    }
    const int st = rbf_spmv_sell_perm_device(ctx, ne, ns, slice_off, sell_col, sell_val, row_at, col_at, x, x_work,
                                             alpha, beta, y);
    if (ctx->timing) {
        cudaEventRecord(t1, ctx->stream);
        cudaEventSynchronize(t1);
        cudaEventElapsedTime(&ctx->last_ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    return st;
}

int rbf_build_count_ragged(rbf_ctx *ctx, int64_t ns, int64_t ne, const int64_t *adj_ptr, const rbf_hermite *herm,
                           int64_t *row_ptr_out, int64_t *nnz_out) {
    RBF_TRY(check_ctx(ctx));
    if (ne < 0 || ns < 1 || !adj_ptr) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid sizes or null adjacency");
    if (herm && herm->is_boundary && ne > ns)
        return rbf_fail(ctx, RBF_ERR_DIMENSION, "Hermite builds evaluate at the data points (ne <= ns)");
    BoundaryDev b;
    RBF_TRY(bind_boundary(ctx, herm, ns, 1, b));
    InArray ap;
    RBF_TRY(ap.bind(ctx, adj_ptr, sizeof(int64_t) * (ne + 1)));
    OutArray rp;
    RBF_TRY(rp.bind(ctx, row_ptr_out, sizeof(int64_t) * (ne + 1)));
    int64_t nnz = 0;
    RBF_TRY(rbf_count_rows_device(ctx, ne, 0, b.any ? b.isb.as<uint8_t>() : nullptr, b.any ? b.g2b.as<int32_t>() : nullptr,
                                  b.any ? b.alpha.as<double>() : nullptr, b.any ? b.beta.as<double>() : nullptr,
                                  rp.as<int64_t>(), &nnz, ap.as<int64_t>()));
    RBF_TRY(rp.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nnz_out) *nnz_out = nnz;
    return RBF_OK;
}

int rbf_build_count_normal_dof(rbf_ctx *ctx, int64_t ns, int64_t ne, const int64_t *adj_ptr, const int32_t *adj_idx,
                               const rbf_hermite *herm, int64_t *row_ptr_out, int64_t *nnz_out) {
    RBF_TRY(check_ctx(ctx));
    if (ne < 0 || ns < 1 || !adj_ptr || !adj_idx)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "invalid sizes or null adjacency");
    if (herm && herm->is_boundary && ne > ns)
        return rbf_fail(ctx, RBF_ERR_DIMENSION, "Hermite builds evaluate at the data points (ne <= ns)");
    BoundaryDev b;
    RBF_TRY(bind_boundary(ctx, herm, ns, 1, b));
    InArray ap, ai;
    RBF_TRY(ap.bind(ctx, adj_ptr, sizeof(int64_t) * (ne + 1)));
    int64_t ends[2] = {0, 0};
    RBF_CUDA(ctx, cudaMemcpyAsync(&ends[0], ap.as<int64_t>(), sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaMemcpyAsync(&ends[1], ap.as<int64_t>() + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ends[0] != 0 || ends[1] < 0 || ends[1] > (int64_t)RBF_MAX_STENCIL * ne)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "adj_ptr must start at 0 and hold at most %d neighbours per stencil",
                        RBF_MAX_STENCIL);
    RBF_TRY(ai.bind(ctx, adj_idx, sizeof(int32_t) * ends[1]));
    bool idx_ok = true;
    RBF_TRY(rbf_check_indices(ctx, ai.as<int32_t>(), ends[1], (int32_t)ns, &idx_ok));
    if (!idx_ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "adj_idx holds indices outside [0, %lld)", (long long)ns);
    OutArray rp;
    RBF_TRY(rp.bind(ctx, row_ptr_out, sizeof(int64_t) * (ne + 1)));
    int64_t nnz = 0;
    RBF_TRY(rbf_count_rows_device(ctx, ne, 0, b.any ? b.isb.as<uint8_t>() : nullptr, b.any ? b.g2b.as<int32_t>() : nullptr,
                                  b.any ? b.alpha.as<double>() : nullptr, b.any ? b.beta.as<double>() : nullptr,
                                  rp.as<int64_t>(), &nnz, ap.as<int64_t>(), ai.as<int32_t>()));
    RBF_TRY(rp.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nnz_out) *nnz_out = nnz;
    return RBF_OK;
}

int rbf_build_batched(rbf_ctx *ctx, const rbf_build_cfg *cfg, const double *data, int64_t ns, const double *eval,
                      int64_t ne, const int64_t *adj_ptr, const int32_t *adj_idx, const int8_t *poly_deg_per,
                      const rbf_hermite *herm, const int64_t *row_ptr, int32_t *col, double *val, int8_t *status_out,
                      rbf_build_stats *stats, int32_t tune) {
    RBF_TRY(check_ctx(ctx));
    if (!cfg || !adj_ptr) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "null configuration or adjacency");
    const int dim = cfg->dim;
    if (dim < 1 || dim > 3) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "dim must be 1, 2 or 3 (got %d)", dim);
    if (!(cfg->phs == 1 || cfg->phs == 3 || cfg->phs == 5 || cfg->phs == 7))
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "n must be 1, 3, 5, or 7 (got n=%d)", cfg->phs);
    if (cfg->poly_deg < -1)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "poly_deg must be >= -1 (got %d)", cfg->poly_deg);
    if (cfg->nops < 1 || cfg->nops > RBF_MAX_OPS) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "nops must be in 1..%d", RBF_MAX_OPS);
    if (cfg->precision != RBF_PREC_FP64 && cfg->precision != RBF_PREC_FP32_REFINED)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "batched builds are plain FP64 or FP32-refined");
    if (ns < 1 || ns >= INT32_MAX || ne >= INT32_MAX || ne < 0) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "point counts must be < 2^31");
    if (tune < 0 || tune > 2) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "tune must be 0, 1 or 2");
    StencilParams P;
    memset(&P, 0, sizeof P);
    RBF_TRY(set_operators(ctx, cfg, P));
    if (herm && herm->is_boundary && ne > ns)
        return rbf_fail(ctx, RBF_ERR_DIMENSION, "Hermite builds evaluate at the data points (ne <= ns)");
    BoundaryDev b;
    RBF_TRY(bind_boundary(ctx, herm, ns, dim, b));
    if (b.any_nr)
        for (int r = 0; r < cfg->nops; r++)
            if (P.op_code[r] == RBF_OP_IDENTITY)  // _check_normal_form_support, src/solve/api.jl:79-94
                return rbf_fail(ctx, RBF_ERR_UNSUPPORTED,
                                "Neumann/Robin boundary conditions require the operator's basis action to support "
                                "the normal-derivative form; the identity (regrid) has none");
    InArray d, q, ap, ai, dg, rp;
    RBF_TRY(d.bind(ctx, data, sizeof(double) * ns * dim));
    RBF_TRY(q.bind(ctx, eval, sizeof(double) * ne * dim));
    RBF_TRY(ap.bind(ctx, adj_ptr, sizeof(int64_t) * (ne + 1)));
    int64_t ends[2] = {0, 0};
    RBF_CUDA(ctx, cudaMemcpyAsync(&ends[0], ap.as<int64_t>(), sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaMemcpyAsync(&ends[1], ap.as<int64_t>() + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ends[0] != 0 || ends[1] < 0 || ends[1] > (int64_t)RBF_MAX_STENCIL * ne)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "adj_ptr must start at 0 and hold at most %d neighbours per stencil",
                        RBF_MAX_STENCIL);
    RBF_TRY(ai.bind(ctx, adj_idx, sizeof(int32_t) * ends[1]));
    if (poly_deg_per) RBF_TRY(dg.bind(ctx, poly_deg_per, (size_t)ne));
    RBF_TRY(rp.bind(ctx, row_ptr, sizeof(int64_t) * (ne + 1)));
    bool idx_ok = true;
    RBF_TRY(rbf_check_indices(ctx, ai.as<int32_t>(), ends[1], (int32_t)ns, &idx_ok));
    if (!idx_ok) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "adj_idx holds indices outside [0, %lld)", (long long)ns);
    const bool normal_dof = (cfg->flags & RBF_FLAG_NORMAL_DOF) != 0;
    if (normal_dof && ns + b.nb >= INT32_MAX)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "data points + boundary points must be < 2^31");
    if (normal_dof && b.any_nr && cfg->phs == 1)
        return rbf_fail(ctx, RBF_ERR_UNSUPPORTED,
                        "normal-derivative unknowns need PHS 3, 5 or 7 (r has no normal derivative at r = 0)");
    // size classes (with normal-derivative unknowns: their number m is part of the class)
    StencilParams nd;
    memset(&nd, 0, sizeof nd);
    nd.adjl = ai.as<int32_t>();
    nd.isb = b.any ? b.isb.as<uint8_t>() : nullptr;
    nd.g2b = b.any ? b.g2b.as<int32_t>() : nullptr;
    nd.alpha = b.any ? b.alpha.as<double>() : nullptr;
    nd.beta = b.any ? b.beta.as<double>() : nullptr;
    DevBuf keys;
    RBF_TRY(keys.alloc(ctx, sizeof(int32_t) * (size_t)std::max<int64_t>(ne, 1)));
    std::vector<unsigned long long> hist;
    int err = 0;
    RBF_TRY(rbf_batched_classify(ctx, ne, dim, ap.as<int64_t>(), poly_deg_per ? dg.as<int8_t>() : nullptr,
                                 cfg->poly_deg, normal_dof ? &nd : nullptr, keys.as<int32_t>(), hist, &err));
    if (err & 8) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "adj_ptr must be non-decreasing");
    if (err & 1) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "stencil sizes must be in 1..%d", RBF_MAX_STENCIL);
    if (err & 4) return rbf_fail(ctx, RBF_ERR_ARGUMENT, "polynomial degrees must be in -1..6");
    if (err & 2)
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "a stencil's k + %snumber of monomials exceeds %d",
                        normal_dof ? "Neumann/Robin neighbours + " : "", RBF_MAX_SYSTEM);
    int64_t nnz = 0;
    RBF_CUDA(ctx, cudaMemcpyAsync(&nnz, rp.as<int64_t>() + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nnz < 0 || nnz > (normal_dof ? 2 : 1) * ends[1])
        return rbf_fail(ctx, RBF_ERR_ARGUMENT, "row_ptr is not the layout of this build");
    OutArray oc, ov, os;
    RBF_TRY(oc.bind(ctx, col, sizeof(int32_t) * nnz));
    RBF_TRY(ov.bind(ctx, val, sizeof(double) * nnz * cfg->nops));
    RBF_TRY(os.bind(ctx, status_out, (size_t)ne));
    DevBuf counters;
    RBF_TRY(counters.alloc(ctx, sizeof(unsigned long long) * 8 + sizeof(double)));
    RBF_CUDA(ctx, cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long) * 8 + sizeof(double), ctx->stream));
    P.dim = dim;
    P.phs = cfg->phs;
    P.nops = cfg->nops;
    P.ne = ne;
    P.ns = ns;
    P.nnz = nnz;
    P.data = d.as<double>();
    P.eval = q.as<double>();
    P.adjl = ai.as<int32_t>();
    P.adj_ptr = ap.as<int64_t>();
    P.isb = b.any ? b.isb.as<uint8_t>() : nullptr;
    P.g2b = b.any ? b.g2b.as<int32_t>() : nullptr;
    P.alpha = b.any ? b.alpha.as<double>() : nullptr;
    P.beta = b.any ? b.beta.as<double>() : nullptr;
    P.normals = b.any ? b.normals.as<double>() : nullptr;
    P.row_ptr = rp.as<int64_t>();
    P.col = oc.as<int32_t>();
    P.val = ov.as<double>();
    P.status = os.as<int8_t>();
    P.counters = counters.as<unsigned long long>();
    P.max_resid = reinterpret_cast<double *>(counters.as<unsigned long long>() + 8);
    P.refine_steps = cfg->refine_steps > 0 ? cfg->refine_steps : 6;
    P.tol = cfg->tol > 0 ? cfg->tol : 1e-9;
    P.flags = cfg->flags;
    P.seed = nullptr;
    // one descriptor per size class, largest system first
    std::vector<BinDesc> bins;
    for (int key = 0; key < kRbfBatchKeys; key++) {
        if (!hist[key]) continue;
        BinDesc B;
        memset(&B, 0, sizeof B);
        B.P = P;
        B.P.nnr = key / (65 * 8);
        B.P.k = (key % (65 * 8)) / 8;
        B.P.poly_deg = key % 8 - 1;
        B.P.nmon = monomial_exponents(dim, B.P.poly_deg, B.P.exps);
        B.P.n = B.P.k + B.P.nnr + B.P.nmon;
        B.count = (int64_t)hist[key];
        B.precision = cfg->precision;
        bins.push_back(B);
    }
    std::stable_sort(bins.begin(), bins.end(), [](const BinDesc &a, const BinDesc &c) { return a.P.n > c.P.n; });
    std::vector<int> class_of_key(kRbfBatchKeys, -1);
    std::vector<unsigned long long> class_start(bins.size() + 1, 0ull);
    for (size_t c = 0; c < bins.size(); c++) {
        class_of_key[(bins[c].P.nnr * 65 + bins[c].P.k) * 8 + bins[c].P.poly_deg + 1] = (int)c;
        class_start[c + 1] = class_start[c] + (unsigned long long)bins[c].count;
    }
    DevBuf slots;
    RBF_TRY(slots.alloc(ctx, sizeof(int32_t) * (size_t)std::max<int64_t>(ne, 1)));
    RBF_TRY(rbf_batched_scatter(ctx, ne, keys.as<int32_t>(), class_of_key, class_start, slots.as<int32_t>()));
    for (size_t c = 0; c < bins.size(); c++) bins[c].slots = slots.as<int32_t>() + class_start[c];
    // the split tile's deferred list (refined builds): room for the largest class
    DevBuf defer;
    int64_t max_class = 0;
    for (const auto &bn : bins) max_class = std::max<int64_t>(max_class, bn.count);
    if (cfg->precision == RBF_PREC_FP32_REFINED)
        RBF_TRY(defer.alloc(ctx, sizeof(int32_t) * (size_t)std::max<int64_t>(max_class, 1)));
    RBF_TRY(rbf_batched_tune(ctx, bins, b.any, tune, defer.as<int32_t>()));
    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    cudaEventRecord(ev0, ctx->stream);
    const int st = rbf_batched_run(ctx, bins, defer.as<int32_t>());
    cudaEventRecord(ev1, ctx->stream);
    if (st != RBF_OK) {
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        return st;
    }
    unsigned long long hc[8];
    double hres = 0.0;
    RBF_CUDA(ctx, cudaMemcpyAsync(hc, counters.ptr, sizeof hc, cudaMemcpyDeviceToHost, ctx->stream));
    RBF_CUDA(ctx, cudaMemcpyAsync(&hres, P.max_resid, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    RBF_TRY(oc.finish(ctx));
    RBF_TRY(ov.finish(ctx));
    RBF_TRY(os.finish(ctx));
    RBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    if (stats) {
        stats->n_identity_rows = (int64_t)hc[3];
        stats->n_stencils = ne - (int64_t)hc[3];
        stats->n_singular = (int64_t)hc[0];
        stats->n_fallback = (int64_t)hc[2];
        stats->max_residual = hres;
        stats->ms_build = ms;
        stats->ms_knn = 0.f;
        stats->ms_total = ms;
        stats->n_residuals = (int64_t)hc[4];
        stats->seed_rel_err_mean = 0.0;
    }
    if (hc[1]) return rbf_fail(ctx, RBF_ERR_NOT_FOUND, "evaluation point not found in stencil data (%llu stencils)", hc[1]);
    if (hc[0]) return rbf_fail(ctx, RBF_ERR_SINGULAR, "%llu stencil system(s) are singular", hc[0]);
    return RBF_OK;
}

int rbf_tuning_report(rbf_ctx *ctx, char *buf, int64_t len) {
    if (!ctx || !buf || len < 1) return RBF_ERR_ARGUMENT;
    std::string out;
    char line[256];
    for (const auto &kv : ctx->tune) {
        const unsigned long long k = kv.first;
        const rbf_tune_entry &t = kv.second;
        snprintf(line, sizeof line,
                 "precision=%s dim=%llu phs=%llu nops=%llu k=%llu degree=%lld boundary=%llu op=%llu dudn=%llu: "
                 "tile=%s (warp %.3f ms, block %.3f ms, split %.3f ms, sample %lld)\n",
                 (k & 15) == RBF_PREC_FP64 ? "fp64" : "fp32_refined", (k >> 4) & 15, (k >> 8) & 15, (k >> 12) & 15,
                 (k >> 16) & 255, (long long)((k >> 24) & 15) - 1, (k >> 28) & 1, (k >> 32) & 255, (k >> 40) & 255,
                 t.tile == kTileSplit ? "split" : (t.tile ? "block" : "warp"), t.ms_warp, t.ms_block, t.ms_split,
                 t.sample);
        out += line;
    }
    const size_t m = std::min<size_t>(out.size(), (size_t)len - 1);
    memcpy(buf, out.data(), m);
    buf[m] = 0;
    return RBF_OK;
}

}  // extern "C"
