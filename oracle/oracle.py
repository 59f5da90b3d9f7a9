"""ctypes front end of the CPU oracle (``oracle/rbf_oracle.c``).

TEST INFRASTRUCTURE ONLY.  The oracle is the checker the GPU library is compared
against.  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU
baseline and ``--impl reference`` legs) may import this module; the product path
(``radialbasisfunctions.jl_gb300``) never does.

The C file restates the reference's algorithm (RadialBasisFunctions.jl v0.7.0):
kNN ``src/utils.jl:12-18``, assembly ``src/solve/assembly.jl:95-185``, Hermite rules
``src/solve/assembly.jl:240-468``, rook Bunch-Kaufman ``src/solve/assembly.jl:220-222``,
scatter ``src/solve/execution.jl:39-115,279-303`` and apply
``src/operators/operators.jl:217-218``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "rbf_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "librbf_oracle.so")

OP_IDENT, OP_D1, OP_D2, OP_LAP = 0, 1, 2, 3


def compile_oracle(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, OpenMP)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-std=c11", SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class _Cfg(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("phs", ctypes.c_int), ("poly_deg", ctypes.c_int),
                ("nops", ctypes.c_int), ("op_code", ctypes.c_int * 8), ("op_dim", ctypes.c_int * 8)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(compile_oracle())
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.orc_phs_phi.restype = ctypes.c_double
        L.orc_phs_phi.argtypes = [ctypes.c_int, P, P, ctypes.c_int]
        L.orc_phs_op.restype = ctypes.c_double
        L.orc_phs_op.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int]
        L.orc_phs_op_normal.restype = ctypes.c_double
        L.orc_phs_op_normal.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, ctypes.c_int]
        L.orc_phs_grad.argtypes = [ctypes.c_int, P, P, ctypes.c_int, P]
        L.orc_phs_hess.argtypes = [ctypes.c_int, P, P, ctypes.c_int, P]
        L.orc_monomial_exponents.restype = ctypes.c_int
        L.orc_monomial_exponents.argtypes = [ctypes.c_int, ctypes.c_int, P]
        L.orc_mono_op.argtypes = [ctypes.c_int, ctypes.c_int, P, ctypes.c_int, ctypes.c_int, P, P]
        L.orc_mono_normal.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P, P]
        L.orc_sytrf_rook_u.restype = ctypes.c_int
        L.orc_sytrf_rook_u.argtypes = [ctypes.c_int, P, ctypes.c_int, P]
        L.orc_sytrf_rook_u_fma.restype = ctypes.c_int
        L.orc_sytrf_rook_u_fma.argtypes = [ctypes.c_int, P, ctypes.c_int, P]
        L.orc_sytrs_rook_u.argtypes = [ctypes.c_int, ctypes.c_int, P, ctypes.c_int, P, P, ctypes.c_int]
        L.orc_assemble.restype = ctypes.c_int
        L.orc_assemble.argtypes = [P, P, ctypes.c_int, P, P, P, P]
        L.orc_count_rows.restype = i64
        L.orc_count_rows.argtypes = [i64, ctypes.c_int, P, P, P, P, P]
        L.orc_build.restype = ctypes.c_int
        L.orc_build.argtypes = [P, P, i64, P, i64, P, ctypes.c_int, P, P, P, P, P, P, P, P, ctypes.c_int]
        L.orc_build_local.restype = ctypes.c_int
        L.orc_build_local.argtypes = L.orc_build.argtypes
        L.orc_spmm.argtypes = [i64, i64, P, P, P, ctypes.c_int, P, ctypes.c_double, ctypes.c_double, P,
                               ctypes.c_int]
        L.orc_knn_brute.argtypes = [P, i64, P, i64, ctypes.c_int, ctypes.c_int, P, ctypes.c_int]
        L.orc_knn_grid.restype = ctypes.c_int
        L.orc_knn_grid.argtypes = [P, i64, P, i64, ctypes.c_int, ctypes.c_int, P, ctypes.c_int]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_build_backward.restype = ctypes.c_int
        L.orc_build_backward.argtypes = [P, P, i64, P, i64, P, ctypes.c_int, P, P, P, ctypes.c_int]
        L.orc_interp_matrix.restype = ctypes.c_int
        L.orc_interp_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, i64, P]
        L.orc_interp_eval.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, i64, P, P, i64, P, ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def make_cfg(dim, phs, poly_deg, ops):
    """ops: list of (op_code, op_dim) pairs, op_dim 0-based."""
    c = _Cfg()
    c.dim, c.phs, c.poly_deg, c.nops = dim, phs, poly_deg, len(ops)
    for i, (code, d) in enumerate(ops):
        c.op_code[i] = code
        c.op_dim[i] = d
    return c


# ---------------------------------------------------------------- basis pieces
def phs_phi(p, x, y):
    x, y = _f64(x), _f64(y)
    return lib().orc_phs_phi(p, _p(x), _p(y), x.size)


def phs_op(p, op, odim, x, y):
    x, y = _f64(x), _f64(y)
    return lib().orc_phs_op(p, op, odim, _p(x), _p(y), x.size)


def phs_op_normal(p, op, odim, x, y, n):
    x, y, n = _f64(x), _f64(y), _f64(n)
    return lib().orc_phs_op_normal(p, op, odim, _p(x), _p(y), _p(n), x.size)


def phs_grad(p, x, y):
    x, y = _f64(x), _f64(y)
    g = np.zeros(x.size)
    lib().orc_phs_grad(p, _p(x), _p(y), x.size, _p(g))
    return g


def phs_hess(p, x, y):
    x, y = _f64(x), _f64(y)
    h = np.zeros((x.size, x.size))
    lib().orc_phs_hess(p, _p(x), _p(y), x.size, _p(h))
    return h


def monomial_exponents(dim, deg):
    buf = np.zeros(64 * 3, dtype=np.int32)
    n = lib().orc_monomial_exponents(dim, deg, _p(buf))
    return buf[: n * dim].reshape(n, dim).copy()


def mono_op(dim, deg, op, odim, x):
    e = monomial_exponents(dim, deg)
    x = _f64(x)
    b = np.zeros(len(e))
    e32 = np.ascontiguousarray(e, dtype=np.int32)
    lib().orc_mono_op(dim, len(e), _p(e32), op, odim, _p(x), _p(b))
    return b


def mono_normal(dim, deg, n, x):
    e = np.ascontiguousarray(monomial_exponents(dim, deg), dtype=np.int32)
    x, n = _f64(x), _f64(n)
    b = np.zeros(len(e))
    lib().orc_mono_normal(dim, len(e), _p(e), _p(n), _p(x), _p(b))
    return b


# ---------------------------------------------------------------- rook LDL^T
def sytrf_rook(A):
    """Factor the upper triangle of A (column-major copy); returns (factors, ipiv, info)."""
    n = A.shape[0]
    F = np.asfortranarray(np.array(A, dtype=np.float64))
    ipiv = np.zeros(n, dtype=np.int32)
    info = lib().orc_sytrf_rook_u(n, _p(F), n, _p(ipiv))
    return F, ipiv, info


def sytrs_rook(F, ipiv, B):
    n = F.shape[0]
    Bm = np.asfortranarray(np.array(B, dtype=np.float64).reshape(n, -1))
    lib().orc_sytrs_rook_u(n, Bm.shape[1], _p(F), n, _p(ipiv), _p(Bm), n)
    return Bm


# ---------------------------------------------------------------- per stencil
@dataclass
class HermiteLocal:
    """Local Hermite description, mirrors HermiteStencilData (src/solve/types.jl:66-119)."""
    ptype: np.ndarray  # 0 interior, 1 Dirichlet, 2 Neumann/Robin
    alpha: np.ndarray
    beta: np.ndarray
    normal: np.ndarray  # k x dim
    eval_local: int


class _Herm(ctypes.Structure):
    _fields_ = [("ptype", ctypes.c_int * 160), ("alpha", ctypes.c_double * 160),
                ("beta", ctypes.c_double * 160), ("normal", ctypes.c_double * 480),
                ("eval_local", ctypes.c_int)]


def _herm_struct(h: HermiteLocal, dim):
    s = _Herm()
    k = len(h.ptype)
    for i in range(k):
        s.ptype[i] = int(h.ptype[i])
        s.alpha[i] = float(h.alpha[i])
        s.beta[i] = float(h.beta[i])
        for d in range(dim):
            s.normal[i * dim + d] = float(h.normal[i][d])
    s.eval_local = int(h.eval_local)
    return s


def assemble(dim, phs, poly_deg, ops, X, x0, herm: HermiteLocal | None = None):
    """Returns (A upper-triangular n x n, B n x nops, status)."""
    X = _f64(X)
    k = X.shape[0]
    nmon = len(monomial_exponents(dim, poly_deg)) if poly_deg >= 0 else 0
    n = k + nmon
    A = np.zeros(n * n)
    B = np.zeros(n * len(ops))
    cfg = make_cfg(dim, phs, poly_deg, ops)
    hs = _herm_struct(herm, dim) if herm is not None else None
    st = lib().orc_assemble(ctypes.byref(cfg), _p(X), k, _p(_f64(x0)),
                            ctypes.byref(hs) if hs is not None else None, _p(A), _p(B))
    return A.reshape(n, n).T.copy(), B.reshape(len(ops), n).T.copy(), st


# ---------------------------------------------------------------- global paths
def knn(src, qry, k, brute=False, nthreads=0):
    src, qry = _f64(src), _f64(qry)
    ns, dim = src.shape
    nq = qry.shape[0]
    out = np.zeros((nq, k), dtype=np.int32)
    if brute:
        lib().orc_knn_brute(_p(src), ns, _p(qry), nq, dim, k, _p(out), nthreads)
    else:
        st = lib().orc_knn_grid(_p(src), ns, _p(qry), nq, dim, k, _p(out), nthreads)
        if st != 0:
            raise ValueError("k must not exceed the number of source points")
    return out


@dataclass
class CSR:
    row_ptr: np.ndarray  # int64, ne+1
    col: np.ndarray      # int32, nnz
    val: np.ndarray      # float64, nops x nnz
    status: np.ndarray   # int8 per row
    shape: tuple


def build(data, eval_points, adjl, dim, phs, poly_deg, ops, hermite=None, nthreads=0, frame="raw"):
    """Weights of the operators `ops` on the stencils `adjl` (0-based), sorted rows.

    hermite: None or (is_boundary[uint8 per data point], alpha[nb], beta[nb], normals[nb x dim]).
    frame: "raw" -- the reference's arithmetic (every stencil assembled in the given
    coordinates, src/solve/assembly.jl:95-222); "local" -- the same formulation assembled per
    stencil in its local frame (centred at the eval point, scaled by a power of two): the same
    weights in exact arithmetic, accurate where the raw systems are ill-conditioned (stencils
    small against their distance from the origin).
    """
    data, eval_points = _f64(data), _f64(eval_points)
    adjl = np.ascontiguousarray(adjl, dtype=np.int32)
    ns, ne = data.shape[0], eval_points.shape[0]
    k = adjl.shape[1]
    cfg = make_cfg(dim, phs, poly_deg, ops)
    row_ptr = np.zeros(ne + 1, dtype=np.int64)
    if hermite is not None:
        isb = np.ascontiguousarray(hermite[0], dtype=np.uint8)
        al, be = _f64(hermite[1]), _f64(hermite[2])
        nr = _f64(hermite[3]).reshape(-1)
        g2b = np.full(max(ns, ne), -1, dtype=np.int32)
        g2b[np.nonzero(isb)[0]] = np.arange(int(isb.sum()), dtype=np.int32)
        nnz = lib().orc_count_rows(ne, k, _p(isb), _p(g2b), _p(al), _p(be), _p(row_ptr))
    else:
        isb = al = be = nr = None
        nnz = lib().orc_count_rows(ne, k, None, None, None, None, _p(row_ptr))
    col = np.zeros(nnz, dtype=np.int32)
    val = np.zeros(len(ops) * nnz)
    status = np.zeros(ne, dtype=np.int8)
    fn = lib().orc_build if frame == "raw" else lib().orc_build_local
    fn(ctypes.byref(cfg), _p(data), ns, _p(eval_points), ne, _p(adjl), k, _p(isb), _p(al),
       _p(be), _p(nr), _p(row_ptr), _p(col), _p(val), _p(status), nthreads)
    return CSR(row_ptr, col, val.reshape(len(ops), nnz), status, (ne, ns))


def spmm(csr: CSR, x, op_index=0, alpha=1.0, beta=0.0, y=None, nthreads=0):
    """y = alpha*W*x + beta*y; x is (ns,) or (ns, nf) (column per field)."""
    x = np.asarray(x, dtype=np.float64)
    vec = x.ndim == 1
    xf = np.asfortranarray(x.reshape(x.shape[0], -1))
    nf = xf.shape[1]
    ne, ns = csr.shape
    yf = np.zeros((ne, nf), order="F") if y is None else np.asfortranarray(np.array(y, dtype=np.float64).reshape(ne, nf))
    v = np.ascontiguousarray(csr.val[op_index])
    lib().orc_spmm(ne, ns, _p(csr.row_ptr), _p(csr.col), _p(v), nf, _p(xf), alpha, beta, _p(yf), nthreads)
    return yf[:, 0].copy() if vec else np.ascontiguousarray(yf)


def num_threads():
    return lib().orc_num_threads()


# ---------------------------------------------------------------- global interpolation
def interp_matrix(x, phs, poly_deg):
    """Upper triangle of the Interpolator's collocation matrix (src/interpolation.jl:27-31),
    column-major (Fortran order) numpy array of order n + nmon."""
    x = _f64(x)
    n, dim = x.shape
    nmon = len(monomial_exponents(dim, poly_deg)) if poly_deg >= 0 else 0
    A = np.zeros((n + nmon) * (n + nmon))
    lib().orc_interp_matrix(dim, phs, poly_deg, _p(x), n, _p(A))
    return A.reshape(n + nmon, n + nmon).T  # view: A[i, j] = element (i, j)


def sytrf_rook_restated(A, fused=False):
    """The restated unblocked dsytf2_rook (UPLO = 'U') on a Fortran-ordered copy of A; fused:
    its rank-1 / rank-2 updates as fused multiply-adds (as optimised BLAS kernels do)."""
    n = A.shape[0]
    F = np.asfortranarray(np.array(A, dtype=np.float64))
    ipiv = np.zeros(n, dtype=np.int32)
    f = lib().orc_sytrf_rook_u_fma if fused else lib().orc_sytrf_rook_u
    info = f(n, _p(F), n, _p(ipiv))
    return F, ipiv, info


def rook_steps(ipiv):
    """The pivot steps of a UPLO = 'U' rook factorisation in factorisation order: (k, kstep,
    interchanges), k 1-based, interchanges the (row, row) swaps the step applied in order."""
    n = len(ipiv)
    k = n
    steps = []
    while k >= 1:
        if ipiv[k - 1] > 0:
            kp = int(ipiv[k - 1])
            steps.append((k, 1, [(k, kp)] if kp != k else []))
            k -= 1
        else:
            p, kp = -int(ipiv[k - 1]), -int(ipiv[k - 2])
            sw = []
            if p != k:
                sw.append((k, p))
            if kp != k - 1:
                sw.append((k - 1, kp))
            steps.append((k, 2, sw))
            k -= 2
    return steps


def convert_rook_factor(F, ipiv):
    """Apply each step's interchanges to the factor columns computed before it (columns > k),
    in factorisation order: the factor with one row permutation, as LAPACK's dsyconvf_rook
    (UPLO = 'U', WAY = 'C') leaves it (the D blocks are not moved).  Returns a copy."""
    G = np.array(F, order="F", copy=True)
    n = G.shape[0]
    for k, _, sw in rook_steps(ipiv):
        for a, b in sw:
            if k < n:
                ra, rb = G[a - 1, k:].copy(), G[b - 1, k:].copy()
                G[a - 1, k:], G[b - 1, k:] = rb, ra
    return G


def interp_fit(x, y, phs, poly_deg, solver="restated"):
    """Interpolator(x, y, basis) weights [rbf weights; monomial weights]: the collocation
    matrix factorised by rook Bunch-Kaufman and solved (src/interpolation.jl:27-36).
    solver "restated": this oracle's dsytf2_rook / dsytrs_rook; a callable (A, b) -> w
    substitutes another implementation of the same LAPACK routines."""
    x = _f64(x)
    n = x.shape[0]
    A = interp_matrix(x, phs, poly_deg)
    b = np.zeros(A.shape[0])
    b[:n] = np.asarray(y, np.float64)
    if callable(solver):
        return solver(A, b)
    F, ipiv, info = sytrf_rook_restated(A)
    if info != 0:
        raise np.linalg.LinAlgError("singular collocation matrix")
    return sytrs_rook(F, ipiv, b)[:, 0]


def interp_eval(x, coef, xe, phs, poly_deg, nthreads=0):
    """(rbfi::Interpolator)(xe) for every row of xe (src/interpolation.jl:39-52)."""
    x, xe, coef = _f64(x), _f64(xe), _f64(coef)
    n, dim = x.shape
    m = xe.shape[0]
    out = np.zeros(m)
    lib().orc_interp_eval(dim, phs, poly_deg, _p(x), n, _p(coef), _p(xe), m, _p(out), nthreads)
    return out


def lapack_rook_solver():
    """(A, b) -> x through LAPACK's dsytrf_rook / dsytrs_rook (UPLO = 'U') from scipy's bundled
    OpenBLAS -- the routines bunchkaufman!(A, true) and its ldiv! call; None if not found."""
    import glob
    import os as _os
    try:
        import scipy
    except ImportError:
        return None
    L = None
    for p in glob.glob(_os.path.join(_os.path.dirname(scipy.__file__), "..", "scipy.libs", "libscipy_openblas*.so")):
        cand = ctypes.CDLL(p)
        if hasattr(cand, "scipy_dsytrf_rook_") and hasattr(cand, "scipy_dsytrs_rook_"):
            L = cand
            break
    if L is None:
        return None

    def solve(A, b):
        n = A.shape[0]
        F = np.asfortranarray(A)
        ip = np.zeros(n, dtype=np.int32)
        lw = 64 * n
        w = np.zeros(lw)
        info = ctypes.c_int(0)
        N, LW, R = ctypes.c_int(n), ctypes.c_int(lw), ctypes.c_int(1)
        V = ctypes.c_void_p
        L.scipy_dsytrf_rook_(ctypes.c_char_p(b"U"), ctypes.byref(N), F.ctypes.data_as(V), ctypes.byref(N),
                             ip.ctypes.data_as(V), w.ctypes.data_as(V), ctypes.byref(LW), ctypes.byref(info),
                             ctypes.c_size_t(1))
        if info.value != 0:
            raise np.linalg.LinAlgError("singular collocation matrix")
        B = np.asfortranarray(np.array(b, dtype=np.float64).reshape(n, 1))
        L.scipy_dsytrs_rook_(ctypes.c_char_p(b"U"), ctypes.byref(N), ctypes.byref(R), F.ctypes.data_as(V),
                             ctypes.byref(N), ip.ctypes.data_as(V), B.ctypes.data_as(V), ctypes.byref(N),
                             ctypes.byref(info), ctypes.c_size_t(1))
        return B[:, 0]
    return solve


def build_backward_c(data, eval_points, adjl, dim, phs, poly_deg, ops, dW, nthreads=0):
    """The pullback of the weight build in C (OpenMP): the same rules as
    backward_oracle.build_backward (dW: (len(ops), ne, k), stencil order); returns
    (ddata, deval)."""
    data, eval_points = _f64(data), _f64(eval_points)
    adjl = np.ascontiguousarray(adjl, dtype=np.int32)
    dW = np.ascontiguousarray(dW, dtype=np.float64)
    ns, ne, k = data.shape[0], eval_points.shape[0], adjl.shape[1]
    ddata = np.zeros((ns, dim))
    deval = np.zeros((ne, dim))
    cfg = make_cfg(dim, phs, poly_deg, ops)
    bad = lib().orc_build_backward(ctypes.byref(cfg), _p(data), ns, _p(eval_points), ne, _p(adjl), k, _p(dW),
                                   _p(ddata), _p(deval), nthreads)
    if bad:
        raise np.linalg.LinAlgError(f"{bad} singular stencil systems")
    return ddata, deval
