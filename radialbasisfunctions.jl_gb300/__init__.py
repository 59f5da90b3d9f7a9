"""GB300-native local RBF-FD operators with the interface of RadialBasisFunctions.jl.

Host-side mirror of the reference's operator API for the local RBF-FD hot path
(RadialBasisFunctions.jl v0.7.0).  Every compute step runs in librbffd_gb300.so
(hand-written sm_103a CUDA behind the C ABI of include/rbffd.h); this module only
validates arguments, owns device buffers (through torch) and maps errors to the
reference's exception classes.  There is no CPU fallback.

Reference surface mirrored here (file:line in the reference):
  PHS / PHS1 / PHS3 / PHS5 / PHS7         src/basis/polyharmonic_spline.jl:21-34,43-305
  BoundaryCondition, Dirichlet, Neumann,
  Robin, Internal                         src/solve/types.jl:18-42
  find_neighbors, autoselect_k            src/utils.jl:5-18,39-43
  Laplacian, Partial, Jacobian, Regrid    src/operators/{laplacian,partial,jacobian,regridding}.jl
  laplacian, partial, gradient, jacobian,
  regrid                                  same files
  RadialBasisOperator (+ call, weights,
  update_weights, mul)                    src/operators/operators.jl:50-186,529-602

Indices (neighbour lists, sparse rows) are 0-based.  The `dim` argument of `partial`
keeps the reference's meaning and numbering (1-based dimension index).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _native

__all__ = [
    "PHS", "PHS1", "PHS3", "PHS5", "PHS7", "BoundaryCondition", "Dirichlet", "Neumann", "Robin", "Internal",
    "find_neighbors", "autoselect_k", "Laplacian", "Partial", "Jacobian", "Regrid", "Operators",
    "laplacian", "partial", "gradient", "jacobian", "regrid", "directional", "Directional", "RadialBasisOperator",
    "WeightsCSR", "WeightsSELL",
    "weights", "update_weights", "mul", "DimensionMismatch", "SingularException", "Context", "build_library",
    "Interpolator", "sytrf_rook", "sytrs_rook", "apply_differentiable", "build_weights", "build_weights_backward", "build_weights_differentiable", "build_weights_batched", "ragged_stencils", "tuning_report", "BuildApplyGraph", "reorder_points",
]

build_library = _native.build_library

OP_IDENTITY, OP_PARTIAL1, OP_PARTIAL2, OP_LAPLACIAN = 0, 1, 2, 3
PRECISIONS = {"fp64": 0, "fp32_refined": 1, "learned": 2}


class DimensionMismatch(ValueError):
    """The reference's DimensionMismatch."""


class SingularException(np.linalg.LinAlgError):
    """A stencil's saddle-point system is exactly singular (LAPACK info > 0 in the reference)."""


def _raise(code: int, msg: str):
    if code == -1:
        raise ValueError(msg)
    if code == -2:
        raise DimensionMismatch(msg)
    if code == -4:
        raise SingularException(msg)
    if code == -5:
        raise ValueError(msg)
    if code == -6:
        raise ValueError(msg)
    raise RuntimeError(f"librbffd_gb300 error {code}: {msg}")


# ------------------------------------------------------------------------------ context
class Context:
    """One CUDA context handle of the library (a device + a stream)."""

    _default: dict = {}

    def __init__(self, device: int = 0):
        self.lib = _native.load()
        h = ctypes.c_void_p()
        st = self.lib.rbf_ctx_create(device, ctypes.byref(h))
        if st != 0:
            raise RuntimeError(f"rbf_ctx_create({device}) failed with {st}: no usable CUDA device")
        self.handle = h
        self.device = device
        self._bound = None

    @property
    def h(self):
        """The context handle, bound first to torch's current stream on this device.

        torch's caching allocator recycles a freed tensor's memory in the order of torch's
        stream, so every library launch must be ordered on that same stream: a kernel on
        another stream could still write memory that torch already handed to a new tensor.
        The legacy default stream (handle 0 in torch) is passed as cudaStreamLegacy."""
        torch = _torch()
        s = torch.cuda.current_stream(self.device).cuda_stream or 1
        if s != self._bound:
            self.check(self.lib.rbf_ctx_set_stream(self.handle, ctypes.c_void_p(s)))
            self._bound = s
        return self.handle

    @classmethod
    def default(cls, device: int = 0) -> "Context":
        ctx = cls._default.get(device)
        if ctx is None:
            ctx = cls._default[device] = Context(device)
        return ctx

    def check(self, st: int):
        if st != 0:
            _raise(st, self.lib.rbf_last_error(self.handle).decode())

    def set_stream(self, stream_handle: int | None):
        """Bind a raw cudaStream_t (None: the context's own stream).  Calls through this
        package rebind to torch's current stream; this is for direct C-ABI use."""
        self.check(self.lib.rbf_ctx_set_stream(self.handle, ctypes.c_void_p(stream_handle or 0)))
        self._bound = stream_handle or None

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.rbf_ctx_destroy(self.handle)
        except Exception:
            pass


# ------------------------------------------------------------------------------ arrays
def _torch():
    import torch
    return torch


def _is_torch(x):
    try:
        import torch
        return isinstance(x, torch.Tensor)
    except ImportError:
        return False


def _points(x, name="data"):
    """(N, dim) float64 array: numpy (host) or torch (host or cuda), C-contiguous."""
    if _is_torch(x):
        t = x.detach()
        if t.dtype != _torch().float64:
            t = t.to(_torch().float64)
        t = t.contiguous()
        if t.ndim == 1:
            t = t.reshape(-1, 1)
        return t
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    if a.ndim != 2:
        raise ValueError(f"{name} must be an (N, dim) array of points")
    return a


def _ptr(a):
    if a is None:
        return None
    if _is_torch(a):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def _to_device(a, ctx):
    torch = _torch()
    if _is_torch(a):
        return a.to(torch.device("cuda", ctx.device), torch.float64).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(torch.device("cuda", ctx.device))


def _device_of(*arrays):
    for a in arrays:
        if _is_torch(a) and a.is_cuda:
            return a.device.index or 0
    return 0


# ------------------------------------------------------------------------------ bases
@dataclass(frozen=True)
class _PHSBase:
    poly_deg: int = 2
    order: int = 3

    def __post_init__(self):
        check_poly_deg(self.poly_deg)

    def __repr__(self):
        sup = {1: "¹", 3: "³", 5: "⁵", 7: "⁷"}[self.order]
        return f"Polyharmonic spline (r{sup})\n└─Polynomial augmentation: degree {self.poly_deg}"


class PHS1(_PHSBase):
    def __init__(self, poly_deg: int = 2):
        super().__init__(poly_deg, 1)


class PHS3(_PHSBase):
    def __init__(self, poly_deg: int = 2):
        super().__init__(poly_deg, 3)


class PHS5(_PHSBase):
    def __init__(self, poly_deg: int = 2):
        super().__init__(poly_deg, 5)


class PHS7(_PHSBase):
    def __init__(self, poly_deg: int = 2):
        super().__init__(poly_deg, 7)


def check_poly_deg(poly_deg: int):
    """src/utils.jl:57-66"""
    if poly_deg < -1:
        raise ValueError(f"poly_deg must be >= -1 (got {poly_deg}). Use poly_deg=2 (default) for quadratic, "
                         "poly_deg=0 for constant, or poly_deg=-1 to disable polynomial augmentation.")


def PHS(n: int = 3, poly_deg: int = 2):
    """Polyharmonic spline r^n with degree-poly_deg augmentation (polyharmonic_spline.jl:21-34)."""
    check_poly_deg(poly_deg)
    if n % 2 == 0 or n > 7 or n < 1:
        raise ValueError(f"n must be 1, 3, 5, or 7 (got n={n}). Use PHS(3) for cubic or PHS(5) for quintic.")
    return {1: PHS1, 3: PHS3, 5: PHS5, 7: PHS7}[n](poly_deg)


# ------------------------------------------------------------------------------ boundary conditions
@dataclass(frozen=True)
class BoundaryCondition:
    """B u = alpha*u + beta*du/dn (src/solve/types.jl:18-42)."""
    alpha: float
    beta: float

    def is_dirichlet(self):
        return self.alpha == 1 and self.beta == 0

    def is_neumann(self):
        return self.alpha == 0 and self.beta == 1

    def is_robin(self):
        return self.alpha != 0 and self.beta != 0

    def is_internal(self):
        return self.alpha == 0 and self.beta == 0


def Dirichlet():
    return BoundaryCondition(1.0, 0.0)


def Neumann():
    return BoundaryCondition(0.0, 1.0)


def Robin(alpha: float, beta: float):
    return BoundaryCondition(float(alpha), float(beta))


def Internal():
    return BoundaryCondition(0.0, 0.0)


# ------------------------------------------------------------------------------ operators
class _Op:
    rank = 0

    def ops(self, dim: int):
        raise NotImplementedError


class Laplacian(_Op):
    """∇² (src/operators/laplacian.jl:6-7)."""

    def ops(self, dim):
        return [(OP_LAPLACIAN, 0)]

    def __repr__(self):
        return "Laplacian (∇²f)"


class Partial(_Op):
    """∂ⁿ/∂x_dim (src/operators/partial.jl:6-10,49-61); dim is 1-based as in the reference."""

    def __init__(self, order: int, dim: int):
        if order not in (1, 2):
            raise ValueError("Only first and second order derivatives are supported. "
                             "Use the custom operator for higher orders.")
        self.order, self.dim = order, dim

    def ops(self, dim):
        if not 1 <= self.dim <= dim:
            raise ValueError(f"dimension {self.dim} out of range 1..{dim}")
        return [(OP_PARTIAL1 if self.order == 1 else OP_PARTIAL2, self.dim - 1)]

    def __repr__(self):
        return f"∂ⁿf/∂xᵢ (n = {self.order}, i = {self.dim})"


class Jacobian(_Op):
    """Tuple of first partials, one factorisation with D right-hand sides (jacobian.jl:19,53-62)."""
    rank = 1

    def __init__(self, dim: int | None = None):
        self.dim = dim

    def ops(self, dim):
        return [(OP_PARTIAL1, d) for d in range(dim)]

    def __repr__(self):
        return "Jacobian (J)"


class Regrid(_Op):
    """Interpolation to other points: the operator is the identity (regridding.jl:6-7)."""

    def ops(self, dim):
        return [(OP_IDENTITY, 0)]

    def __repr__(self):
        return "regrid"


class Directional(_Op):
    """∇f⋅v: the gradient weights combined with a direction (src/operators/directional.jl:6-10,
    69-95); v is one direction of length dim or one direction per evaluation point."""

    def __init__(self, v):
        self.v = v

    def ops(self, dim):
        return [(OP_PARTIAL1, d) for d in range(dim)]

    def __repr__(self):
        return "Directional Derivative (∇f⋅v)"


class _Combined(_Op):
    """A sum / difference / scaling of built operators (operator_algebra.jl:245-295)."""

    def __init__(self, desc: str, rank: int):
        self.desc, self.rank = desc, rank

    def __repr__(self):
        return self.desc


class Operators(_Op):
    """Several operators built from one factorisation per stencil (e.g. gradient + Laplacian).

    Not in the reference, which factorises once per operator; the weights are identical."""
    rank = 1

    def __init__(self, *ops: _Op):
        self.parts = ops

    def ops(self, dim):
        out = []
        for p in self.parts:
            out.extend(p.ops(dim))
        return out

    def __repr__(self):
        return " + ".join(map(repr, self.parts))


# ------------------------------------------------------------------------------ neighbours
def autoselect_k(data, basis) -> int:
    """min(N, max(2*binomial(m+d, d), 2d+1)) (src/utils.jl:39-43)."""
    pts = _points(data)
    n, d = pts.shape
    m = basis.poly_deg
    return min(n, max(2 * math.comb(m + d, d) if m >= 0 else 0, 2 * d + 1))


def find_neighbors(data, eval_points=None, k: int | None = None, *, ctx: Context | None = None, out=None):
    """k nearest data points of every eval point, sorted by distance, ties by index (0-based).

    Mirrors find_neighbors(data, [eval_points,] k) (src/utils.jl:5-18).  Returns an
    (N_eval, k) int32 array (numpy for host inputs, torch on the GPU for cuda inputs)."""
    if k is None:
        if isinstance(eval_points, (int, np.integer)):
            k, eval_points = int(eval_points), None
        else:
            raise TypeError("find_neighbors needs k")
    d = _points(data)
    q = d if eval_points is None else _points(eval_points, "eval_points")
    if d.shape[1] != q.shape[1]:
        raise DimensionMismatch("data and eval_points must have the same dimension")
    ctx = ctx or Context.default(_device_of(d, q))
    ne = q.shape[0]
    if out is None:
        if _is_torch(q) and q.is_cuda:
            out = _torch().empty((ne, k), dtype=_torch().int32, device=q.device)
        else:
            out = np.empty((ne, k), dtype=np.int32)
    ctx.check(ctx.lib.rbf_knn(ctx.h, _ptr(d), d.shape[0], _ptr(q), ne, d.shape[1], k, _ptr(out)))
    return out


# ------------------------------------------------------------------------------ weights
class WeightsCSR:
    """Sparse weights on the GPU (CSR, columns ascending within rows).

    The reference returns SparseMatrixCSC (src/solve/execution.jl:105-115); the same
    matrix in CSR is the CSC of its transpose, and to_csc() produces the CSC arrays."""

    def __init__(self, row_ptr, col, val, shape, ctx: Context, sell=None):
        self.row_ptr, self.col, self.val, self.shape, self.ctx = row_ptr, col, val, shape, ctx
        self.sell = sell  # optional WeightsSELL copy of the same operator

    @property
    def nnz(self):
        return int(self.col.shape[0])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val.cpu().numpy(), self.col.cpu().numpy(), self.row_ptr.cpu().numpy()),
                             shape=self.shape)

    def to_csc(self):
        torch = _torch()
        ne, ns = self.shape
        dev = self.col.device
        cp = torch.empty(ns + 1, dtype=torch.int64, device=dev)
        rw = torch.empty(self.nnz, dtype=torch.int32, device=dev)
        vv = torch.empty(self.nnz, dtype=torch.float64, device=dev)
        self.ctx.check(self.ctx.lib.rbf_csr_to_csc(self.ctx.h, ne, ns, _ptr(self.row_ptr), _ptr(self.col),
                                                   _ptr(self.val), _ptr(cp), _ptr(rw), _ptr(vv)))
        return cp, rw, vv

    def apply(self, x, y=None, alpha=1.0, beta=0.0, layout="colmajor"):
        if (self.sell is not None and _is_torch(x) and x.is_cuda and x.ndim == 1 and x.dtype == _torch().float64
                and (y is None or (_is_torch(y) and y.is_cuda and y.is_contiguous() and y.dtype == x.dtype))):
            return self.sell.apply(x, y, alpha, beta)
        return _spmm(self, x, y, alpha, beta, layout)

    def to_sell(self):
        """The same operator in sliced-ELL form (rbf_sell_offsets + rbf_sell_from_csr), for
        repeated single-field applies."""
        torch = _torch()
        ne, ns = self.shape
        dev = self.col.device
        off = torch.empty((ne + 31) // 32 + 1, dtype=torch.int64, device=dev)
        tot = ctypes.c_int64(0)
        self.ctx.check(self.ctx.lib.rbf_sell_offsets(self.ctx.h, ne, _ptr(self.row_ptr), _ptr(off), ctypes.byref(tot)))
        c = torch.empty(tot.value, dtype=torch.int32, device=dev)
        v = torch.empty(tot.value, dtype=torch.float64, device=dev)
        self.ctx.check(self.ctx.lib.rbf_sell_from_csr(self.ctx.h, ne, _ptr(self.row_ptr), _ptr(self.col),
                                                      _ptr(self.val), _ptr(off), _ptr(c), _ptr(v)))
        return WeightsSELL(off, c, v, self.shape, self.ctx)

    def to_sell_ordered(self, data, eval_points=None, row_at=None, col_at=None):
        """The sliced copy in a locality order (rbf_sell_offsets_perm + rbf_sell_from_csr_perm):
        rows in the Morton order of the eval points and columns in that of the data points
        (rbf_reorder_points; one order when the eval points are the data points), applied with
        x and y in the caller's order.  For operators on unordered points applied many times."""
        torch = _torch()
        ne, ns = self.shape
        dev = self.col.device
        d = _points(data)
        if col_at is None:
            col_at, _ = reorder_points(d if _is_torch(d) else torch.from_numpy(d).to(dev), ctx=self.ctx)
        if row_at is None:
            if eval_points is None:
                row_at = col_at
            else:
                q = _points(eval_points, "eval_points")
                row_at, _ = reorder_points(q if _is_torch(q) else torch.from_numpy(q).to(dev), ctx=self.ctx)
        row_at = torch.as_tensor(row_at).to(dev, torch.int32).contiguous()
        col_at = torch.as_tensor(col_at).to(dev, torch.int32).contiguous()
        if row_at.numel() != ne or col_at.numel() != ns:
            raise DimensionMismatch("row_at / col_at must hold one entry per row / column")
        off = torch.empty((ne + 31) // 32 + 1, dtype=torch.int64, device=dev)
        tot = ctypes.c_int64(0)
        self.ctx.check(self.ctx.lib.rbf_sell_offsets_perm(self.ctx.h, ne, _ptr(self.row_ptr), _ptr(row_at), _ptr(off),
                                                          ctypes.byref(tot)))
        c = torch.empty(max(tot.value, 1), dtype=torch.int32, device=dev)
        v = torch.empty(max(tot.value, 1), dtype=torch.float64, device=dev)
        self.ctx.check(self.ctx.lib.rbf_sell_from_csr_perm(self.ctx.h, ne, ns, _ptr(self.row_ptr), _ptr(self.col),
                                                           _ptr(self.val), _ptr(row_at), _ptr(col_at), _ptr(off),
                                                           _ptr(c), _ptr(v)))
        return WeightsSELLOrdered(off, c, v, row_at, col_at, self.shape, self.ctx)

    def __matmul__(self, x):
        return self.apply(x)


class WeightsSELLOrdered:
    """An operator's sliced copy in a locality order of its rows and columns (see
    WeightsCSR.to_sell_ordered): y = alpha W x + beta y for one field in the caller's order."""

    def __init__(self, slice_off, col, val, row_at, col_at, shape, ctx: Context):
        self.slice_off, self.col, self.val, self.row_at, self.col_at = slice_off, col, val, row_at, col_at
        self.shape, self.ctx = shape, ctx
        self._work = None

    def apply(self, x, y=None, alpha=1.0, beta=0.0):
        torch = _torch()
        ne, ns = self.shape
        dev = self.col.device
        xt = torch.as_tensor(x, dtype=torch.float64).to(dev).contiguous()
        if xt.ndim != 1 or xt.shape[0] != ns:
            raise DimensionMismatch(f"the sliced apply takes one field of {ns} values")
        out = y if y is not None else torch.zeros(ne, dtype=torch.float64, device=dev)
        if out.dtype != torch.float64 or not out.is_cuda or not out.is_contiguous() or out.shape != (ne,):
            raise DimensionMismatch("y must be a contiguous float64 CUDA vector of the operator's row count")
        if self._work is None:
            self._work = torch.empty(max(ns, 1), dtype=torch.float64, device=dev)
        self.ctx.check(self.ctx.lib.rbf_spmv_sell_perm(self.ctx.h, ne, ns, _ptr(self.slice_off), _ptr(self.col),
                                                       _ptr(self.val), _ptr(self.row_at), _ptr(self.col_at), _ptr(xt),
                                                       _ptr(self._work), float(alpha),
                                                       float(beta) if y is not None else 0.0, _ptr(out)))
        return out

    def __matmul__(self, x):
        return self.apply(x)


class WeightsSELL:
    """An operator in sliced-ELL form (slices of 32 rows, entry j of a slice's rows
    contiguous): y = alpha W x + beta y for one field on the GPU (rbf_spmv_sell), the
    product of the CSR it was made from."""

    def __init__(self, slice_off, col, val, shape, ctx: Context):
        self.slice_off, self.col, self.val, self.shape, self.ctx = slice_off, col, val, shape, ctx

    def apply(self, x, y=None, alpha=1.0, beta=0.0):
        torch = _torch()
        ne, ns = self.shape
        xt = torch.as_tensor(x, dtype=torch.float64).to(self.col.device).contiguous()
        if xt.ndim != 1 or xt.shape[0] != ns:
            raise DimensionMismatch(f"the sliced apply takes one field of {ns} values")
        out = y if y is not None else torch.zeros(ne, dtype=torch.float64, device=self.col.device)
        if out.dtype != torch.float64 or not out.is_cuda or not out.is_contiguous() or out.shape != (ne,):
            raise DimensionMismatch("y must be a contiguous float64 CUDA vector of the operator's row count")
        self.ctx.check(self.ctx.lib.rbf_spmv_sell(self.ctx.h, ne, _ptr(self.slice_off), _ptr(self.col),
                                                  _ptr(self.val), _ptr(xt), float(alpha),
                                                  float(beta) if y is not None else 0.0, _ptr(out)))
        return out

    def __matmul__(self, x):
        return self.apply(x)


def _spmm(W: WeightsCSR, x, y=None, alpha=1.0, beta=0.0, layout="colmajor"):
    torch = _torch()
    ne, ns = W.shape
    ctx = W.ctx
    host = not (_is_torch(x) and x.is_cuda)
    if _is_torch(x):
        xt = x.detach().to(torch.float64).contiguous()
    else:
        xt = np.asarray(x, dtype=np.float64)
    if xt.shape[0] != ns:
        raise DimensionMismatch(f"operand has {xt.shape[0]} rows, operator has {ns} columns")
    nf = 1 if xt.ndim == 1 else int(np.prod(xt.shape[1:]))
    if layout == "colmajor" and nf > 1:
        # (ns, nf) with fields in columns -> column-major buffer (field f contiguous)
        xb = xt.reshape(ns, nf).T.contiguous() if _is_torch(xt) else np.ascontiguousarray(xt.reshape(ns, nf).T)
        lay, ldx, ldy = 0, ns, ne
    else:
        xb = xt.reshape(ns, nf).contiguous() if _is_torch(xt) else np.ascontiguousarray(xt.reshape(ns, nf))
        lay, ldx, ldy = 1, nf, nf
    out_shape = (ne,) if xt.ndim == 1 else (ne,) + tuple(xt.shape[1:])
    if host:
        yb = np.zeros((nf, ne) if lay == 0 else (ne, nf), dtype=np.float64)
        if y is not None and beta != 0.0:
            yy = np.asarray(y, dtype=np.float64).reshape(ne, nf)
            yb[:] = yy.T if lay == 0 else yy
    else:
        yb = torch.zeros((nf, ne) if lay == 0 else (ne, nf), dtype=torch.float64, device=xt.device)
        if y is not None and beta != 0.0:
            yy = y.reshape(ne, nf).to(torch.float64)
            yb.copy_(yy.T if lay == 0 else yy)
    if nf == 1:
        ldx = ldy = 1
    ctx.check(ctx.lib.rbf_spmm(ctx.h, ne, ns, _ptr(W.row_ptr), _ptr(W.col), _ptr(W.val), nf, lay, _ptr(xb),
                               ldx, float(alpha), float(beta), _ptr(yb), ldy))
    res = yb.T if lay == 0 else yb
    res = res.reshape(out_shape)
    if y is not None:
        if _is_torch(y):
            y.copy_(res if _is_torch(res) else torch.from_numpy(np.ascontiguousarray(res)))
        else:
            y[...] = res.cpu().numpy() if _is_torch(res) else res
        return y
    return res


def _hermite_arrays(hermite, ns, dim):
    if hermite is None:
        return None
    if isinstance(hermite, dict):
        isb, bcs, normals = hermite["is_boundary"], hermite["bc"], hermite["normals"]
    else:
        isb, bcs, normals = hermite.is_boundary, hermite.bc, hermite.normals
    isb = np.ascontiguousarray(np.asarray(isb, dtype=np.uint8))
    if isb.shape[0] != ns:
        raise DimensionMismatch(f"length(is_boundary) = {isb.shape[0]} must equal the number of data points ({ns})")
    alpha = np.ascontiguousarray([float(b.alpha) for b in bcs], dtype=np.float64)
    beta = np.ascontiguousarray([float(b.beta) for b in bcs], dtype=np.float64)
    nrm = np.ascontiguousarray(np.asarray(normals, dtype=np.float64).reshape(-1, dim) if len(bcs) else
                               np.zeros((0, dim)))
    nb = int(isb.sum())
    if len(bcs) != nb or nrm.shape[0] != nb:
        raise DimensionMismatch(f"boundary_conditions ({len(bcs)}) and normals ({nrm.shape[0]}) must each have "
                                f"one entry per boundary point (count(is_boundary) = {nb})")
    return isb, alpha, beta, nrm


def build_weights(ops, data, eval_points, adjl, basis, hermite=None, precision="fp64", *, ctx=None,
                  refine_steps=0, tol=0.0, return_status=False, stats=None, flags=0, seed=None, sell=False):
    """Weights of `ops` (list of (op_code, op_dim)) on stencils adjl; returns a list of WeightsCSR.

    The drop-in for _build_weights (src/solve/api.jl:26-35, 167-196).  sell=True has the
    build also write a sliced-ELL copy (WeightsCSR.sell), which single-field applies use."""
    torch = _torch()
    d = _points(data)
    q = d if eval_points is None else _points(eval_points, "eval_points")
    ns, dim = d.shape
    ne = q.shape[0]
    ctx = ctx or Context.default(_device_of(d, q, adjl))
    dev = torch.device("cuda", ctx.device)
    if _is_torch(adjl):
        a = adjl.to(torch.int32).contiguous()
    else:
        a = np.ascontiguousarray(np.asarray(adjl, dtype=np.int32))
    if a.ndim != 2 or a.shape[0] != ne:
        raise DimensionMismatch("adjl must be an (N_eval, k) array of 0-based data indices")
    k = int(a.shape[1])
    cfg = _native.BuildCfg()
    cfg.dim, cfg.phs, cfg.poly_deg, cfg.nops = dim, basis.order, basis.poly_deg, len(ops)
    for i, (c, od) in enumerate(ops):
        cfg.op_code[i] = c
        cfg.op_dim[i] = od
    cfg.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    cfg.refine_steps = refine_steps
    cfg.tol = tol
    cfg.flags = flags
    if seed is not None:
        seed = seed.to(torch.float32).contiguous()
        cfg.seed = seed.data_ptr()
    herm = _hermite_arrays(hermite, ns, dim)
    hs = None
    keep = []
    if herm is not None:
        isb, al, be, nr = herm
        hs = _native.Hermite(isb.ctypes.data, al.ctypes.data, be.ctypes.data, nr.ctypes.data, len(al))
        keep.append(herm)
    row_ptr = torch.empty(ne + 1, dtype=torch.int64, device=dev)
    nnz = ctypes.c_int64(0)
    ctx.check(ctx.lib.rbf_build_count(ctx.h, ns, ne, k, ctypes.byref(hs) if hs else None, _ptr(row_ptr),
                                      ctypes.byref(nnz)))
    col = torch.empty(nnz.value, dtype=torch.int32, device=dev)
    val = torch.empty((len(ops), nnz.value), dtype=torch.float64, device=dev)
    status = torch.empty(ne, dtype=torch.int8, device=dev) if return_status else None
    sells = [None] * len(ops)
    if sell:
        off = torch.empty((ne + 31) // 32 + 1, dtype=torch.int64, device=dev)
        tot = ctypes.c_int64(0)
        ctx.check(ctx.lib.rbf_sell_offsets(ctx.h, ne, _ptr(row_ptr), _ptr(off), ctypes.byref(tot)))
        scol = torch.empty(tot.value, dtype=torch.int32, device=dev)
        sval = torch.empty((len(ops), tot.value), dtype=torch.float64, device=dev)
        cfg.sell_slice_off, cfg.sell_col, cfg.sell_val, cfg.sell_nnz = _ptr(off), _ptr(scol), _ptr(sval), tot.value
        sells = [WeightsSELL(off, scol, sval[i], (ne, ns), ctx) for i in range(len(ops))]
    st = _native.BuildStats() if stats is None else stats
    ctx.check(ctx.lib.rbf_build(ctx.h, ctypes.byref(cfg), _ptr(d), ns, _ptr(q), ne, _ptr(a), k,
                                ctypes.byref(hs) if hs else None, _ptr(row_ptr), _ptr(col), _ptr(val),
                                _ptr(status), ctypes.byref(st)))
    Ws = [WeightsCSR(row_ptr, col, val[i], (ne, ns), ctx, sell=sells[i]) for i in range(len(ops))]
    if return_status:
        return Ws, status
    return Ws


def build_weights_backward(ops, data, eval_points, adjl, basis, row_ptr, dW, *, ctx=None, flags=0,
                           precision="fp64", tol=0.0):
    """Gradients (ddata, deval) of L = sum(dW * val) for the build
    build_weights(ops, data, eval_points, adjl, basis, flags=flags) whose CSR row_ptr is
    given, dW shaped like its values (len(ops), nnz).  The pullback of _build_weights
    (src/solve/ad_shared.jl:63-157, src/solve/backward.jl:31-222); eval_points None means
    the data points, whose full gradient is then ddata + deval.  PHS 1/3/5/7; the identity,
    first partials and the Laplacian; interior stencils.  precision "fp64" solves each stencil
    in FP64; "fp32_refined" refines an FP32 factorisation to tol (default 1e-11) with the FP64
    solve as fallback."""
    torch = _torch()
    d = _points(data)
    q = None if eval_points is None else _points(eval_points, "eval_points")
    ns, dim = d.shape
    ne = ns if q is None else q.shape[0]
    ctx = ctx or Context.default(_device_of(d, adjl, dW))
    dev = torch.device("cuda", ctx.device)
    a = adjl.to(torch.int32).contiguous() if _is_torch(adjl) else \
        np.ascontiguousarray(np.asarray(adjl, dtype=np.int32))
    if a.ndim != 2 or a.shape[0] != ne:
        raise DimensionMismatch("adjl must be an (N_eval, k) array of 0-based data indices")
    k = int(a.shape[1])
    g = dW.to(torch.float64).contiguous() if _is_torch(dW) else np.ascontiguousarray(np.asarray(dW, np.float64))
    if g.ndim == 1:
        g = g.reshape(1, -1)
    if g.shape[0] != len(ops) or g.shape[1] != ne * k:
        raise DimensionMismatch("dW must be shaped (number of operators, nnz) with nnz = N_eval * k")
    cfg = _native.BuildCfg()
    cfg.dim, cfg.phs, cfg.poly_deg, cfg.nops = dim, basis.order, basis.poly_deg, len(ops)
    for i, (c, od) in enumerate(ops):
        cfg.op_code[i] = c
        cfg.op_dim[i] = od
    cfg.flags = flags
    cfg.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    cfg.tol = tol
    ddata = torch.empty((ns, dim), dtype=torch.float64, device=dev)
    deval = torch.empty((ne, dim), dtype=torch.float64, device=dev)
    ctx.check(ctx.lib.rbf_build_backward(ctx.h, ctypes.byref(cfg), _ptr(d), ns, _ptr(q), ne, _ptr(a), k,
                                         _ptr(row_ptr), _ptr(g), _ptr(ddata), _ptr(deval)))
    return ddata, deval


def build_weights_differentiable(ops, data, eval_points, adjl, basis, *, ctx=None, flags=0, precision="fp64"):
    """build_weights as a torch autograd function of the point positions (the rrule of
    _build_weights, src/solve/ad_shared.jl:130-157): returns (row_ptr, col, val) with
    val (len(ops), nnz) differentiable with respect to data and eval_points (CUDA float64
    tensors).  eval_points None evaluates at the data points."""
    torch = _torch()

    class _BuildFn(torch.autograd.Function):
        @staticmethod
        def forward(fctx, x, y):
            Ws = build_weights(ops, x.detach(), None if y is None else y.detach(), adjl, basis, ctx=ctx,
                               flags=flags, precision=precision)
            val = torch.stack([W.val for W in Ws])
            fctx.save_for_backward(x, y if y is not None else x)
            fctx.row_ptr = Ws[0].row_ptr
            fctx.same = y is None
            fctx.mark_non_differentiable(Ws[0].row_ptr, Ws[0].col)
            return Ws[0].row_ptr, Ws[0].col, val

        @staticmethod
        def backward(fctx, _g_rp, _g_col, g_val):
            x, y = fctx.saved_tensors
            gd, ge = build_weights_backward(ops, x.detach(), None if fctx.same else y.detach(), adjl, basis,
                                            fctx.row_ptr, g_val.contiguous(), ctx=ctx, flags=flags,
                                            precision=precision)
            if fctx.same:
                return gd + ge, None
            return gd, ge

    x = data if _is_torch(data) else torch.as_tensor(np.asarray(data, np.float64))
    return _BuildFn.apply(x, eval_points)


class Interpolator:
    """Global RBF interpolant, Interpolator(x, y, basis=PHS()) (src/interpolation.jl:22-37):
    the collocation matrix of all points is assembled, factorised (rook Bunch-Kaufman) and
    solved on the GPU.  Calling it evaluates at one point (a length-dim vector: a float) or
    at many (an (m, dim) array: an array of m values) (src/interpolation.jl:39-52)."""

    def __init__(self, x, y, basis=None, *, ctx: Context | None = None):
        torch = _torch()
        basis = basis if basis is not None else PHS()
        d = _points(x, "x")
        n, dim = d.shape
        yy = y.to(torch.float64).contiguous() if _is_torch(y) else np.ascontiguousarray(np.asarray(y, np.float64))
        if yy.ndim != 1 or yy.shape[0] != n:
            raise DimensionMismatch("y must hold one value per point")
        self.ctx = ctx or Context.default(_device_of(d, yy))
        dev = torch.device("cuda", self.ctx.device)
        self.x = _to_device(d, self.ctx)
        self.y = y
        self.rbf_basis = basis
        self.dim = dim
        nmon = math.comb(dim + basis.poly_deg, dim) if basis.poly_deg >= 0 else 0
        coef = torch.empty(n + nmon, dtype=torch.float64, device=dev)
        self.ctx.check(self.ctx.lib.rbf_interp_fit(self.ctx.h, dim, basis.order, basis.poly_deg, _ptr(self.x), n,
                                                   _ptr(_to_device(yy, self.ctx)), _ptr(coef)))
        self.coef = coef
        self.rbf_weights = coef[:n]
        self.monomial_weights = coef[n:]
        self._in_type = "torch.Tensor" if _is_torch(x) else "numpy.ndarray"
        self._out_type = "torch.float64" if _is_torch(y) else "float64"

    def __call__(self, xe):
        torch = _torch()
        single = False
        if _is_torch(xe):
            q = xe.to(torch.float64)
        else:
            q = np.asarray(xe, np.float64)
        if q.ndim == 1:
            if q.shape[0] != self.dim:
                raise DimensionMismatch("point dimension differs from the interpolator's")
            q = q.reshape(1, -1)
            single = True
        if q.ndim != 2 or q.shape[1] != self.dim:
            raise DimensionMismatch("points must be (m, dim)")
        qd = _to_device(q, self.ctx)
        m = qd.shape[0]
        out = torch.empty(m, dtype=torch.float64, device=qd.device)
        self.ctx.check(self.ctx.lib.rbf_interp_eval(self.ctx.h, self.dim, self.rbf_basis.order,
                                                    self.rbf_basis.poly_deg, _ptr(self.x), self.x.shape[0],
                                                    _ptr(self.coef), _ptr(qd), m, _ptr(out)))
        if single:
            return float(out[0])
        if _is_torch(xe):
            return out if xe.is_cuda else out.cpu()
        return out.cpu().numpy()

    def __repr__(self):
        sup = {1: "¹", 3: "³", 5: "⁵", 7: "⁷"}[self.rbf_basis.order]
        return ("Interpolator\n"
                f"├─Input type: {self._in_type} (dim {self.dim})\n"
                f"├─Output type: {self._out_type}\n"
                f"├─Number of points: {self.x.shape[0]}\n"
                f"└─Basis: Polyharmonic spline (r{sup}) with degree {self.rbf_basis.poly_deg} Monomial")


def sytrf_rook(A, *, ctx: Context | None = None):
    """bunchkaufman!(Symmetric(A, :U), true) on the GPU: (factors, ipiv, info) of the dense
    symmetric matrix A (its upper triangle is read), LAPACK dsytrf_rook's pivots and
    arithmetic; the factor columns carry the later interchanges (dsyconvf_rook form)."""
    torch = _torch()
    ctx = ctx or Context.default(_device_of(A))
    F = _to_device(A, ctx).t().contiguous()  # column-major storage of A
    n = F.shape[0]
    ipiv = torch.empty(n, dtype=torch.int32, device=F.device)
    info = ctypes.c_int64(0)
    ctx.check(ctx.lib.rbf_sytrf_rook(ctx.h, n, _ptr(F), n, _ptr(ipiv), ctypes.byref(info)))
    return F.t(), ipiv, int(info.value)


def sytrs_rook(F, ipiv, b, *, ctx: Context | None = None):
    """Solve A x = b with the factors of sytrf_rook (b: n or (n, nrhs))."""
    torch = _torch()
    ctx = ctx or Context.default(_device_of(F))
    Fc = F.t().contiguous()
    B = _to_device(b, ctx)
    one = B.ndim == 1
    Bc = B.reshape(B.shape[0], -1).t().contiguous()  # column-major right-hand sides
    n = Fc.shape[0]
    ctx.check(ctx.lib.rbf_sytrs_rook(ctx.h, n, Bc.shape[0], _ptr(Fc), n, _ptr(ipiv.to(torch.int32).contiguous()),
                                     _ptr(Bc), n))
    return Bc[0] if one else Bc.t()


def apply_differentiable(W, x, val=None):
    """y = W x as a torch autograd function of the field x (n, or (n, nf)) and of the values
    `val` (W's values by default; pass the differentiable values of
    build_weights_differentiable to reach the point positions).  The backward applies W^T to
    the cotangent through the library (the transposed CSR from rbf_csr_to_csc, then the same
    apply) and gives the values' cotangent g[row] x[col] -- the rules the reference's AD
    extensions define for op(x) (ext/RadialBasisFunctionsMooncakeExt / EnzymeExt, on
    _eval_op, src/operators/operators.jl:217-218)."""
    torch = _torch()

    class _ApplyFn(torch.autograd.Function):
        @staticmethod
        def forward(fctx, v, xx):
            Wv = WeightsCSR(W.row_ptr, W.col, v.detach().contiguous(), W.shape, W.ctx)
            fctx.save_for_backward(v, xx)
            return Wv.apply(xx.detach().contiguous())

        @staticmethod
        def backward(fctx, g):
            v, xx = fctx.saved_tensors
            ne, ns = W.shape
            g = g.contiguous()
            dv = dx = None
            if fctx.needs_input_grad[1]:
                cp, rw, vv = WeightsCSR(W.row_ptr, W.col, v.detach().contiguous(), W.shape, W.ctx).to_csc()
                dx = WeightsCSR(cp, rw, vv, (ns, ne), W.ctx).apply(g)
            if fctx.needs_input_grad[0]:
                rows = torch.repeat_interleave(torch.arange(ne, device=g.device), W.row_ptr[1:] - W.row_ptr[:-1])
                cols = W.col.long()
                prod = g[rows] * xx.detach()[cols]
                dv = prod if prod.ndim == 1 else prod.sum(-1)
            return dv, dx

    v = W.val if val is None else val
    return _ApplyFn.apply(v, x)


def reorder_points(data, k=None, ctx=None):
    """reorder_points!(x, k) (src/utils.jl:45-55): returns (perm, x[perm]) with the points
    ordered along a Morton curve for locality (0-based perm; the reference's SymRCM order
    is another locality order with the same contract).  k is accepted for the reference's
    signature and not needed."""
    torch = _torch()
    d = _points(data)
    n, dim = d.shape
    ctx = ctx or Context.default(_device_of(d))
    if _is_torch(d) and d.is_cuda:
        perm = torch.empty(n, dtype=torch.int32, device=d.device)
        out = torch.empty_like(d)
    elif _is_torch(d):
        perm = torch.empty(n, dtype=torch.int32)
        out = torch.empty_like(d)
    else:
        perm = np.empty(n, dtype=np.int32)
        out = np.empty_like(d)
    ctx.check(ctx.lib.rbf_reorder_points(ctx.h, _ptr(d), n, dim, _ptr(perm), _ptr(out)))
    return perm, out


# ------------------------------------------------------------------------------ batched (uneven) build
def ragged_stencils(adjl, k_per):
    """Ragged adjacency (adj_ptr, adj_idx) keeping the k_per[e] nearest of each row of a
    uniform neighbour list adjl (rows sorted by distance, as find_neighbors returns them)."""
    torch = _torch()
    a = adjl if _is_torch(adjl) else torch.from_numpy(np.ascontiguousarray(adjl, dtype=np.int32))
    kp = k_per if _is_torch(k_per) else torch.as_tensor(np.asarray(k_per), dtype=torch.int64)
    kp = kp.to(a.device, torch.int64)
    if kp.numel() != a.shape[0] or int(kp.min()) < 1 or int(kp.max()) > a.shape[1]:
        raise ValueError("k_per must hold one stencil size in 1..k per row of adjl")
    keep = torch.arange(a.shape[1], device=a.device)[None, :] < kp[:, None]
    adj_idx = a[keep].to(torch.int32).contiguous()
    adj_ptr = torch.zeros(a.shape[0] + 1, dtype=torch.int64, device=a.device)
    adj_ptr[1:] = torch.cumsum(kp, 0)
    return adj_ptr, adj_idx


def build_weights_batched(ops, data, eval_points, adj_ptr, adj_idx, basis, hermite=None, precision="fp64", *,
                          poly_deg=None, tune=1, ctx=None, refine_steps=0, tol=0.0, return_status=False,
                          stats=None, flags=0, normal_dof=False):
    """Weights of `ops` on ragged stencils (the neighbours of eval point e are
    adj_idx[adj_ptr[e]:adj_ptr[e+1]]), with an optional polynomial degree per stencil
    (poly_deg, int8 array; basis.poly_deg otherwise), all in one persistent launch binned by
    system size with autotuned tile shapes (tune: 0 cached/heuristic, 1 tune new classes,
    2 re-tune).  Returns a list of WeightsCSR like build_weights.

    normal_dof (with a Hermite boundary; no counterpart in the reference): every
    Neumann/Robin stencil point carries u and du/dn as unknowns, so a stencil with m such
    neighbours solves a (k + m + nmon) system (binned by that size).  The operators then
    have ns + nb columns, applied to [u; du/dn at the boundary points in boundary order];
    Dirichlet eval rows stay identity rows and every other row takes the operator itself."""
    torch = _torch()
    d = _points(data)
    q = d if eval_points is None else _points(eval_points, "eval_points")
    ns, dim = d.shape
    ne = q.shape[0]
    ctx = ctx or Context.default(_device_of(d, q, adj_idx))
    dev = torch.device("cuda", ctx.device)

    def arr(x, dtype_t, dtype_n):
        if _is_torch(x):
            return x.to(dtype_t).contiguous()
        return np.ascontiguousarray(np.asarray(x, dtype=dtype_n))

    ap = arr(adj_ptr, torch.int64, np.int64)
    ai = arr(adj_idx, torch.int32, np.int32)
    if ap.shape[0] != ne + 1:
        raise DimensionMismatch("adj_ptr must have N_eval + 1 entries")
    pd = None if poly_deg is None else arr(poly_deg, torch.int8, np.int8)
    if pd is not None and pd.shape[0] != ne:
        raise DimensionMismatch("poly_deg must have one entry per eval point")
    cfg = _native.BuildCfg()
    cfg.dim, cfg.phs, cfg.poly_deg, cfg.nops = dim, basis.order, basis.poly_deg, len(ops)
    for i, (c, od) in enumerate(ops):
        cfg.op_code[i] = c
        cfg.op_dim[i] = od
    cfg.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    cfg.refine_steps = refine_steps
    cfg.tol = tol
    cfg.flags = flags | (_native.FLAG_NORMAL_DOF if normal_dof else 0)
    herm = _hermite_arrays(hermite, ns, dim)
    hs = None
    nb = 0
    if herm is not None:
        isb, al, be, nr = herm
        hs = _native.Hermite(isb.ctypes.data, al.ctypes.data, be.ctypes.data, nr.ctypes.data, len(al))
        nb = len(al)
    row_ptr = torch.empty(ne + 1, dtype=torch.int64, device=dev)
    nnz = ctypes.c_int64(0)
    if normal_dof:
        ctx.check(ctx.lib.rbf_build_count_normal_dof(ctx.h, ns, ne, _ptr(ap), _ptr(ai),
                                                     ctypes.byref(hs) if hs else None, _ptr(row_ptr),
                                                     ctypes.byref(nnz)))
    else:
        ctx.check(ctx.lib.rbf_build_count_ragged(ctx.h, ns, ne, _ptr(ap), ctypes.byref(hs) if hs else None,
                                                 _ptr(row_ptr), ctypes.byref(nnz)))
    col = torch.empty(nnz.value, dtype=torch.int32, device=dev)
    val = torch.empty((len(ops), nnz.value), dtype=torch.float64, device=dev)
    status = torch.empty(ne, dtype=torch.int8, device=dev) if return_status else None
    st = _native.BuildStats() if stats is None else stats
    ctx.check(ctx.lib.rbf_build_batched(ctx.h, ctypes.byref(cfg), _ptr(d), ns, _ptr(q), ne, _ptr(ap), _ptr(ai),
                                        _ptr(pd), ctypes.byref(hs) if hs else None, _ptr(row_ptr), _ptr(col),
                                        _ptr(val), _ptr(status), ctypes.byref(st), int(tune)))
    ncols = ns + nb if normal_dof else ns
    Ws = [WeightsCSR(row_ptr, col, val[i], (ne, ncols), ctx) for i in range(len(ops))]
    if return_status:
        return Ws, status
    return Ws


class BuildApplyGraph:
    """Weight build on fixed stencils followed by y = W x, captured once in a CUDA graph
    (rbf_plan_*).  data/eval_points/x are device tensors the graph reads in place: write new
    coordinates or a new field into them, then call replay() -- one graph launch on torch's
    current stream rebuilds the weights (into .weights) and applies them (into .y)."""

    def __init__(self, op, data, eval_points, adjl, basis, x, precision="fp64", op_index=0, ctx=None,
                 refine_steps=0, tol=0.0):
        torch = _torch()
        ops = [op] if isinstance(op, tuple) else list(op)
        self.data = data
        self.eval = data if eval_points is None else eval_points
        for t, nm in ((data, "data"), (self.eval, "eval_points"), (x, "x")):
            if not (_is_torch(t) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError(f"{nm} must be a contiguous float64 CUDA tensor (the graph reads it in place)")
        if not (_is_torch(adjl) and adjl.is_cuda and adjl.dtype == torch.int32 and adjl.is_contiguous()):
            raise ValueError("adjl must be a contiguous int32 CUDA tensor")
        ns, dim = data.shape
        ne, k = adjl.shape
        self.ctx = ctx or Context.default(data.device.index or 0)
        dev = data.device
        self.x = x
        self.adjl = adjl
        self.row_ptr = torch.empty(ne + 1, dtype=torch.int64, device=dev)
        nnz = ctypes.c_int64(0)
        self.ctx.check(self.ctx.lib.rbf_build_count(self.ctx.h, ns, ne, k, None, _ptr(self.row_ptr), ctypes.byref(nnz)))
        self.col = torch.empty(nnz.value, dtype=torch.int32, device=dev)
        self.val = torch.empty((len(ops), nnz.value), dtype=torch.float64, device=dev)
        self.y = torch.empty(ne, dtype=torch.float64, device=dev)
        cfg = _native.BuildCfg()
        cfg.dim, cfg.phs, cfg.poly_deg, cfg.nops = dim, basis.order, basis.poly_deg, len(ops)
        for i, (c, od) in enumerate(ops):
            cfg.op_code[i] = c
            cfg.op_dim[i] = od
        cfg.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        cfg.refine_steps = refine_steps
        cfg.tol = tol
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.rbf_plan_create(self.ctx.h, ctypes.byref(cfg), _ptr(data), ns, _ptr(self.eval), ne,
                                                    _ptr(adjl), k, _ptr(self.row_ptr), _ptr(self.col), _ptr(self.val),
                                                    op_index, _ptr(x), _ptr(self.y), ctypes.byref(h)))
        self.plan = h
        self.weights = [WeightsCSR(self.row_ptr, self.col, self.val[i], (ne, ns), self.ctx) for i in range(len(ops))]

    def replay(self):
        self.ctx.h  # bind the plan's context to torch's current stream
        self.ctx.check(self.ctx.lib.rbf_plan_launch(self.plan))
        return self.y

    def counters(self):
        s, f, r = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
        self.ctx.check(self.ctx.lib.rbf_plan_counters(self.plan, ctypes.byref(s), ctypes.byref(f), ctypes.byref(r)))
        return {"singular": s.value, "fallback": f.value, "residuals": r.value}

    def __del__(self):
        try:
            if getattr(self, "plan", None):
                self.ctx.lib.rbf_plan_destroy(self.plan)
                self.plan = None
        except Exception:
            pass


def tuning_report(ctx=None):
    """The batched build's tuning table of a context: one line per size class."""
    ctx = ctx or Context.default(0)
    buf = ctypes.create_string_buffer(1 << 16)
    ctx.check(ctx.lib.rbf_tuning_report(ctx.handle, buf, len(buf)))
    return buf.value.decode()


# ------------------------------------------------------------------------------ operator object
class RadialBasisOperator:
    """Operator of data with a radial basis and monomial augmentation (operators.jl:50-143).

    weights are device CSR matrices (a tuple for Jacobian / Operators)."""

    def __init__(self, L: _Op, data, eval_points=None, basis=None, k: int | None = None, adjl=None,
                 hermite=None, precision: str = "fp64", ctx: Context | None = None):
        self.L = L
        data = _points(data)
        ev = None if eval_points is None else _points(eval_points, "eval_points")
        self.ctx = ctx or Context.default(_device_of(data, ev))
        # points live on the GPU for the operator's lifetime (one host->device copy)
        self.data = _to_device(data, self.ctx)
        self.eval_points = self.data if ev is None else _to_device(ev, self.ctx)
        self.basis = basis if basis is not None else PHS(3, poly_deg=2)
        self.k = k if k is not None else autoselect_k(self.data, self.basis)
        self.adjl = adjl if adjl is not None else find_neighbors(self.data, self.eval_points, self.k, ctx=self.ctx)
        self.hermite = hermite
        self.precision = precision
        self.weights = None
        self.valid_cache = False
        self.update_weights()

    @property
    def dim(self):
        return self.data.shape[1]

    def _build(self):
        ops = self.L.ops(self.dim)
        Ws = build_weights(ops, self.data, self.eval_points, self.adjl, self.basis, self.hermite, self.precision,
                           ctx=self.ctx)
        if isinstance(self.L, Directional):
            return _directional_weights(Ws, self.L.v, self.dim)
        return Ws[0] if (len(Ws) == 1 and self.L.rank == 0) else tuple(Ws)

    # ---- operator algebra (src/operators/operator_algebra.jl:245-295): the weights of the
    # result are combined on the device; the result rebuilds its parts when updated
    def _check_compatible(self, other):
        torch = _torch()
        if not isinstance(other, RadialBasisOperator):
            return NotImplemented
        if self.L.rank != other.L.rank:
            raise ValueError(f"Cannot combine operators with different output ranks: {self.L!r} (rank "
                             f"{self.L.rank}) and {other.L!r} (rank {other.L.rank})")
        if self.data.shape != other.data.shape or not torch.allclose(self.data, other.data):
            raise ValueError("Can not add operators that were not built with the same data.")
        a1, a2 = torch.as_tensor(self.adjl), torch.as_tensor(other.adjl)
        if a1.shape != a2.shape or not torch.equal(a1.to(a2.device, torch.int64), a2.to(torch.int64)):
            raise ValueError("Can not add operators that do not have the same stencils.")

    def _combined(self, other, alpha, beta, desc):
        def combine():
            for op in (self, other) if other is not None else (self,):
                if not op.valid_cache:
                    op.update_weights()
            if other is None:
                return _map_weights(lambda w: _axpby(w, alpha, None, 0.0), self.weights)
            return _map_weights(lambda w1, w2: _axpby(w1, alpha, w2, beta), self.weights, other.weights)
        return _DerivedOperator(_Combined(desc, self.L.rank), self, combine)

    def __add__(self, other):
        if self._check_compatible(other) is NotImplemented:
            return NotImplemented
        return self._combined(other, 1.0, 1.0, f"{self.L!r} + {other.L!r}")

    def __sub__(self, other):
        if self._check_compatible(other) is NotImplemented:
            return NotImplemented
        return self._combined(other, 1.0, -1.0, f"{self.L!r} - {other.L!r}")

    def __mul__(self, alpha):
        if not isinstance(alpha, (int, float, np.number)):
            return NotImplemented
        return self._combined(None, float(alpha), 0.0, f"{float(alpha)} * {self.L!r}")

    __rmul__ = __mul__

    def __truediv__(self, alpha):
        if not isinstance(alpha, (int, float, np.number)):
            return NotImplemented
        return self._combined(None, 1.0 / float(alpha), 0.0, f"{self.L!r} / {float(alpha)}")

    def __neg__(self):
        return self._combined(None, -1.0, 0.0, f"-{self.L!r}")

    def update_weights(self):
        """Rebuild the weights from data / eval_points (operators.jl:589-602)."""
        self.weights = self._build()
        self.valid_cache = True

    def invalidate_cache(self):
        self.valid_cache = False

    def __call__(self, x, y=None):
        if not self.valid_cache:
            self.update_weights()
        if isinstance(self.weights, tuple):
            outs = [W.apply(x) for W in self.weights]
            if _is_torch(outs[0]):
                res = _torch().stack(outs, dim=-1)
            else:
                res = np.stack(outs, axis=-1)
            if y is not None:
                y[...] = res
                return y
            return res
        return self.weights.apply(x, y)

    @property
    def shape(self):
        return (self.eval_points.shape[0], self.data.shape[0])

    def __repr__(self):
        return f"RadialBasisOperator\n├─Operator: {self.L!r}\n├─Data type: float64\n├─Number of weights: " \
               f"{self.weights.nnz if isinstance(self.weights, WeightsCSR) else self.weights[0].nnz}\n" \
               f"└─Basis: {self.basis!r}"


class _DerivedOperator(RadialBasisOperator):
    """An operator whose weights come from other built operators (sum, difference, scaling);
    it shares their points and stencils and rebuilds them when updated."""

    def __init__(self, L, template: RadialBasisOperator, combine):
        self.L = L
        self._combine = combine
        self.ctx, self.data, self.eval_points = template.ctx, template.data, template.eval_points
        self.basis, self.k, self.adjl = template.basis, template.k, template.adjl
        self.hermite, self.precision = template.hermite, template.precision
        self.weights = None
        self.valid_cache = False
        self.update_weights()

    def _build(self):
        return self._combine()


def _map_weights(fn, *ws):
    if isinstance(ws[0], tuple):
        return tuple(fn(*parts) for parts in zip(*ws))
    return fn(*ws)


def _axpby(W1: WeightsCSR, alpha, W2, beta):
    """alpha * W1 + beta * W2 on the device (W2 of the same structure, or None)."""
    torch = _torch()
    out = torch.empty_like(W1.val)
    ctx = W1.ctx
    ctx.check(ctx.lib.rbf_weights_axpby(ctx.h, W1.nnz, float(alpha), _ptr(W1.val), float(beta),
                                        _ptr(W2.val) if W2 is not None else None, _ptr(out)))
    return WeightsCSR(W1.row_ptr, W1.col, out, W1.shape, ctx)


def _directional_weights(Ws, v, dim):
    """sum_i v_i W_i (directional.jl:69-82): v of length dim, or one direction per row."""
    torch = _torch()
    W0 = Ws[0]
    ne = W0.shape[0]
    vt = torch.as_tensor(v, dtype=torch.float64).to(W0.val.device)
    if vt.ndim == 1 and vt.shape[0] == dim:
        per_row = 0
    elif vt.ndim == 2 and vt.shape == (ne, dim):
        per_row = 1
    elif vt.ndim == 1 and vt.shape[0] == ne * dim:
        vt, per_row = vt.reshape(ne, dim), 1
    else:
        raise ValueError(f"Direction vector length {tuple(vt.shape)} must equal dimension {dim} or data length {ne}")
    vt = vt.contiguous()
    nnz = W0.nnz
    base = W0.val
    if not all(W.val.data_ptr() == base.data_ptr() + 8 * i * nnz for i, W in enumerate(Ws)):
        base = torch.stack([W.val for W in Ws])
    out = torch.empty_like(W0.val)
    ctx = W0.ctx
    ctx.check(ctx.lib.rbf_weights_directional(ctx.h, ne, _ptr(W0.row_ptr), dim, _ptr(base), nnz, _ptr(vt), per_row,
                                              _ptr(out)))
    return WeightsCSR(W0.row_ptr, W0.col, out, W0.shape, ctx)


def weights(op: RadialBasisOperator):
    """operators.jl:569-572"""
    if not op.valid_cache:
        op.update_weights()
    return op.weights


def update_weights(op: RadialBasisOperator):
    op.update_weights()


def mul(y, op: RadialBasisOperator, x, alpha: float = 1.0, beta: float = 0.0):
    """y = alpha * op * x + beta * y (mul!, operators.jl:529-542; rank-0 operators only)."""
    if not op.valid_cache:
        op.update_weights()
    if isinstance(op.weights, tuple):
        raise ValueError("mul is only defined for rank-0 operators with scalar weights")
    return op.weights.apply(x, y, alpha, beta)


# ------------------------------------------------------------------------------ front ends
def laplacian(data, basis=None, **kw):
    """laplacian(data; basis=PHS(3; poly_deg=2), eval_points, k, adjl, hermite)"""
    return RadialBasisOperator(Laplacian(), data, basis=basis, **kw)


def partial(data, order: int, dim: int, basis=None, **kw):
    """partial(data, order, dim; ...) with dim 1-based as in the reference."""
    return RadialBasisOperator(Partial(order, dim), data, basis=basis, **kw)


def jacobian(data, basis=None, **kw):
    d = _points(data)
    return RadialBasisOperator(Jacobian(d.shape[1]), d, basis=basis, **kw)


def gradient(data, basis=None, **kw):
    """gradient(data; ...) = jacobian(data; ...) (gradient.jl:32)."""
    return jacobian(data, basis=basis, **kw)


def directional(data, v, basis=None, **kw):
    """directional(data, v; basis, eval_points, k, adjl, hermite) (directional.jl:37-40): the
    directional derivative ∇f⋅v with a constant direction or one direction per point."""
    return RadialBasisOperator(Directional(v), data, basis=basis, **kw)


def regrid(data, eval_points, basis=None, **kw):
    """regrid(data, eval_points; basis, k, adjl) (regridding.jl:38-47)."""
    return RadialBasisOperator(Regrid(), data, eval_points=eval_points, basis=basis, **kw)


# ------------------------------------------------------------------------------ checkpoint / resume
from .checkpoint import load_operator, load_weights, save_operator, save_weights  # noqa: E402
