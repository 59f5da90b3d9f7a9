"""rbf_build_csr / rbf_csr_free: the boundary form that returns its own sparse matrix (the
library allocates the CSR arrays, as _build_weights returns its SparseMatrixCSC,
src/solve/api.jl:26-35).  Its arrays equal those of the two-call build (rbf_build_count +
rbf_build into caller buffers) bit for bit; on an error nothing stays allocated."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    return g.load_package()


class _Dev:
    """A device array owned by the library, viewed by torch without a copy."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3}


def _cfg(pkg, ops, dim, phs=3, deg=2):
    n = pkg._native
    cfg = n.BuildCfg()
    cfg.dim, cfg.phs, cfg.poly_deg, cfg.nops = dim, phs, deg, len(ops)
    for i, (c, od) in enumerate(ops):
        cfg.op_code[i] = c
        cfg.op_dim[i] = od
    cfg.precision = pkg.PRECISIONS["fp64"]
    return cfg


@pytest.mark.parametrize("boundary", [False, True])
def test_owned_csr_equals_two_call_build(pkg, boundary):
    rng = np.random.default_rng(21)
    X = rng.uniform(0.0, 1.0, (3000, 3))
    herm, hs = None, None
    if boundary:  # Dirichlet rows on x = 1: one entry per row, so nnz < ne * k
        hi = X[:, 0] > 0.97
        X[hi, 0] = 1.0
        herm = dict(is_boundary=hi, bc=[pkg.BoundaryCondition(1.0, 0.0)] * int(hi.sum()),
                    normals=np.tile([1.0, 0.0, 0.0], (int(hi.sum()), 1)))
    Xd = torch.from_numpy(X).cuda()
    adjl = pkg.find_neighbors(Xd, k=30)
    ops = [(pkg.OP_LAPLACIAN, 0), (pkg.OP_PARTIAL1, 1)]
    Ws = pkg.build_weights(ops, Xd, None, adjl, pkg.PHS(3, poly_deg=2), herm)
    ctx = pkg.Context.default()
    keep = None
    if herm is not None:
        keep = pkg._hermite_arrays(herm, len(X), 3)
        isb, al, be, nr = keep
        hs = pkg._native.Hermite(isb.ctypes.data, al.ctypes.data, be.ctypes.data, nr.ctypes.data, len(al))
    cfg = _cfg(pkg, ops, 3)
    out = pkg._native.Csr()
    a = adjl.to(torch.int32).contiguous()
    ctx.check(ctx.lib.rbf_build_csr(ctx.h, ctypes.byref(cfg), Xd.data_ptr(), len(X), Xd.data_ptr(), len(X), a.data_ptr(),
                                    30, ctypes.byref(hs) if hs else None, None, None, ctypes.byref(out)))
    try:
        assert (out.ne, out.ns, out.nnz, out.nops) == (len(X), len(X), Ws[0].nnz, 2)
        if boundary:
            assert out.nnz < len(X) * 30
        rp = torch.as_tensor(_Dev(out.row_ptr, out.ne + 1, "<i8"), device="cuda")
        col = torch.as_tensor(_Dev(out.col, out.nnz, "<i4"), device="cuda")
        val = torch.as_tensor(_Dev(out.val, 2 * out.nnz, "<f8"), device="cuda")
        assert torch.equal(rp, Ws[0].row_ptr) and torch.equal(col, Ws[0].col)
        assert torch.equal(val[:out.nnz], Ws[0].val) and torch.equal(val[out.nnz:], Ws[1].val)
    finally:
        ctx.check(ctx.lib.rbf_csr_free(ctx.h, ctypes.byref(out)))
    assert out.nnz == 0 and not out.row_ptr and not out.col and not out.val


def test_owned_csr_error_leaves_nothing(pkg):
    X = torch.rand((500, 2), dtype=torch.float64, device="cuda")
    adjl = pkg.find_neighbors(X, k=12).to(torch.int32).contiguous()
    ctx = pkg.Context.default()
    cfg = _cfg(pkg, [(pkg.OP_LAPLACIAN, 0)], 2, phs=2)  # PHS order 2 does not exist
    out = pkg._native.Csr()
    st = ctx.lib.rbf_build_csr(ctx.h, ctypes.byref(cfg), X.data_ptr(), 500, X.data_ptr(), 500, adjl.data_ptr(), 12,
                               None, None, None, ctypes.byref(out))
    assert st == -1  # RBF_ERR_ARGUMENT, the reference's ArgumentError
    assert b"n must be 1, 3, 5, or 7" in ctx.lib.rbf_last_error(ctx.handle)
    assert out.nnz == 0 and not out.row_ptr and not out.col and not out.val
