"""rbf_spmm_noalloc: the apply for callers that cannot allocate device memory.

It must give what rbf_spmm gives (same tolerance as the other apply tests), twice in a row
on the shared fixed scratch array, and refuse operands larger than that array.  The file
name makes pytest collect it last."""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

APPLY_TOL = 1e-10
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def setup():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    pkg = g.load_package()
    z = np.load(os.path.join(GOLD, "oracle_small_lap2d.npz"))
    X = torch.from_numpy(z["points"]).cuda()
    op = pkg.laplacian(X, k=20, adjl=torch.from_numpy(z["adjl"]).cuda())
    return pkg, op.weights


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _apply(pkg, W, fn, Xcm, Ycm, nf, alpha, beta):
    ctx = W.ctx
    ne, ns = W.shape
    st = fn(ctx.handle, ne, ns, _p(W.row_ptr), _p(W.col), _p(W.val), nf, 0, _p(Xcm), ns, alpha, beta, _p(Ycm), ne)
    return st


def test_noalloc_matches_allocating_apply_twice(setup):
    pkg, W = setup
    L = W.ctx.lib
    ne, ns = W.shape
    nf = 7
    gen = torch.Generator(device="cuda").manual_seed(3)
    for call in range(2):  # the second call reuses the scratch left by the first
        Xcm = torch.randn((nf, ns), generator=gen, dtype=torch.float64, device="cuda")  # column-major fields
        Y0 = torch.randn((nf, ne), generator=gen, dtype=torch.float64, device="cuda")
        Yref, Ynoa = Y0.clone(), Y0.clone()
        alpha, beta = 1.5, (0.0 if call == 0 else -0.25)
        assert _apply(pkg, W, L.rbf_spmm, Xcm, Yref, nf, alpha, beta) == 0
        st = _apply(pkg, W, L.rbf_spmm_noalloc, Xcm, Ynoa, nf, alpha, beta)
        assert st == 0, L.rbf_last_error(W.ctx.handle).decode()
        torch.cuda.synchronize()
        scale = float(Yref.abs().max())
        assert float((Ynoa - Yref).abs().max()) <= APPLY_TOL * scale
    # single field needs no scratch and must match as well
    x = torch.randn(ns, generator=gen, dtype=torch.float64, device="cuda")
    y1 = torch.zeros(ne, dtype=torch.float64, device="cuda")
    y2 = torch.zeros(ne, dtype=torch.float64, device="cuda")
    assert _apply(pkg, W, L.rbf_spmm, x, y1, 1, 1.0, 0.0) == 0
    assert _apply(pkg, W, L.rbf_spmm_noalloc, x, y2, 1, 1.0, 0.0) == 0
    assert float((y1 - y2).abs().max()) <= APPLY_TOL * float(y1.abs().max())


def test_noalloc_rejects_oversize_and_host_pointers(setup):
    pkg, W = setup
    L = W.ctx.lib
    ne, ns = W.shape
    nf_big = (4 << 20) // (ns + ne) + 1  # one field more than the fixed scratch holds
    x = torch.zeros((2, ns), dtype=torch.float64, device="cuda")
    y = torch.zeros((2, ne), dtype=torch.float64, device="cuda")
    st = L.rbf_spmm_noalloc(W.ctx.handle, ne, ns, _p(W.row_ptr), _p(W.col), _p(W.val), nf_big, 0, _p(x), ns,
                            1.0, 0.0, _p(y), ne)
    assert st == -1 and b"exceeds the fixed scratch" in L.rbf_last_error(W.ctx.handle)
    xh = np.zeros((2, ns))
    yh = np.zeros((2, ne))
    st = L.rbf_spmm_noalloc(W.ctx.handle, ne, ns, _p(W.row_ptr), _p(W.col), _p(W.val), 2, 0,
                            xh.ctypes.data_as(ctypes.c_void_p), ns, 1.0, 0.0, yh.ctypes.data_as(ctypes.c_void_p), ne)
    assert st == -1 and b"device pointer" in L.rbf_last_error(W.ctx.handle)


def test_noalloc_many_fields_and_interleaved(setup):
    """Past 32 fields the staged apply runs in chunks of 32 over the scratch; the interleaved
    layout needs no staging but takes the same chunked kernel loop.  Both against rbf_spmm,
    two calls in a row each."""
    pkg, W = setup
    L = W.ctx.lib
    ne, ns = W.shape
    gen = torch.Generator(device="cuda").manual_seed(11)
    for call in range(2):
        nf = 40
        Xcm = torch.randn((nf, ns), generator=gen, dtype=torch.float64, device="cuda")
        Y0 = torch.randn((nf, ne), generator=gen, dtype=torch.float64, device="cuda")
        Yref, Ynoa = Y0.clone(), Y0.clone()
        beta = 0.0 if call == 0 else 0.5
        assert _apply(pkg, W, L.rbf_spmm, Xcm, Yref, nf, -0.75, beta) == 0
        assert _apply(pkg, W, L.rbf_spmm_noalloc, Xcm, Ynoa, nf, -0.75, beta) == 0, \
            L.rbf_last_error(W.ctx.handle).decode()
        torch.cuda.synchronize()
        assert float((Ynoa - Yref).abs().max()) <= APPLY_TOL * float(Yref.abs().max())
        nf = 7  # interleaved: field f of point i at X[i * nf + f]
        Xil = torch.randn((ns, nf), generator=gen, dtype=torch.float64, device="cuda")
        Y0 = torch.randn((ne, nf), generator=gen, dtype=torch.float64, device="cuda")
        Yref, Ynoa = Y0.clone(), Y0.clone()
        for fn, Yt in ((L.rbf_spmm, Yref), (L.rbf_spmm_noalloc, Ynoa)):
            st = fn(W.ctx.handle, ne, ns, _p(W.row_ptr), _p(W.col), _p(W.val), nf, 1, _p(Xil), nf, 2.0, beta,
                    _p(Yt), nf)
            assert st == 0, L.rbf_last_error(W.ctx.handle).decode()
        torch.cuda.synchronize()
        assert float((Ynoa - Yref).abs().max()) <= APPLY_TOL * float(Yref.abs().max())


def test_noalloc_operator_without_data_points(setup):
    """An operator with no data points has only empty rows: Y = beta * Y, and the staged
    path must not launch its copy of X (zero blocks)."""
    pkg, W = setup
    L = W.ctx.lib
    ne, nf = 5, 3
    rp = torch.zeros(ne + 1, dtype=torch.int64, device="cuda")
    col = torch.zeros(1, dtype=torch.int32, device="cuda")
    val = torch.zeros(1, dtype=torch.float64, device="cuda")
    x = torch.zeros(1, dtype=torch.float64, device="cuda")
    Y = torch.arange(nf * ne, dtype=torch.float64, device="cuda").reshape(nf, ne)
    Y0 = Y.clone()
    st = L.rbf_spmm_noalloc(W.ctx.handle, ne, 0, _p(rp), _p(col), _p(val), nf, 0, _p(x), 0, 1.0, 0.5, _p(Y), ne)
    assert st == 0, L.rbf_last_error(W.ctx.handle).decode()
    torch.cuda.synchronize()
    assert torch.equal(Y, 0.5 * Y0)
