"""The sliced-ELL copy of an operator (rbf_sell_offsets / rbf_sell_from_csr / the copy the
build writes with cfg.sell_*) and its apply (rbf_spmv_sell): the copy holds exactly the CSR's
entries, and its product equals the CSR product up to summation order, bounded per row by
1e-14 of sum_j |w_j x_j| (the rounding scale of that row)."""
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


def sell_to_rows(S, ne):
    """(columns, values) of every row from the sliced arrays (host)."""
    off = S.slice_off.cpu().numpy()
    col = S.col.cpu().numpy()
    val = S.val.cpu().numpy()
    rows = []
    for r in range(ne):
        s, ln = r // 32, r % 32
        w = (off[s + 1] - off[s]) // 32
        idx = off[s] + 32 * np.arange(w) + ln
        rows.append((col[idx], val[idx]))
    return rows


def csr_rows(W):
    rp = W.row_ptr.cpu().numpy()
    col = W.col.cpu().numpy()
    val = W.val.cpu().numpy()
    return [(col[rp[r]:rp[r + 1]], val[rp[r]:rp[r + 1]]) for r in range(len(rp) - 1)]


def check_same_rows(S, W):
    ne = W.shape[0]
    for (sc, sv), (cc, cv) in zip(sell_to_rows(S, ne), csr_rows(W)):
        n = len(cc)
        assert np.array_equal(sc[:n], cc) and np.array_equal(sv[:n], cv)
        assert (sc[n:] == 0).all() and (sv[n:] == 0.0).all()  # padding


def check_product(W, y, x):
    """y against the host CSR product, per row within 1e-14 * sum |w x|."""
    A = W.to_scipy()
    xs = x.cpu().numpy()
    ref = A @ xs
    scale = abs(A) @ np.abs(xs)
    assert (np.abs(y.cpu().numpy() - ref) <= 1e-14 * scale + 1e-300).all()


def test_from_csr_uniform(pkg):
    rng = np.random.default_rng(11)
    X = torch.from_numpy(rng.uniform(0, 1, (20000, 3))).cuda()
    adjl = pkg.find_neighbors(X, k=30)
    W = pkg.build_weights([(3, 0)], X, None, adjl, pkg.PHS(3, poly_deg=2), precision="fp32_refined")[0]
    S = W.to_sell()
    assert S.col.shape[0] == W.nnz  # equal row lengths: no padding
    check_same_rows(S, W)
    x = torch.sin(4 * X[:, 0]) + X[:, 1] * X[:, 2]
    check_product(W, S.apply(x), x)


def test_build_writes_copy_ragged_and_multi_op(pkg):
    """Hermite build (Dirichlet identity rows of length 1 beside full rows) of the gradient:
    the copy the build writes holds each operator's rows, padded slices included."""
    rng = np.random.default_rng(12)
    m = 70
    g = np.stack(np.meshgrid(np.linspace(0, 1, m), np.linspace(0, 1, m), indexing="ij"), -1).reshape(-1, 2)
    g = g + rng.uniform(-0.2, 0.2, g.shape) / m * ((g > 0) & (g < 1))
    isb = (g[:, 0] == 0) | (g[:, 0] == 1) | (g[:, 1] == 0) | (g[:, 1] == 1)
    bpts = g[isb]
    normals = np.zeros((int(isb.sum()), 2))
    normals[bpts[:, 0] == 0, 0] = -1
    normals[bpts[:, 0] == 1, 0] = 1
    normals[(bpts[:, 1] == 0) & (normals[:, 0] == 0), 1] = -1
    normals[(bpts[:, 1] == 1) & (normals[:, 0] == 0), 1] = 1
    bc = [pkg.Dirichlet() if p[1] > 0.5 else pkg.Neumann() for p in bpts]
    herm = dict(is_boundary=isb, bc=bc, normals=normals)
    X = torch.from_numpy(g).cuda()
    adjl = pkg.find_neighbors(X, k=20)
    Ws = pkg.build_weights([(1, 0), (1, 1)], X, None, adjl, pkg.PHS(3, poly_deg=2), hermite=herm,
                           precision="fp32_refined", sell=True)
    rp = Ws[0].row_ptr.cpu().numpy()
    assert (np.diff(rp) == 1).any() and (np.diff(rp) == 20).any()
    assert Ws[0].sell.col.shape[0] > Ws[0].nnz  # padded slices
    x = torch.cos(3 * X[:, 0]) * X[:, 1]
    for W in Ws:
        check_same_rows(W.sell, W)
        y = W.apply(x)  # single CUDA field: the sliced apply
        check_product(W, y, x)


def test_alpha_beta(pkg):
    rng = np.random.default_rng(13)
    X = torch.from_numpy(rng.uniform(0, 1, (5000, 2))).cuda()
    adjl = pkg.find_neighbors(X, k=20)
    W = pkg.build_weights([(3, 0)], X, None, adjl, pkg.PHS(3, poly_deg=2), sell=True)[0]
    x = torch.exp(X[:, 0]) - X[:, 1]
    y0 = torch.linspace(-1, 1, 5000, dtype=torch.float64, device="cuda")
    y = y0.clone()
    W.sell.apply(x, y, alpha=0.5, beta=-2.0)
    A = W.to_scipy()
    ref = 0.5 * (A @ x.cpu().numpy()) - 2.0 * y0.cpu().numpy()
    scale = 0.5 * (abs(A) @ np.abs(x.cpu().numpy())) + 2.0 * np.abs(y0.cpu().numpy())
    assert (np.abs(y.cpu().numpy() - ref) <= 1e-14 * scale).all()
    with pytest.raises(pkg.DimensionMismatch):
        W.sell.apply(x[:100])
