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


def test_ordered_copy_on_unordered_points(pkg, orc):
    """The copy in the Morton order of the points (to_sell_ordered): x and y stay in the caller's
    order; the product equals the oracle's within 1e-10, and the plain sliced copy's bit for bit
    (each row keeps its entries and their summation order, all rows have k entries)."""
    rng = np.random.default_rng(31)
    X = rng.uniform(0, 1, (40000, 3))
    Xd = torch.from_numpy(X).cuda()
    adjl = orc.knn(X, X, 30)
    ref = orc.build(X, X, adjl, 3, 3, 2, [(orc.OP_LAP, 0)])
    W = pkg.build_weights([(3, 0)], Xd, None, torch.from_numpy(adjl).cuda(), pkg.PHS(3, poly_deg=2), sell=True)[0]
    S = W.to_sell_ordered(Xd)
    # the ordered copy holds every row's entries, columns mapped to their Morton positions
    pos = torch.empty_like(S.col_at)
    pos[S.col_at.long()] = torch.arange(len(X), dtype=torch.int32, device="cuda")
    rows = sell_to_rows(S, len(X))
    ra = S.row_at.cpu().numpy()
    posh = pos.cpu().numpy()
    for r in range(0, len(X), 997):
        c, v = rows[r]
        cu, vu = csr_rows(W)[ra[r]]
        assert np.array_equal(c, posh[cu]) and np.array_equal(v, vu)
    f = np.sin(4 * X[:, 0]) * np.cos(3 * X[:, 1]) * np.exp(X[:, 2])
    fd = torch.from_numpy(f).cuda()
    y = S.apply(fd)
    yr = orc.spmm(ref, f)
    assert float(np.abs(y.cpu().numpy() - yr).max()) <= 1e-10 * np.abs(yr).max()
    assert torch.equal(y, W.sell.apply(fd))
    # beta != 0 accumulates into y in the caller's order
    y0 = torch.from_numpy(rng.standard_normal(len(X))).cuda()
    y1 = y0.clone()
    S.apply(fd, y1, alpha=-0.5, beta=2.0)
    assert torch.allclose(y1, -0.5 * y + 2.0 * y0, rtol=1e-14, atol=1e-12 * float(y.abs().max()))


def test_ordered_copy_regrid_and_uneven_rows(pkg, orc):
    """Eval points distinct from the data points (two orders) and rows of uneven length
    (Dirichlet identity rows of one entry among k-entry rows): within 1e-10 of the oracle."""
    rng = np.random.default_rng(32)
    S_ = rng.uniform(0, 1, (20000, 2))
    T_ = rng.uniform(0.05, 0.95, (15000, 2))
    adjl = orc.knn(S_, T_, 12)
    ref = orc.build(S_, T_, adjl, 2, 3, 1, [(orc.OP_IDENT, 0)])
    W = pkg.build_weights([(0, 0)], torch.from_numpy(S_).cuda(), torch.from_numpy(T_).cuda(),
                          torch.from_numpy(adjl).cuda(), pkg.PHS(3, poly_deg=1))[0]
    So = W.to_sell_ordered(torch.from_numpy(S_).cuda(), torch.from_numpy(T_).cuda())
    f = S_[:, 0] ** 2 - S_[:, 1]
    y = So.apply(torch.from_numpy(f).cuda()).cpu().numpy()
    yr = orc.spmm(ref, f)
    assert np.abs(y - yr).max() <= 1e-10 * np.abs(yr).max()
    # a square with Dirichlet boundary rows (identity rows hold one entry)
    xs = np.linspace(0, 1, 61)
    P = np.array([(x, yv) for x in xs for yv in xs])
    isb = (P[:, 0] == 0) | (P[:, 0] == 1) | (P[:, 1] == 0) | (P[:, 1] == 1)
    nrm = np.zeros((int(isb.sum()), 2))
    nrm[:, 0] = 1.0
    herm = dict(is_boundary=isb, bc=[pkg.BoundaryCondition(1.0, 0.0)] * int(isb.sum()), normals=nrm)
    op = pkg.laplacian(P, basis=pkg.PHS(3, poly_deg=2), k=15, hermite=herm)
    Wh = op.weights
    Sh = Wh.to_sell_ordered(torch.from_numpy(P).cuda())
    u = np.sin(P[:, 0]) * np.cos(2 * P[:, 1])
    y0 = Wh.apply(torch.from_numpy(u).cuda()).cpu().numpy()
    y1 = Sh.apply(torch.from_numpy(u).cuda()).cpu().numpy()
    # rows of 1/h^2-sized weights cancel to O(1) results: two summation orders agree to the
    # apply bar (1e-10 relative), not to the last bits
    assert np.abs(y1 - y0).max() <= 1e-10 * np.abs(y0).max()


def test_ordered_copy_rejects_bad_orders(pkg):
    rng = np.random.default_rng(33)
    X = torch.from_numpy(rng.uniform(0, 1, (3000, 2))).cuda()
    W = pkg.build_weights([(3, 0)], X, None, pkg.find_neighbors(X, k=12), pkg.PHS(3, poly_deg=2))[0]
    bad = torch.arange(3000, dtype=torch.int32, device="cuda")
    bad[7] = 3000
    with pytest.raises(ValueError):
        W.to_sell_ordered(X, row_at=bad, col_at=torch.arange(3000, dtype=torch.int32, device="cuda"))
    with pytest.raises(ValueError):
        W.to_sell_ordered(X, row_at=torch.arange(3000, dtype=torch.int32, device="cuda"), col_at=bad)
