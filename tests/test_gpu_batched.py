"""The batched build of uneven stencils (one persistent launch over size classes, autotuned
tile shapes) against the one-size builds it must reproduce."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

LU = 4  # RBF_FLAG_FP64_LU: the one-size FP64 build with the batched build's LU solver


@pytest.fixture(scope="module")
def pkg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    return g.load_package()


def rows_of(W, rows):
    rp = W.row_ptr.cpu().numpy()
    col = W.col.cpu().numpy()
    val = W.val.cpu().numpy()
    return [(col[rp[r]:rp[r + 1]], val[rp[r]:rp[r + 1]]) for r in rows]


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_uniform_batch_equals_build(pkg, precision):
    """Uniform stencils through the batched path give the one-size build's weights: the same
    per-stencil code, bit for bit in FP64 (warp tiles: the symmetric indefinite solve), within
    1e-8 of the LU (RBF_FLAG_FP64_LU) and in the refined form."""
    rng = np.random.default_rng(1)
    X = torch.from_numpy(rng.uniform(0, 1, (20000, 3))).cuda()
    adjl = pkg.find_neighbors(X, k=30)
    basis = pkg.PHS(3, poly_deg=2)
    W0 = pkg.build_weights([(3, 0)], X, None, adjl, basis, precision="fp64")[0]
    ap, ai = pkg.ragged_stencils(adjl, torch.full((20000,), 30))
    W1 = pkg.build_weights_batched([(3, 0)], X, None, ap, ai, basis, precision=precision, tune=0)[0]
    assert torch.equal(W1.row_ptr, W0.row_ptr) and torch.equal(W1.col, W0.col)
    if precision == "fp64":
        assert torch.equal(W1.val, W0.val)
        Wlu = pkg.build_weights([(3, 0)], X, None, adjl, basis, precision="fp64", flags=LU)[0]
        d = (W1.val - Wlu.val).abs().reshape(-1, 30).amax(1) / Wlu.val.abs().reshape(-1, 30).amax(1)
        assert float(d.max()) <= 1e-8
    else:
        d = (W1.val - W0.val).abs().reshape(-1, 30).amax(1) / W0.val.abs().reshape(-1, 30).amax(1)
        assert float(d.max()) <= 1e-8


def test_block_tile_bit_identical(pkg):
    """A class above n = 64 runs with the block tile (128 threads factorise one system); its
    factorisation is bit-identical to the one-warp kernel's."""
    rng = np.random.default_rng(2)
    X = torch.from_numpy(rng.uniform(0, 1, (3000, 3))).cuda()
    adjl = pkg.find_neighbors(X, k=60)
    basis = pkg.PHS(3, poly_deg=2)  # n = 70
    W0 = pkg.build_weights([(3, 0), (1, 0)], X, None, adjl, basis, precision="fp64", flags=LU)
    ap, ai = pkg.ragged_stencils(adjl, torch.full((3000,), 60))
    W1 = pkg.build_weights_batched([(3, 0), (1, 0)], X, None, ap, ai, basis, precision="fp64", tune=0)
    for a, b in zip(W1, W0):
        assert torch.equal(a.col, b.col)
        assert torch.equal(a.val, b.val)


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_mixed_sizes_and_degrees(pkg, precision):
    """Stencils of sizes 12/20/30 and degrees 1/2 in one batch: every row equals the row of a
    uniform build of its own (k, degree) class."""
    rng = np.random.default_rng(3)
    n = 30000
    X = torch.from_numpy(rng.uniform(0, 1, (n, 2))).cuda()
    adjl = pkg.find_neighbors(X, k=30)
    kp = rng.choice([12, 20, 30], n)
    deg = rng.choice([1, 2], n).astype(np.int8)
    ap, ai = pkg.ragged_stencils(adjl, torch.from_numpy(kp))
    st = pkg._native.BuildStats()
    W = pkg.build_weights_batched([(3, 0)], X, None, ap, ai, pkg.PHS(3, poly_deg=2), precision=precision,
                                  poly_deg=deg, tune=1, stats=st)[0]
    assert int(W.row_ptr[-1]) == int(kp.sum())
    for k in (12, 20, 30):
        for dg in (1, 2):
            sel = np.nonzero((kp == k) & (deg == dg))[0]
            ref = pkg.build_weights([(3, 0)], X, X[torch.from_numpy(sel).cuda()], adjl[torch.from_numpy(sel).cuda(), :k],
                                    pkg.PHS(3, poly_deg=dg), precision="fp64")[0]
            got = rows_of(W, sel)
            want = rows_of(ref, range(len(sel)))
            for (c1, v1), (c2, v2) in zip(got, want):
                assert np.array_equal(c1, c2)
                err = np.abs(v1 - v2).max() / np.abs(v2).max()
                # autotuned classes may run block tiles (the LU) against the one-size
                # symmetric indefinite solve: equal to within rounding, not bit for bit
                assert err <= (1e-10 if precision == "fp64" else 1e-8), (k, dg, err)


def test_hermite_in_batch(pkg):
    """Hermite boundary stencils (Dirichlet identity rows, Neumann neighbours) in the batched
    path equal the one-size Hermite build."""
    rng = np.random.default_rng(4)
    m = 40
    g = np.stack(np.meshgrid(np.linspace(0, 1, m), np.linspace(0, 1, m), indexing="ij"), -1).reshape(-1, 2)
    g = g + rng.uniform(-0.2, 0.2, g.shape) / m * ((g > 0) & (g < 1))
    isb = (g[:, 0] == 0) | (g[:, 0] == 1) | (g[:, 1] == 0) | (g[:, 1] == 1)
    nb = int(isb.sum())
    bpts = g[isb]
    normals = np.zeros((nb, 2))
    normals[bpts[:, 0] == 0, 0] = -1
    normals[bpts[:, 0] == 1, 0] = 1
    normals[(bpts[:, 1] == 0) & (normals[:, 0] == 0), 1] = -1
    normals[(bpts[:, 1] == 1) & (normals[:, 0] == 0), 1] = 1
    bc = [pkg.Dirichlet() if p[1] > 0.5 else pkg.Neumann() for p in bpts]
    herm = dict(is_boundary=isb, bc=bc, normals=normals)
    X = torch.from_numpy(g).cuda()
    adjl = pkg.find_neighbors(X, k=20)
    basis = pkg.PHS(3, poly_deg=2)
    W0 = pkg.build_weights([(3, 0)], X, None, adjl, basis, hermite=herm, precision="fp64")[0]
    ap, ai = pkg.ragged_stencils(adjl, torch.full((len(g),), 20))
    W1 = pkg.build_weights_batched([(3, 0)], X, None, ap, ai, basis, hermite=herm, precision="fp64", tune=0)[0]
    assert torch.equal(W1.row_ptr, W0.row_ptr) and torch.equal(W1.col, W0.col)
    assert torch.equal(W1.val, W0.val)


def test_autotuner_records_classes(pkg):
    """tune=2 times both tiles on each class with at least 1024 stencils and caches the choice."""
    rng = np.random.default_rng(5)
    n = 8000
    X = torch.from_numpy(rng.uniform(0, 1, (n, 3))).cuda()
    adjl = pkg.find_neighbors(X, k=40)
    kp = np.where(np.arange(n) % 2 == 0, 20, 40)
    ap, ai = pkg.ragged_stencils(adjl, torch.from_numpy(kp))
    pkg.build_weights_batched([(3, 0)], X, None, ap, ai, pkg.PHS(3, poly_deg=1), precision="fp64", tune=2)
    rep = pkg.tuning_report()
    assert "k=20 degree=1" in rep and "k=40 degree=1" in rep, rep
    assert "tile=" in rep and "sample 4000" in rep, rep


def test_batched_errors(pkg):
    X = np.random.default_rng(6).uniform(0, 1, (200, 2))
    basis = pkg.PHS(3, poly_deg=2)
    adjl = pkg.find_neighbors(X, k=10)
    ap, ai = pkg.ragged_stencils(torch.from_numpy(adjl), torch.full((200,), 10))
    bad = ap.clone()
    bad[5:] += 70  # one stencil of 80 neighbours: above the maximum stencil size
    with pytest.raises(ValueError):
        pkg.build_weights_batched([(3, 0)], X, None, bad, torch.cat([ai, ai[:70]]), basis)
    with pytest.raises(ValueError):
        pkg.build_weights_batched([(3, 0)], X, None, ap, ai, basis, poly_deg=np.full(200, 9, np.int8))
    with pytest.raises(ValueError):
        pkg.build_weights_batched([(3, 0)], X, None, ap, ai, basis, precision="learned")


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_build_apply_graph(pkg, precision):
    """The captured build -> apply graph, replayed after the points move and the field
    changes in place, gives exactly the weights and the result of the direct calls."""
    rng = np.random.default_rng(7)
    n = 20000
    X = torch.from_numpy(rng.uniform(0, 1, (n, 3))).cuda()
    adjl = pkg.find_neighbors(X, k=30).to(torch.int32).contiguous()
    f = torch.sin(4 * X[:, 0]).contiguous()
    basis = pkg.PHS(3, poly_deg=2)
    G = pkg.BuildApplyGraph((3, 0), X, None, adjl, basis, f, precision=precision)
    for step in range(3):
        X.add_(torch.from_numpy(rng.uniform(-1e-4, 1e-4, (n, 3))).cuda())  # points move, stencils stay
        f.copy_(torch.sin(4 * X[:, 0]) * (1 + step))
        y = G.replay().clone()
        W = pkg.build_weights([(3, 0)], X, None, adjl, basis, precision=precision)[0]
        assert torch.equal(G.weights[0].col, W.col)
        assert torch.equal(G.weights[0].val, W.val)
        assert torch.equal(y, W.apply(f))
    c = G.counters()
    assert c["singular"] == 0
    if precision == "fp32_refined":
        assert c["residuals"] >= n


def test_split_tile_for_40_row_classes(pkg):
    """FP32-refined classes of 40-row single-operator systems can run the split-row register
    kernel (the split tile, its own launch with the general kernel finishing what it hands
    over): the autotuner times it beside the warp and block tiles, and every row of a mixed
    batch equals (to 1e-8) the row of a one-size refined build of its class."""
    rng = np.random.default_rng(7)
    n = 12000
    X = torch.from_numpy(rng.uniform(0, 1, (n, 3))).cuda()
    adjl = pkg.find_neighbors(X, k=30)
    kp = np.where(np.arange(n) % 3 == 0, 20, 30)
    ap, ai = pkg.ragged_stencils(adjl, torch.from_numpy(kp))
    basis = pkg.PHS(3, poly_deg=2)
    st = pkg._native.BuildStats()
    W = pkg.build_weights_batched([(3, 0)], X, None, ap, ai, basis, precision="fp32_refined", tune=2, stats=st)[0]
    rep = pkg.tuning_report()
    line = [ln for ln in rep.splitlines() if "precision=fp32_refined dim=3 phs=3 nops=1 k=30 degree=2 boundary=0" in ln]
    assert line and "split " in line[0] and "split 0.000 ms" not in line[0], rep
    assert int(st.n_stencils) == n
    for k in (20, 30):
        sel = np.nonzero(kp == k)[0]
        sd = torch.from_numpy(sel).cuda()
        ref = pkg.build_weights([(3, 0)], X, X[sd], adjl[sd, :k], basis, precision="fp32_refined")[0]
        for (c1, v1), (c2, v2) in zip(rows_of(W, sel), rows_of(ref, range(len(sel)))):
            assert np.array_equal(c1, c2)
            assert np.abs(v1 - v2).max() <= 1e-8 * np.abs(v2).max()
