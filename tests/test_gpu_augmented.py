"""The normal-derivative (Hermite-Birkhoff) batched build, RBF_FLAG_NORMAL_DOF: every
Neumann/Robin stencil point carries u and du/dn, so boundary-adjacent stencils solve
(k + m + nmon) systems of uneven size in the one persistent launch.  Against the CPU
restatement (oracle/augmented_oracle.py): structure bit-exact, weights within 1e-8 per row
(row max-norm, relative), and the exactness of the reference's Hermite tests
(test/hermite.jl:50-139): the weights reproduce the operator on the polynomial space."""
import numpy as np
import pytest

from test_oracle_augmented import apply_aug, mixed_square

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

W_TOL = 1e-8


@pytest.fixture(scope="module")
def pkg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    return g.load_package()


def herm_dict(pkg, isb, al, be, nrm):
    return dict(is_boundary=isb, bc=[pkg.BoundaryCondition(a, b) for a, b in zip(al, be)], normals=nrm)


def compare(W, rp, col, val, rows=None):
    """GPU rows (all, or `rows`) against the oracle's: structure equal, weights within W_TOL."""
    grp = W.row_ptr.cpu().numpy()
    gcol = W.col.cpu().numpy()
    gval = W.val.cpu().numpy()
    rows = np.arange(len(grp) - 1) if rows is None else rows
    worst = 0.0
    for t, e in enumerate(rows):
        c = gcol[grp[e]:grp[e + 1]]
        assert np.array_equal(c, col[rp[t]:rp[t + 1]]), e
        v, vr = gval[grp[e]:grp[e + 1]], val[rp[t]:rp[t + 1]]
        worst = max(worst, float(np.abs(v - vr).max() / np.abs(vr).max()))
    assert worst <= W_TOL, worst
    return worst


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_square_mixed_boundary(pkg, orc, precision):
    from oracle import augmented_oracle as A
    X, isb, al, be, nrm = mixed_square(m=41)
    ns = len(X)
    adjl = orc.knn(X, X, 20)
    rp, col, val = A.build_augmented(X, adjl, 2, 3, 2, [(orc.OP_LAP, 0)], (isb, al, be, nrm))
    ap, ai = pkg.ragged_stencils(torch.from_numpy(adjl).cuda(), torch.full((ns,), 20))
    W, status = pkg.build_weights_batched([(3, 0)], torch.from_numpy(X).cuda(), None, ap, ai, pkg.PHS(3, poly_deg=2),
                                          hermite=herm_dict(pkg, isb, al, be, nrm), precision=precision,
                                          normal_dof=True, return_status=True)
    W = W[0]
    b = np.nonzero(isb)[0]
    assert W.shape == (ns, ns + len(b))
    compare(W, rp, col, val[0])
    s = status.cpu().numpy()
    dirichlet = np.zeros(ns, bool)
    dirichlet[b] = (al == 1.0) & (be == 0.0)
    assert np.array_equal(s == 2, dirichlet)
    # the quadratic's Laplacian through the GPU apply, u and du/dn as data
    u = X[:, 0] ** 2 + X[:, 1] ** 2 + 1.0
    f = np.concatenate([u, (2.0 * X[b] * nrm).sum(1)])
    y = W.apply(torch.from_numpy(f).cuda()).cpu().numpy()
    assert np.abs(y[~dirichlet] - 4.0).max() < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_cube_ragged_multi_operator(pkg, orc, precision):
    """3D, ragged k (20 and 30) and per-stencil degrees (1 and 2), gradient + Laplacian, PHS5:
    classes differ in k, degree and the number of du/dn unknowns (sizes up to the 50s)."""
    from oracle import augmented_oracle as A
    rng = np.random.default_rng(21)
    n = 4000
    X = rng.uniform(0.0, 1.0, (n, 3))
    lo, hi = X[:, 0] < 0.05, X[:, 0] > 0.95
    X[lo, 0], X[hi, 0] = 0.0, 1.0
    isb = lo | hi
    b = np.nonzero(isb)[0]
    al = np.where(hi[b], 1.0, 0.0)
    be = np.where(hi[b], 0.0, 1.0)
    nrm = np.zeros((len(b), 3))
    nrm[:, 0] = np.where(hi[b], 1.0, -1.0)
    k_of = np.where(np.arange(n) % 2 == 0, 30, 20)
    deg_of = np.where(np.arange(n) % 3 == 0, 1, 2).astype(np.int8)
    adjl = orc.knn(X, X, 30)
    ops = [(1, 0), (1, 1), (3, 0)]
    Xd = torch.from_numpy(X).cuda()
    ap, ai = pkg.ragged_stencils(torch.from_numpy(adjl).cuda(), torch.from_numpy(k_of))
    st = pkg._native.BuildStats()
    W = pkg.build_weights_batched(ops, Xd, None, ap, ai, pkg.PHS(5, poly_deg=2), hermite=herm_dict(pkg, isb, al, be, nrm),
                                  precision=precision, poly_deg=torch.from_numpy(deg_of), normal_dof=True, stats=st,
                                  tune=2)
    assert int(st.n_singular) == 0
    # the oracle on the boundary-adjacent stencils of each (k, degree) and a few interior ones
    nr_pt = np.zeros(n, bool)
    nr_pt[b[be != 0.0]] = True
    m_of = np.array([nr_pt[adjl[e, :k_of[e]]].sum() for e in range(n)])
    rows = np.concatenate([np.nonzero((m_of > 0) & ~hi)[0][:240], np.nonzero(m_of == 0)[0][:60]])
    assert m_of.max() >= 8
    for kk in (20, 30):
        for dg in (1, 2):
            sel = rows[(k_of[rows] == kk) & (deg_of[rows] == dg)]
            if len(sel) == 0:
                continue
            rp, col, val = A.build_augmented(X, _full(adjl, kk, sel, n), 3, 5, dg, ops, (isb, al, be, nrm), rows=sel)
            for q in range(3):
                compare(W[q], rp, col, val[q], rows=sel)
    # exactness: a quadratic's gradient and Laplacian from u and du/dn
    u = X[:, 0] ** 2 + 2 * X[:, 1] * X[:, 2] + X[:, 2]
    f = np.concatenate([u, (np.stack([2 * X[b, 0], 2 * X[b, 2], 2 * X[b, 1] + 1], 1) * nrm).sum(1)])
    fd = torch.from_numpy(f).cuda()
    want = [2 * X[:, 0], 2 * X[:, 2], np.full(n, 2.0)]
    q2 = deg_of == 2
    for q in range(3):
        y = W[q].apply(fd).cpu().numpy()
        assert np.abs(y[q2 & ~hi] - want[q][q2 & ~hi]).max() < 1e-7, q


def _full(adjl, kk, sel, n):
    """An adjacency table whose rows `sel` hold their first kk neighbours (the oracle reads
    only the rows it builds)."""
    out = np.zeros((n, kk), dtype=adjl.dtype)
    out[sel] = adjl[sel, :kk]
    return out


def test_rejections(pkg):
    """PHS1 has no normal derivative at r = 0; the one-size build does not take the flag."""
    X, isb, al, be, nrm = mixed_square(m=11)
    Xd = torch.from_numpy(X).cuda()
    adjl = pkg.find_neighbors(Xd, k=9)
    ap, ai = pkg.ragged_stencils(adjl, torch.full((len(X),), 9))
    with pytest.raises(Exception, match="PHS 3, 5 or 7"):
        pkg.build_weights_batched([(3, 0)], Xd, None, ap, ai, pkg.PHS(1, poly_deg=1),
                                  hermite=herm_dict(pkg, isb, al, be, nrm), normal_dof=True)
    with pytest.raises(Exception, match="rbf_build_batched"):
        pkg.build_weights([(3, 0)], Xd, None, adjl, pkg.PHS(3, poly_deg=1), hermite=herm_dict(pkg, isb, al, be, nrm),
                          flags=pkg._native.FLAG_NORMAL_DOF)
