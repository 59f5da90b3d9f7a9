"""The reference's operator accuracy tests, restated on the GPU path through the operator
API (test/operators/laplacian.jl, gradient.jl, partial.jl, regrid.jl): Franke-like
f = 1 + sin(4x) + cos(3x) + sin(2y) on 10,000 Halton points (the radical-inverse sequence of
bases 2 and 3 from index 1, the points HaltonSequences.jl gives), mean percent error below
the reference's thresholds.  The reference draws its 100 off-grid eval points with Julia's
MersenneTwister; seeded numpy points stand in (the thresholds do not depend on them).  The
IMQ and Gaussian variants of these tests are outside this library (PHS bases only)."""
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


def halton(n, base):
    out = np.zeros(n)
    idx = np.arange(1, n + 1)
    f = 1.0
    while idx.any():
        f /= base
        out += f * (idx % base)
        idx //= base
    return out


X = np.stack([halton(10_000, 2), halton(10_000, 3)], 1)
X2 = np.random.default_rng(345).uniform(0, 1, (100, 2))


def f(p):
    return 1 + np.sin(4 * p[:, 0]) + np.cos(3 * p[:, 0]) + np.sin(2 * p[:, 1])


def df_dx(p):
    return 4 * np.cos(4 * p[:, 0]) - 3 * np.sin(3 * p[:, 0])


def df_dy(p):
    return 2 * np.cos(2 * p[:, 1])


def d2f_dxx(p):
    return -16 * np.sin(4 * p[:, 0]) - 9 * np.cos(3 * p[:, 0])


def d2f_dyy(p):
    return -4 * np.sin(2 * p[:, 1])


def mpe(test, correct):
    """mean_percent_error (test/test_utils.jl)"""
    return float(np.mean(np.abs((np.asarray(test) - correct) / correct)) * 100)


def test_laplacian(pkg):
    y = f(X)
    L = pkg.laplacian(X, pkg.PHS(3, poly_deg=4))
    assert mpe(L(y), d2f_dxx(X) + d2f_dyy(X)) < 10
    assert isinstance(pkg.laplacian(X), pkg.RadialBasisOperator)  # default PHS(3; poly_deg=2)
    L2 = pkg.laplacian(X, eval_points=X.copy(), basis=pkg.PHS(3, poly_deg=4))
    assert mpe(L2(y), d2f_dxx(X) + d2f_dyy(X)) < 10


def test_gradient(pkg):
    y = f(X)
    g = pkg.gradient(X, pkg.PHS(3, poly_deg=2))(y)
    assert g.shape == (10_000, 2)
    assert mpe(g[:, 0], df_dx(X)) < 10 and mpe(g[:, 1], df_dy(X)) < 10
    g2 = pkg.gradient(X, eval_points=X2, basis=pkg.PHS(3, poly_deg=2))(y)
    assert g2.shape == (100, 2)
    assert mpe(g2[:, 0], df_dx(X2)) < 10 and mpe(g2[:, 1], df_dy(X2)) < 10


def test_partials(pkg):
    y = f(X)
    assert mpe(pkg.partial(X, 1, 1, pkg.PHS(3, poly_deg=2))(y), df_dx(X)) < 10
    assert mpe(pkg.partial(X, 1, 2, pkg.PHS(3, poly_deg=2))(y), df_dy(X)) < 10
    assert mpe(pkg.partial(X, 2, 1, pkg.PHS(3, poly_deg=4))(y), d2f_dxx(X)) < 10
    assert mpe(pkg.partial(X, 2, 2, pkg.PHS(3, poly_deg=4))(y), d2f_dyy(X)) < 10
    assert mpe(pkg.partial(X, 1, 1, eval_points=X2, basis=pkg.PHS(3, poly_deg=2))(y), df_dx(X2)) < 10
    assert mpe(pkg.partial(X, 1, 2, eval_points=X2, basis=pkg.PHS(3, poly_deg=2))(y), df_dy(X2)) < 10
    with pytest.raises(ValueError):
        pkg.partial(X, 3, 1)


def test_regrid(pkg):
    y = f(X)
    assert mpe(pkg.regrid(X, X2, pkg.PHS(3, poly_deg=2))(y), f(X2)) < 0.1
    r = pkg.regrid(X, X2)  # default basis
    assert isinstance(r, pkg.RadialBasisOperator) and mpe(r(y), f(X2)) < 0.1
    assert isinstance(pkg.regrid(X, X2, basis=pkg.PHS(5, poly_deg=3)), pkg.RadialBasisOperator)


def test_directional(pkg):
    """test/operators/directional.jl: one direction, one per point, other eval points, and the
    reference's errors for a direction of the wrong dimension or count."""
    y = f(X)
    rng = np.random.default_rng(456)
    v = np.array([2.0, 1.0]) / np.hypot(2.0, 1.0)
    d = pkg.directional(X, v, pkg.PHS(3, poly_deg=2))(y)
    assert mpe(d, df_dx(X) * v[0] + df_dy(X) * v[1]) < 10
    V = rng.uniform(0, 1, (10_000, 2))
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    d = pkg.directional(X, V, pkg.PHS(3, poly_deg=2))(y)
    assert mpe(d, df_dx(X) * V[:, 0] + df_dy(X) * V[:, 1]) < 10
    d = pkg.directional(X, V, eval_points=X.copy(), basis=pkg.PHS(3, poly_deg=2))(y)
    assert mpe(d, df_dx(X) * V[:, 0] + df_dy(X) * V[:, 1]) < 10
    with pytest.raises(ValueError):
        pkg.directional(X, np.array([2.0, 1.0, 0.5]))(y)
    with pytest.raises(ValueError):
        pkg.directional(X, V[:-1])(y)


def test_operator_algebra(pkg):
    """test/operators/operator_algebra.jl:9-35: sums and differences of partials reproduce the
    derivatives of a linear field exactly (MPE < 1e-6); operators on other data or other
    stencils cannot be combined."""
    x = X[:1000]
    y = 2 * x[:, 0] + 3 * x[:, 1]
    dx = pkg.partial(x, 1, 1)
    dy = pkg.partial(x, 1, 2)
    assert mpe((dx + dy)(y), np.full(1000, 5.0)) < 1e-6
    assert mpe((dx - dy)(y), np.full(1000, -1.0)) < 1e-6
    with pytest.raises(ValueError):
        dx + pkg.partial(x[:500], 1, 2)
    adjl = np.asarray(dx.adjl.cpu() if hasattr(dx.adjl, "cpu") else dx.adjl).copy()
    adjl[[0, 1]] = adjl[[1, 0]]
    with pytest.raises(ValueError):
        dx + pkg.partial(x, 1, 2, adjl=adjl)
