"""Operator algebra on built operators (operator_algebra.jl:245-295) and the directional
derivative (directional.jl:69-95), combined on the device: bit-identical to the host
arithmetic of the reference on the component weights (products and sums rounded
separately, left to right), the reference's errors for incompatible operands."""
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


@pytest.fixture(scope="module")
def cloud():
    rng = np.random.default_rng(21)
    return rng.uniform(0, 1, (6000, 3))


def vals(op):
    W = op.weights
    return W.val.cpu().numpy() if not isinstance(W, tuple) else [w.val.cpu().numpy() for w in W]


def test_sum_difference_scaling(pkg, cloud):
    X = torch.from_numpy(cloud).cuda()
    L = pkg.laplacian(X, k=30)
    P = pkg.partial(X, 1, 1, k=30, adjl=L.adjl)
    S = L + 2.0 * P
    D = L - P
    N = -L
    Q = L / 4.0
    lv, pv = vals(L), vals(P)
    assert np.array_equal(vals(S), lv + 2.0 * pv)
    assert np.array_equal(vals(D), lv - pv)
    assert np.array_equal(vals(N), -1.0 * lv)
    assert np.array_equal(vals(Q), (1.0 / 4.0) * lv)
    assert torch.equal(S.weights.col, L.weights.col) and torch.equal(S.weights.row_ptr, L.weights.row_ptr)
    f = torch.sin(3 * X[:, 0]) * X[:, 1] + X[:, 2] ** 2
    y = S(f)
    y_ref = L(f) + 2.0 * P(f)
    assert (y - y_ref).abs().max() <= 1e-9 * y_ref.abs().max()
    # an updated sum rebuilds its parts
    S.invalidate_cache()
    S.update_weights()
    assert np.array_equal(vals(S), lv + 2.0 * pv)


def test_jacobian_sum(pkg, cloud):
    X = torch.from_numpy(cloud).cuda()
    J = pkg.jacobian(X, k=30)
    J2 = J + J
    for a, b in zip(vals(J2), vals(J)):
        assert np.array_equal(a, b + b)


def test_incompatible(pkg, cloud):
    X = torch.from_numpy(cloud).cuda()
    L30 = pkg.laplacian(X, k=30)
    L20 = pkg.laplacian(X, k=20)
    with pytest.raises(ValueError, match="same stencils"):
        L30 + L20
    with pytest.raises(ValueError, match="same data"):
        L30 + pkg.laplacian(X + 1e-3, k=30)
    with pytest.raises(ValueError, match="output ranks"):
        L30 + pkg.jacobian(X, k=30, adjl=L30.adjl)


def test_directional_constant_and_per_point(pkg, cloud):
    X = torch.from_numpy(cloud).cuda()
    J = pkg.jacobian(X, k=30)
    jv = vals(J)
    v = np.array([0.3, -1.1, 0.7])
    Dc = pkg.directional(X, v, k=30, adjl=J.adjl)
    assert np.array_equal(vals(Dc), (jv[0] * v[0] + jv[1] * v[1]) + jv[2] * v[2])
    nrm = cloud - 0.5
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    Dp = pkg.directional(X, nrm, k=30, adjl=J.adjl)
    rows = np.repeat(np.arange(len(cloud)), np.diff(J.weights[0].row_ptr.cpu().numpy()))
    want = (nrm[rows, 0] * jv[0] + nrm[rows, 1] * jv[1]) + nrm[rows, 2] * jv[2]
    assert np.array_equal(vals(Dp), want)
    # a linear field is reproduced exactly (up to rounding): grad f . n = (2, 3, -1) . n
    f = 2 * X[:, 0] + 3 * X[:, 1] - X[:, 2]
    got = Dp(f).cpu().numpy()
    assert np.abs(got - nrm @ np.array([2.0, 3.0, -1.0])).max() < 1e-9
    with pytest.raises(ValueError):
        pkg.directional(X, np.ones(5), k=30, adjl=J.adjl)


def test_axpby_power_of_two_scalings_exact(pkg):
    """Scalings by +-1 and other powers of two move the exponent on the integer pipe; the
    results must equal the rounded products and sums bit for bit, also where the product
    leaves the normal range (zeros, subnormals, overflow to infinity) or the input is not
    finite."""
    ctx = pkg.Context.default(0)
    rng = np.random.default_rng(5)
    special = np.array([0.0, -0.0, 5e-324, -2.5e-310, 2.2250738585072014e-308, 1e308, -1.7e308, np.inf, -np.inf,
                        1.0, -3.0, 0.1])
    a = np.concatenate([special, rng.standard_normal(4000) * 10.0 ** rng.integers(-300, 300, 4000)])
    b = np.concatenate([special[::-1], rng.standard_normal(4000)])
    ad, bd = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.empty_like(ad)
    for alpha, beta in [(1.0, 2.0), (-1.0, 1.0), (0.5, -0.25), (2.0 ** 600, 1.0), (3.0, -1.0), (1.0, 0.3),
                        (-0.7, 1.1)]:
        for with_b in (True, False):
            st = ctx.lib.rbf_weights_axpby(ctx.h, len(a), alpha, pkg._ptr(ad), beta,
                                           pkg._ptr(bd) if with_b else None, pkg._ptr(out))
            assert st == 0
            torch.cuda.synchronize()
            with np.errstate(over="ignore", invalid="ignore"):
                ref = alpha * a + beta * b if with_b else alpha * a
            got = out.cpu().numpy()
            same = (got.view(np.int64) == ref.view(np.int64)) | (np.isnan(got) & np.isnan(ref))
            assert same.all(), (alpha, beta, with_b, a[~same][:4], got[~same][:4], ref[~same][:4])
