"""Pins the oracle's pullback of the weight build (oracle/backward_oracle.py) the way the
reference validates its own AD rules: against central finite differences of the forward
build (test/extensions/ad_test_utils.jl make_build_weights_test_data / validate_gradient,
used by test/extensions/mooncake_ext.jl:82-125 and enzyme_ext.jl: a 5 x 5 grid, k = 10,
loss sum(W.nzval .^ 2), rtol 1e-3 there, 1e-6 here), plus 3D clouds with separate eval
points and all the operators the GPU adjoint supports."""
import numpy as np
import pytest

OP_IDENT, OP_D1, OP_LAP = 0, 1, 3


@pytest.fixture(scope="module")
def bo(orc):
    from oracle import backward_oracle
    return backward_oracle


def grid_points():
    # make_build_weights_test_data: SVector(0.1 + 0.8 i / 5, 0.1 + 0.8 j / 5), i, j = 1..5
    return np.array([[0.1 + 0.8 * i / 5, 0.1 + 0.8 * j / 5] for i in range(1, 6) for j in range(1, 6)])


def fd_gradient(f, x, h):
    g = np.zeros_like(x)
    for idx in np.ndindex(x.shape):
        xp = x.copy()
        xm = x.copy()
        xp[idx] += h
        xm[idx] -= h
        g[idx] = (f(xp) - f(xm)) / (2 * h)
    return g


@pytest.mark.parametrize("phs,deg,op", [(3, 2, (OP_D1, 0)), (3, 2, (OP_LAP, 0)), (1, 1, (OP_D1, 0)),
                                        (3, 1, (OP_D1, 0)), (5, 1, (OP_D1, 0)), (7, 1, (OP_D1, 0)),
                                        (5, 2, (OP_LAP, 0)), (7, 2, (OP_LAP, 0)), (1, 1, (OP_LAP, 0))])
def test_grid_sum_of_squares(orc, bo, phs, deg, op):
    """eval points = data points; L = sum(W.nzval^2) as in the reference's AD tests."""
    X = grid_points()
    adjl = orc.knn(X, X, 10)
    ops = [op]

    def weights(P):
        return bo.csr_to_stencil_order(orc.build(P, P, adjl, 2, phs, deg, ops), adjl)

    w = weights(X)
    gd, ge = bo.build_backward(X, X, adjl, 2, phs, deg, ops, 2.0 * w)
    got = gd + ge
    want = fd_gradient(lambda P: float(np.sum(weights(P) ** 2)), X, 1e-6)
    scale = np.abs(want).max()
    assert scale > 0
    assert np.abs(got - want).max() <= 1e-6 * scale


@pytest.mark.parametrize("phs,ops", [(3, [(OP_LAP, 0)]), (5, [(OP_D1, 0), (OP_D1, 1), (OP_D1, 2)]),
                                     (7, [(OP_IDENT, 0)]), (3, [(OP_IDENT, 0), (OP_LAP, 0)])])
def test_cloud3d_separate_eval(orc, bo, phs, ops):
    rng = np.random.default_rng(5)
    data = rng.uniform(0, 1, (60, 3))
    ev = rng.uniform(0.2, 0.8, (12, 3))
    k = 20
    adjl = orc.knn(data, ev, k)
    dW = rng.standard_normal((len(ops), len(ev), k))
    gd, ge = bo.build_backward(data, ev, adjl, 3, phs, 2, ops, dW)
    f_data = fd_gradient(lambda P: bo.loss(P, ev, adjl, 3, phs, 2, ops, dW), data, 1e-6)
    f_eval = fd_gradient(lambda Q: bo.loss(data, Q, adjl, 3, phs, 2, ops, dW), ev, 1e-6)
    assert np.abs(gd - f_data).max() <= 1e-6 * np.abs(f_data).max()
    assert np.abs(ge - f_eval).max() <= 1e-6 * np.abs(f_eval).max()
    # points outside every stencil get no gradient
    used = np.zeros(len(data), bool)
    used[np.unique(adjl)] = True
    assert np.all(gd[~used] == 0.0)


@pytest.mark.parametrize("phs,ops,dim", [(3, [(OP_LAP, 0)], 3), (5, [(OP_D1, 0), (OP_D1, 1), (OP_D1, 2)], 3),
                                         (1, [(OP_D1, 1), (OP_LAP, 0)], 2), (7, [(OP_IDENT, 0)], 3)])
def test_c_pullback_matches(orc, bo, phs, ops, dim):
    """The C restatement (timed as the CPU baseline of the adjoint) equals the Python one to
    the rounding of their solvers (rook Bunch-Kaufman there, numpy's LU here; 1.4e-12 apart on
    PHS7's poorly conditioned systems)."""
    rng = np.random.default_rng(21)
    data = rng.uniform(0, 1, (200, dim))
    ev = rng.uniform(0.2, 0.8, (30, dim))
    k = 20
    adjl = orc.knn(data, ev, k)
    dW = rng.standard_normal((len(ops), len(ev), k))
    pd, pe = bo.build_backward(data, ev, adjl, dim, phs, 2, ops, dW)
    cd, ce = orc.build_backward_c(data, ev, adjl, dim, phs, 2, ops, dW)
    assert np.abs(cd - pd).max() <= 1e-10 * np.abs(pd).max()
    assert np.abs(ce - pe).max() <= 1e-10 * np.abs(pe).max()
