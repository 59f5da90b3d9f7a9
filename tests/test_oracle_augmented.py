"""The CPU restatement of the normal-derivative (Hermite-Birkhoff) stencils
(oracle/augmented_oracle.py) against the exactness the formulation guarantees, in the manner of
the reference's Hermite exactness tests (test/hermite.jl:50-139,
test/solve/integration/laplacian_end_to_end.jl:45-78): with u and du/dn as data, the weights
reproduce the operator on the polynomial space exactly."""
import numpy as np
import pytest


def mixed_square(m=21, jitter=0.2, seed=3):
    """m x m points on [0,1]^2, interior jittered: Neumann on x = 0 (normal -x), Robin
    (alpha 1, beta 0.5) on y = 0 (normal -y), Dirichlet on x = 1 and y = 1 (corners Dirichlet)."""
    g = np.linspace(0.0, 1.0, m)
    X = np.array([(x, y) for y in g for x in g])
    inner = (X[:, 0] > 0) & (X[:, 0] < 1) & (X[:, 1] > 0) & (X[:, 1] < 1)
    X[inner] += np.random.default_rng(seed).uniform(-jitter, jitter, (int(inner.sum()), 2)) / (m - 1)
    isb = ~inner
    neu = isb & (X[:, 0] == 0) & (X[:, 1] > 0) & (X[:, 1] < 1)
    rob = isb & (X[:, 1] == 0) & (X[:, 0] > 0) & (X[:, 0] < 1)
    b = np.nonzero(isb)[0]
    alpha = np.where(neu[b], 0.0, 1.0)
    beta = np.where(neu[b], 1.0, np.where(rob[b], 0.5, 0.0))
    normals = np.zeros((len(b), 2))
    normals[neu[b], 0] = -1.0
    normals[rob[b], 1] = -1.0
    normals[~(neu[b] | rob[b]), 0] = 1.0
    return X, isb, alpha, beta, normals


def apply_aug(rp, col, val, f):
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    y = np.zeros(len(rp) - 1)
    np.add.at(y, rows, val * f[col])
    return y


def test_quadratic_laplacian_exact_2d(orc):
    from oracle import augmented_oracle as A
    X, isb, al, be, nrm = mixed_square()
    adjl = orc.knn(X, X, 15)
    rp, col, val = A.build_augmented(X, adjl, 2, 3, 2, [(orc.OP_LAP, 0)], (isb, al, be, nrm))
    ns, b = len(X), np.nonzero(isb)[0]
    u = X[:, 0] ** 2 + X[:, 1] ** 2 + 1.0
    dudn = (2.0 * X[b] * nrm).sum(1)
    y = apply_aug(rp, col, val[0], np.concatenate([u, dudn]))
    dirichlet = np.zeros(ns, bool)
    dirichlet[b] = (al == 1.0) & (be == 0.0)
    assert np.abs(y[~dirichlet] - 4.0).max() < 1e-9
    assert np.array_equal(y[dirichlet], u[dirichlet])
    # row lengths: k + the Neumann/Robin neighbours; identity rows hold one entry
    nr = np.zeros(ns + 1, bool)
    nr[b] = ~((al == 1.0) & (be == 0.0))
    lens = np.where(dirichlet, 1, 15 + nr[adjl].sum(1))
    assert np.array_equal(np.diff(rp), lens)
    assert lens.max() > 15
    # columns ascending, derivative columns at ns + boundary ordinal
    for e in range(ns):
        c = col[rp[e]:rp[e + 1]]
        assert np.all(np.diff(c) > 0)
        assert np.all(c[c >= ns] - ns < len(b))


def test_quadratic_gradient_and_laplacian_exact_3d(orc):
    from oracle import augmented_oracle as A
    rng = np.random.default_rng(11)
    X = rng.uniform(0.0, 1.0, (1500, 3))
    lo = X[:, 0] < 0.06
    X[lo, 0] = 0.0
    isb = lo
    nb = int(isb.sum())
    normals = np.zeros((nb, 3))
    normals[:, 0] = -1.0
    adjl = orc.knn(X, X, 30)
    ops = [(orc.OP_D1, 0), (orc.OP_D1, 2), (orc.OP_LAP, 0)]
    rows = np.concatenate([np.nonzero(isb)[0][:60], np.nonzero(~isb)[0][:40]])
    rp, col, val = A.build_augmented(X, adjl, 3, 5, 2, ops, (isb, np.zeros(nb), np.ones(nb), normals), rows=rows)
    b = np.nonzero(isb)[0]
    u = X[:, 0] ** 2 + 2 * X[:, 1] * X[:, 2] + X[:, 2] + 1.0
    f = np.concatenate([u, -2.0 * X[b, 0]])  # du/dn = -du/dx
    want = [2 * X[rows, 0], 2 * X[rows, 1] + 1.0, np.full(len(rows), 2.0)]
    for q in range(3):
        y = apply_aug(rp, col, val[q], f)
        assert np.abs(y - want[q]).max() < 1e-8, q
