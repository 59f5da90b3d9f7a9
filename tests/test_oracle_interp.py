"""Pins the oracle's global interpolation (oracle.interp_fit / interp_eval: the collocation
matrix of src/interpolation.jl:27-31 solved by the restated dsytf2_rook / dsytrs_rook) to the
reference's own tests (test/operators/interpolation.jl: Franke's function on 10,000 Halton
points, PHS3 degree 2, |interp(0.5, 0.5) - franke| < 1e-5; the two-point 1D PHS1 case) and to
LAPACK's dsytrf_rook (the routine bunchkaufman!(A, true) calls); and checks on the CPU the
converted-factor solve the GPU uses (one row permutation, U, D, U^T)."""
import numpy as np
import pytest


def halton(n, base):
    """Radical-inverse (Halton) sequence, indices 1..n: the points HaltonSequences.jl's
    HaltonPoint gives (a seeded stand-in would do for the 1e-5 check as well)."""
    out = np.zeros(n)
    for i in range(n):
        f, r, k = 1.0, 0.0, i + 1
        while k > 0:
            f /= base
            r += f * (k % base)
            k //= base
        out[i] = r
    return out


def franke(p):
    x, y = p[..., 0], p[..., 1]
    a = 0.75 * np.exp(-(9 * x - 2) ** 2 / 4 - (9 * y - 2) ** 2 / 4)
    b = 0.75 * np.exp(-(9 * x + 1) ** 2 / 49 - (9 * y + 1) / 10)
    c = 0.5 * np.exp(-(9 * x - 7) ** 2 / 4 - (9 * y - 3) ** 2 / 4)
    d = 0.2 * np.exp(-(9 * x - 4) ** 2 - (9 * y - 7) ** 2)
    return a + b + c - d


def converted_solve(orc, F, ipiv, b):
    """x = A^-1 b from the converted factor: b[perm], U^-1, D^-1, U^-T, scatter through perm
    (the order of the GPU solve)."""
    G = orc.convert_rook_factor(F, ipiv)
    n = G.shape[0]
    perm = np.arange(n)
    blk = np.zeros(n, dtype=int)
    for k, kstep, sw in orc.rook_steps(ipiv):
        for a, c in sw:
            perm[[a - 1, c - 1]] = perm[[c - 1, a - 1]]
        if kstep == 2:
            blk[k - 1], blk[k - 2] = 1, 2
    U = np.triu(G, 1)
    for k in range(1, n + 1):
        if blk[k - 1] == 1:
            U[k - 2, k - 1] = 0.0
    U += np.eye(n)
    D = np.zeros((n, n))
    for k in range(1, n + 1):
        if blk[k - 1] == 0:
            D[k - 1, k - 1] = G[k - 1, k - 1]
        elif blk[k - 1] == 1:
            D[k - 2:k, k - 2:k] = [[G[k - 2, k - 2], G[k - 2, k - 1]], [G[k - 2, k - 1], G[k - 1, k - 1]]]
    y = np.linalg.solve(U, b[perm])
    z = np.linalg.solve(U.T, np.linalg.solve(D, y))
    x = np.empty(n)
    x[perm] = z
    return x, U, D, perm


def test_two_point_phs1(orc):
    """interpolation.jl:36-39: the last data point is reproduced."""
    x = np.array([[0.0], [1.0]])
    y = np.array([0.0, 1.0])
    w = orc.interp_fit(x, y, 1, 1)
    v = orc.interp_eval(x, w, x[1:], 1, 1)
    assert abs(v[0] - 1.0) <= 1.5e-8


@pytest.mark.parametrize("phs,deg", [(3, 2), (1, 1), (5, 2), (3, 0)])
def test_restated_vs_lapack_and_converted_solve(orc, phs, deg):
    solver = orc.lapack_rook_solver()
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 1, (500, 2))
    y = franke(x)
    w = orc.interp_fit(x, y, phs, deg)
    xe = rng.uniform(0, 1, (200, 2))
    v = orc.interp_eval(x, w, xe, phs, deg)
    if solver is not None:
        wl = orc.interp_fit(x, y, phs, deg, solver=solver)
        vl = orc.interp_eval(x, wl, xe, phs, deg)
        assert np.abs(v - vl).max() <= 1e-10 * np.abs(vl).max()
    # the converted factorisation reproduces A and its solve equals dsytrs_rook's
    A = orc.interp_matrix(x, phs, deg)
    Asym = np.triu(A) + np.triu(A, 1).T
    F, ipiv, info = orc.sytrf_rook_restated(A)
    assert info == 0
    b = np.zeros(A.shape[0])
    b[:len(x)] = y
    xs, U, D, perm = converted_solve(orc, F, ipiv, b)
    P = np.eye(len(perm))[:, perm]  # P e_r = e_perm[r]: (P v)[perm[r]] = v[r]
    R = P @ U @ D @ U.T @ P.T
    assert np.abs(R - Asym).max() <= 1e-12 * np.abs(Asym).max()
    assert np.abs(xs - w).max() <= 1e-6 * np.abs(w).max()
    assert np.abs(orc.interp_eval(x, xs, xe, phs, deg) - v).max() <= 1e-10 * np.abs(v).max()


def test_franke_halton_10k(orc):
    """interpolation.jl:19-27 with LAPACK's dsytrf_rook (the restated unblocked routine is
    exercised at smaller sizes above)."""
    solver = orc.lapack_rook_solver()
    if solver is None:
        pytest.skip("scipy's LAPACK not found")
    x = np.stack([halton(10_000, 2), halton(10_000, 3)], 1)
    y = franke(x)
    w = orc.interp_fit(x, y, 3, 2, solver=solver)
    v = orc.interp_eval(x, w, np.array([[0.5, 0.5]]), 3, 2)
    assert abs(v[0] - franke(np.array([0.5, 0.5]))) < 1e-5
