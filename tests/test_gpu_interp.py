"""Global interpolation on the GPU (rbf_interp_fit / rbf_interp_eval, rbf_sytrf_rook /
rbf_sytrs_rook) against the oracle: the rook Bunch-Kaufman factors and pivots bit-exact
against the restated dsytf2_rook with its updates as fused multiply-adds (after its
interchanges are carried to the earlier factor columns, the form the GPU keeps), the solve
and the fitted weights within rounding, the
evaluation bit-exact for the same weights; the reference's own tests
(test/operators/interpolation.jl): Franke's function on 10,000 Halton points,
|interp(0.5, 0.5) - franke| < 1e-5, and the two-point PHS1 case."""
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
    return (0.75 * np.exp(-(9 * x - 2) ** 2 / 4 - (9 * y - 2) ** 2 / 4)
            + 0.75 * np.exp(-(9 * x + 1) ** 2 / 49 - (9 * y + 1) / 10)
            + 0.5 * np.exp(-(9 * x - 7) ** 2 / 4 - (9 * y - 3) ** 2 / 4)
            - 0.2 * np.exp(-(9 * x - 4) ** 2 - (9 * y - 7) ** 2))


def sym_upper_equal(a, b):
    return np.array_equal(np.triu(a), np.triu(b))


@pytest.mark.parametrize("dim,phs,deg,n", [(2, 3, 2, 600), (3, 5, 2, 400), (1, 1, 1, 300), (2, 3, -1, 250),
                                           (3, 7, 3, 300)])
def test_factor_bit_exact(pkg, orc, dim, phs, deg, n):
    rng = np.random.default_rng(dim * 10 + phs)
    x = rng.uniform(0, 1, (n, dim))
    A = np.ascontiguousarray(orc.interp_matrix(x, phs, deg))
    F0, ip0, info0 = orc.sytrf_rook_restated(A, fused=True)
    want = orc.convert_rook_factor(F0, ip0)
    F, ip, info = pkg.sytrf_rook(torch.from_numpy(A).cuda())
    assert info == info0 == 0
    assert np.array_equal(ip.cpu().numpy(), ip0)
    assert sym_upper_equal(F.cpu().numpy(), want)
    # the solve: same factors, a different summation order than dsytrs_rook
    b = rng.standard_normal(A.shape[0])
    xs = pkg.sytrs_rook(F, ip, torch.from_numpy(b).cuda()).cpu().numpy()
    xo = orc.sytrs_rook(F0, ip0, b)[:, 0]
    Asym = np.triu(A) + np.triu(A, 1).T
    # residual of the GPU solve as good as the oracle's
    ro = np.abs(Asym @ xo - b).max()
    rg = np.abs(Asym @ xs - b).max()
    assert rg <= 10 * max(ro, 1e-14 * np.abs(b).max())


def test_indefinite_and_singular(pkg, orc):
    rng = np.random.default_rng(1)
    M = rng.standard_normal((300, 300))
    A = M + M.T
    A[:, 7] = A[7, :] = 0.0
    A[100, 100] = 0.0
    F0, ip0, info0 = orc.sytrf_rook_restated(A, fused=True)
    F, ip, info = pkg.sytrf_rook(torch.from_numpy(A).cuda())
    assert info == info0 and info > 0
    assert np.array_equal(ip.cpu().numpy(), ip0)
    assert sym_upper_equal(F.cpu().numpy(), orc.convert_rook_factor(F0, ip0))
    # several right-hand sides on a nonsingular matrix
    A = M + M.T
    F, ip, info = pkg.sytrf_rook(torch.from_numpy(A).cuda())
    B = rng.standard_normal((300, 3))
    X = pkg.sytrs_rook(F, ip, torch.from_numpy(B).cuda()).cpu().numpy()
    assert np.abs(A @ X - B).max() <= 1e-9 * np.abs(B).max()


@pytest.mark.parametrize("dim,phs,deg,n", [(2, 3, 2, 800), (3, 3, 1, 600), (2, 5, 2, 500), (1, 1, 1, 200)])
def test_fit_and_eval_vs_oracle(pkg, orc, dim, phs, deg, n):
    rng = np.random.default_rng(n)
    x = rng.uniform(0, 1, (n, dim))
    y = np.sin(3 * x[:, 0]) + (x[:, 1] ** 2 if dim > 1 else 0.0)
    w0 = orc.interp_fit(x, y, phs, deg)
    I = pkg.Interpolator(torch.from_numpy(x).cuda(), y, pkg.PHS(phs, poly_deg=deg))
    w = I.coef.cpu().numpy()
    assert np.abs(w - w0).max() <= 1e-6 * np.abs(w0).max()
    xe = rng.uniform(0, 1, (3000, dim))
    v = I(xe)
    v0 = orc.interp_eval(x, w0, xe, phs, deg)
    assert np.abs(v - v0).max() <= 1e-10 * np.abs(v0).max()
    # the evaluation itself is bit-exact for the same weights
    assert np.array_equal(v, orc.interp_eval(x, w, xe, phs, deg))
    # the data are reproduced
    assert np.abs(I(x) - y).max() <= 1e-9 * np.abs(y).max()


def test_reference_franke_10k(pkg):
    x = np.stack([halton(10_000, 2), halton(10_000, 3)], 1)
    y = franke(x)
    I = pkg.Interpolator(x, y, pkg.PHS(3, poly_deg=2))
    assert abs(I(np.array([0.5, 0.5])) - franke(np.array([0.5, 0.5]))) < 1e-5
    assert np.abs(I(x[::97]) - y[::97]).max() < 1e-9
    r = repr(I)
    assert r.startswith("Interpolator\n") and "Number of points: 10000" in r
    assert r.endswith("Basis: Polyharmonic spline (r³) with degree 2 Monomial")


def test_two_point_phs1(pkg):
    I = pkg.Interpolator(np.array([[0.0], [1.0]]), np.array([0.0, 1.0]), pkg.PHS(1, poly_deg=1))
    assert abs(I(np.array([1.0])) - 1.0) <= 1.5e-8


def test_singular_systems(pkg, orc):
    """LAPACK reports only exactly zero pivots: duplicated points leave a tiny nonzero pivot
    (no error, as in the reference), points that cannot carry the polynomial block give
    exactly zero columns (SingularException, as bunchkaufman!(A, true) raises)."""
    x = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0], [1.0, 1.0], [0.5, 0.3]])
    A = np.ascontiguousarray(orc.interp_matrix(x, 3, 1))
    F0, ip0, info0 = orc.sytrf_rook_restated(A, fused=True)
    F, ip, info = pkg.sytrf_rook(torch.from_numpy(A).cuda())
    assert info == info0 == 0 and np.array_equal(ip.cpu().numpy(), ip0)
    with pytest.raises(pkg.SingularException):
        pkg.Interpolator(np.zeros((2, 2)), np.arange(2.0), pkg.PHS(3, poly_deg=1))


def test_c_abi_host_pointers(pkg, orc):
    """The entry points with host (numpy) arrays, as a ccall with Julia Vectors passes them:
    the same results as with device arrays; a malformed ipiv is rejected."""
    import ctypes
    ctx = pkg.Context.default(0)
    L, h = ctx.lib, ctx.h
    P = ctypes.c_void_p
    rng = np.random.default_rng(12)
    x = rng.uniform(0, 1, (300, 2))
    y = np.cos(2 * x[:, 0]) * x[:, 1]
    coef = np.zeros(306)
    ctx.check(L.rbf_interp_fit(h, 2, 3, 2, x.ctypes.data_as(P), 300, y.ctypes.data_as(P), coef.ctypes.data_as(P)))
    I = pkg.Interpolator(torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda(), pkg.PHS(3, poly_deg=2))
    assert np.array_equal(coef, I.coef.cpu().numpy())
    xe = rng.uniform(0, 1, (500, 2))
    out = np.zeros(500)
    ctx.check(L.rbf_interp_eval(h, 2, 3, 2, x.ctypes.data_as(P), 300, coef.ctypes.data_as(P), xe.ctypes.data_as(P), 500,
                                out.ctypes.data_as(P)))
    assert np.array_equal(out, I(xe))
    # dense factorisation and solve on host arrays (column-major)
    A = np.asfortranarray(orc.interp_matrix(x, 3, 2))
    ipiv = np.zeros(306, dtype=np.int32)
    info = ctypes.c_int64(-1)
    ctx.check(L.rbf_sytrf_rook(h, 306, A.ctypes.data_as(P), 306, ipiv.ctypes.data_as(P), ctypes.byref(info)))
    F0, ip0, _ = orc.sytrf_rook_restated(orc.interp_matrix(x, 3, 2), fused=True)
    assert info.value == 0 and np.array_equal(ipiv, ip0)
    assert np.array_equal(np.triu(A), np.triu(orc.convert_rook_factor(F0, ip0)))
    b = np.asfortranarray(np.r_[y, np.zeros(6)].reshape(306, 1))
    ctx.check(L.rbf_sytrs_rook(h, 306, 1, A.ctypes.data_as(P), 306, ipiv.ctypes.data_as(P), b.ctypes.data_as(P), 306))
    assert np.abs(b[:, 0] - coef).max() <= 1e-9 * np.abs(coef).max()
    bad = ipiv.copy()
    bad[5] = 400
    with pytest.raises(ValueError, match="ipiv"):
        ctx.check(L.rbf_sytrs_rook(h, 306, 1, A.ctypes.data_as(P), 306, bad.ctypes.data_as(P), b.ctypes.data_as(P),
                                   306))
