"""The headline workload's shape against the oracle: 3D points i.i.d. uniform in the unit cube,
PHS3 with degree-2 polynomials, k = 30 (40 x 40 saddle-point systems), the Laplacian.

Every build path the headline runs through is compared with the oracle's weights (the
reference algorithm: raw-coordinate assembly, rook Bunch-Kaufman): the plain FP64 build, the
FP32-factorised FP64-refined build (the split-row register kernel for 40-row systems), the
learned + refined build seeded by a trained surrogate, and the kernel that finishes the stencils
the split-row kernel hands over (boundary stencils with Hermite rows, refinements that do not
reach tolerance).  Bars: neighbour lists and CSR structure bit-exact; weights within 1e-8 per
row (max-norm, relative); applied results within 1e-10 relative (the reference's Float64
weights, src/solve/assembly.jl:201-222; Float32-vs-Float64 comparison of test/float32.jl)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N = 20_000
K = 30
W_TOL = 1e-8
APPLY_TOL = 1e-10


@pytest.fixture(scope="module")
def pkg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    p = g.load_package()
    from importlib import import_module
    p.learned = import_module(p.__name__ + ".learned")
    return p


@pytest.fixture(scope="module")
def cloud(pkg, orc):
    X = np.random.default_rng(4242).uniform(0.0, 1.0, (N, 3))
    adjl = orc.knn(X, X, K)
    Xd = torch.from_numpy(X).cuda()
    got = pkg.find_neighbors(Xd, k=K).cpu().numpy()
    assert np.array_equal(got, adjl), "kNN differs from the oracle"
    ref = orc.build(X, X, adjl, 3, 3, 2, [(orc.OP_LAP, 0)])
    return X, Xd, adjl, ref


def row_rel_err(row_ptr, v, vref):
    rows = np.repeat(np.arange(len(row_ptr) - 1), np.diff(row_ptr))
    num = np.zeros(len(row_ptr) - 1)
    den = np.zeros(len(row_ptr) - 1)
    np.maximum.at(num, rows, np.abs(v - vref))
    np.maximum.at(den, rows, np.abs(vref))
    ok = den > 0
    return float((num[ok] / den[ok]).max())


def check(W, ref, X, op_index=0):
    assert np.array_equal(W.row_ptr.cpu().numpy(), ref.row_ptr)
    assert np.array_equal(W.col.cpu().numpy(), ref.col)
    err = row_rel_err(ref.row_ptr, W.val.cpu().numpy(), ref.val[op_index])
    assert err <= W_TOL, f"row-relative weight error {err:.3e} > {W_TOL}"
    f = np.sin(4 * X[:, 0]) * np.cos(3 * X[:, 1]) * np.exp(X[:, 2])
    y = W.apply(torch.from_numpy(f).cuda()).cpu().numpy()
    import oracle.oracle as O
    yr = O.spmm(ref, f, op_index)
    assert np.abs(y - yr).max() <= APPLY_TOL * np.abs(yr).max()
    return err


def test_fp64_build(pkg, cloud):
    X, Xd, adjl, ref = cloud
    W = pkg.build_weights([(3, 0)], Xd, None, torch.from_numpy(adjl).cuda(), pkg.PHS(3, poly_deg=2))[0]
    check(W, ref, X)


def test_fp32_refined_split_kernel(pkg, cloud):
    X, Xd, adjl, ref = cloud
    st = pkg._native.BuildStats()
    W, status = pkg.build_weights([(3, 0)], Xd, None, torch.from_numpy(adjl).cuda(), pkg.PHS(3, poly_deg=2),
                                  precision="fp32_refined", stats=st, return_status=True)
    W = W[0]
    check(W, ref, X)
    assert int(st.n_stencils) == N
    # refinement reaches tolerance on almost every stencil of this distribution
    assert int(st.n_fallback) <= N // 100
    assert 1.5 <= float(st.n_residuals) / N <= 3.0
    # the sliced-ELL copy the build writes beside the CSR applies the same operator
    Ws = pkg.build_weights([(3, 0)], Xd, None, torch.from_numpy(adjl).cuda(), pkg.PHS(3, poly_deg=2),
                           precision="fp32_refined", sell=True)[0]
    assert Ws.sell is not None
    check(Ws, ref, X)


def test_deferred_kernel_on_failed_refinements(pkg, cloud):
    """A tolerance no refinement reaches: the split-row kernel hands every stencil to the
    deferred kernel, whose own refinement fails as well and whose FP64 fallback solves it."""
    X, Xd, adjl, ref = cloud
    st = pkg._native.BuildStats()
    W, status = pkg.build_weights([(3, 0)], Xd, None, torch.from_numpy(adjl).cuda(), pkg.PHS(3, poly_deg=2),
                                  precision="fp32_refined", tol=1e-30, stats=st, return_status=True)
    check(W[0], ref, X)
    s = status.cpu().numpy()
    assert (s == 3).sum() >= N * 0.99, np.unique(s, return_counts=True)
    assert int(st.n_fallback) == int((s == 3).sum())


@pytest.fixture(scope="module")
def bcloud(pkg, orc):
    """The same cloud with the points within 0.02 of the faces x = 0 and x = 1 moved onto them:
    Neumann boundary points (outward normal -x) on x = 0, Dirichlet ones on x = 1."""
    X = np.random.default_rng(4242).uniform(0.0, 1.0, (N, 3))
    lo, hi = X[:, 0] < 0.02, X[:, 0] > 0.98
    X[lo, 0], X[hi, 0] = 0.0, 1.0
    isb = lo | hi
    nb = int(isb.sum())
    alpha = np.where(hi[isb], 1.0, 0.0)
    beta = np.where(hi[isb], 0.0, 1.0)
    normals = np.zeros((nb, 3))
    normals[:, 0] = np.where(hi[isb], 1.0, -1.0)
    adjl = orc.knn(X, X, K)
    ref = orc.build(X, X, adjl, 3, 3, 2, [(orc.OP_LAP, 0)], hermite=(isb.astype(np.uint8), alpha, beta, normals))
    assert (ref.status == 2).sum() == int(hi.sum()) and (ref.status == 0).sum() == N - int(hi.sum())
    herm = dict(is_boundary=isb, bc=[pkg.BoundaryCondition(a, b) for a, b in zip(alpha, beta)], normals=normals)
    return X, torch.from_numpy(X).cuda(), torch.from_numpy(adjl).cuda(), ref, herm, hi, isb


def check_quadratic(W, X, isb, lo, refined=False):
    """Laplacian of u = |x|^2 + 1 (du/dn = 0 on x = 0) is 6 at every interior eval point.  FP64
    weights meet it to 1e-8; refined weights carry the error the refinement accepts, at most its
    enforced contraction (1e-3) times its tolerance (1e-9) relative, so their bar adds
    1e-12 sum |w_j u_j| per row."""
    u = (X ** 2).sum(1) + 1.0
    u[lo] = 0.0  # Neumann data at the x = 0 points
    y = W.apply(torch.from_numpy(u).cuda()).cpu().numpy()
    bar = np.full(len(X), 1e-8)
    if refined:
        rp, col, val = W.row_ptr.cpu().numpy(), W.col.cpu().numpy(), W.val.cpu().numpy()
        wu = np.zeros(len(X))
        np.add.at(wu, np.repeat(np.arange(len(X)), np.diff(rp)), np.abs(val * u[col]))
        bar += 1e-12 * wu
    assert (np.abs(y - 6.0) <= bar)[~isb].all()


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_boundary_stencils(pkg, bcloud, precision):
    """Hermite rows (Neumann neighbours) and Dirichlet identity rows in the 40-row build: the
    split-row kernel defers every boundary stencil to the general refined solve."""
    X, Xd, a, ref, herm, hi, isb = bcloud
    W, status = pkg.build_weights([(3, 0)], Xd, None, a, pkg.PHS(3, poly_deg=2), hermite=herm,
                                  precision=precision, return_status=True)
    check(W[0], ref, X)
    s = status.cpu().numpy()
    assert (s == 2).sum() == int(hi.sum())  # Dirichlet eval rows: identity
    check_quadratic(W[0], X, isb, isb & ~hi, refined=precision != "fp64")


@pytest.fixture(scope="module")
def trained(pkg):
    L = pkg.learned
    basis = pkg.PHS(3, poly_deg=2)
    Xb, T = L.training_set(60_000, 60_000, K, 3, basis, [(3, 0)], seed=77)
    model, _ = L.train_surrogate(Xb, T, K, 3, hidden=(128, 128, 128), epochs=3, batch=2048, lr=2e-3)
    return model


def test_learned_build(pkg, orc, cloud, trained):
    """The learned + refined build (a surrogate trained on solver stencils seeds the split-row
    kernel) meets the same bar against the oracle, interior and boundary stencils alike."""
    X, Xd, adjl, ref = cloud
    st = pkg._native.BuildStats()
    W = pkg.learned.build_learned(trained, [(3, 0)], Xd, torch.from_numpy(adjl).cuda(), pkg.PHS(3, poly_deg=2),
                                  stats=st)[0]
    check(W, ref, X)
    assert 0.0 < float(st.seed_rel_err_mean) < 1.0

def test_learned_build_boundary(pkg, bcloud, trained):
    X, Xd, a, ref, herm, hi, isb = bcloud
    seed = trained.predict(trained.features(Xd, None, a))
    Wb = pkg.build_weights([(3, 0)], Xd, None, a, pkg.PHS(3, poly_deg=2), hermite=herm, precision="learned",
                           seed=seed)[0]
    check(Wb, ref, X)
    check_quadratic(Wb, X, isb, isb & ~hi, refined=True)


def test_what_the_trained_surrogate_gains(pkg, cloud, trained):
    """What training the surrogate gains over the method without it, on held-out stencils of the
    headline shape.  The solver judges each seed by its first FP32-refined correction,
    |x1 - seed| / |x1| (the seed's relative error): training must cut it well below the untrained
    network's.  The work of the refinement is not reduced by any seed: its first FP32 solve lands
    at the FP32 floor (about cond * 2^-24) from any start, so the FP64 residuals per stencil stay
    those of the unseeded build up to the seeded start's own residual on the stencils where the
    seed is worse than zero (measured 4-5 % more; asserted within 10 %), and every build meets
    the 1e-8 bar."""
    X, Xd, adjl, ref = cloud
    a = torch.from_numpy(adjl).cuda()
    L = pkg.learned
    untrained = L.StencilMLP(K, 3, hidden=(128, 128, 128), seed=1, out_scale=trained.out_scale)
    res = {}
    for name, model in (("trained", trained), ("untrained", untrained), ("unseeded", None)):
        st = pkg._native.BuildStats()
        if model is None:
            W = pkg.build_weights([(3, 0)], Xd, None, a, pkg.PHS(3, poly_deg=2), precision="fp32_refined", stats=st)[0]
        else:
            W = L.build_learned(model, [(3, 0)], Xd, a, pkg.PHS(3, poly_deg=2), stats=st)[0]
        check(W, ref, X)
        res[name] = (float(st.seed_rel_err_mean), float(st.n_residuals) / int(st.n_stencils))
    assert res["trained"][0] <= 0.7 * res["untrained"][0], res
    assert res["trained"][1] <= 1.10 * res["unseeded"][1], res
