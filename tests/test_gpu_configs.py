"""Parity at the shapes of the non-headline workloads, at sizes the oracle finishes in
seconds: the unit-disk Hermite problem (Dirichlet upper half-circle, Neumann lower, PHS3
degree 3, k = 30, one persistent batched launch) and the regrid onto a Gaussian-mixture
target cloud (PHS3 degree 1, k = 20) applied to 32 fields.  Bars as in test_gpu_parity:
structure bit-exact, weights within 1e-8 per row, applied results within 1e-10."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

W_TOL = 1e-8
APPLY_TOL = 1e-10


@pytest.fixture(scope="module")
def pkg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    return g.load_package()


def row_rel_err(row_ptr, v, vref):
    ne = len(row_ptr) - 1
    rows = np.repeat(np.arange(ne), np.diff(row_ptr))
    num = np.zeros(ne)
    den = np.zeros(ne)
    np.maximum.at(num, rows, np.abs(v - vref))
    np.maximum.at(den, rows, np.abs(vref))
    den[den == 0] = 1.0
    return float((num / den).max())


def unit_disk(n_grid, n_boundary, seed):
    """Jittered grid clipped to the open unit disk plus equispaced boundary points with
    outward normals; Dirichlet on the upper half-circle, Neumann on the lower."""
    rng = np.random.default_rng(seed)
    m = int(math.sqrt(n_grid * 4 / math.pi))
    h = 2.0 / m
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 2)
    P = -1 + (g + 0.5) * h + rng.uniform(-0.3 * h, 0.3 * h, g.shape)
    P = P[np.hypot(P[:, 0], P[:, 1]) < 1 - 0.5 * h]
    t = 2 * math.pi * (np.arange(n_boundary) + 0.5) / n_boundary
    B = np.stack([np.cos(t), np.sin(t)], 1)
    X = np.concatenate([P, B])
    isb = np.zeros(len(X), dtype=bool)
    isb[len(P):] = True
    dirichlet = B[:, 1] > 0
    alpha = np.where(dirichlet, 1.0, 0.0)
    beta = np.where(dirichlet, 0.0, 1.0)
    return X, isb, B.copy(), alpha, beta


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_unit_disk_hermite_batched(pkg, orc, precision):
    X, isb, normals, alpha, beta = unit_disk(3000, 240, seed=31)
    adjl = orc.knn(X, X, 30)
    assert np.array_equal(pkg.find_neighbors(X, k=30), adjl)
    ref = orc.build(X, X, adjl, 2, 3, 3, [(orc.OP_LAP, 0)], hermite=(isb.astype(np.uint8), alpha, beta, normals))
    bcs = [pkg.BoundaryCondition(a, b) for a, b in zip(alpha, beta)]
    herm = dict(is_boundary=isb, bc=bcs, normals=normals)
    Xd = torch.from_numpy(X).cuda()
    ap, ai = pkg.ragged_stencils(torch.from_numpy(adjl).cuda(), torch.full((len(X),), 30))
    W, status = pkg.build_weights_batched([(3, 0)], Xd, None, ap, ai, pkg.PHS(3, poly_deg=3), hermite=herm,
                                          precision=precision, tune=1, return_status=True)
    W = W[0]
    assert np.array_equal(W.row_ptr.cpu().numpy(), ref.row_ptr)
    assert np.array_equal(W.col.cpu().numpy(), ref.col)
    assert row_rel_err(ref.row_ptr, W.val.cpu().numpy(), ref.val[0]) <= W_TOL
    st = status.cpu().numpy()
    bi = np.nonzero(isb)[0]
    assert (st[bi[alpha == 1.0]] == 2).all()  # Dirichlet eval points: identity rows
    # Laplacian of u = x^2 + y^2 + 1 (= 4) with Neumann data g = du/dn = 2 x.n on the lower arc
    u = X[:, 0] ** 2 + X[:, 1] ** 2 + 1.0
    for b, i in enumerate(bi):
        if alpha[b] == 0.0:
            u[i] = 2 * X[i] @ normals[b]
    r = W.apply(u)
    if precision == "fp64":
        assert np.abs(r[~isb] - 4.0).max() < 1e-8
    else:
        # refined weights carry the error the refinement accepts: at most the contraction bound
        # it enforces (1e-3) times its tolerance (1e-9), relative, so the bar grows with
        # sum |w_j u_j|; asked for 1e-11 the same kernels meet the FP64 bar
        rows = np.repeat(np.arange(len(X)), np.diff(ref.row_ptr))
        wu = np.zeros(len(X))
        np.add.at(wu, rows, np.abs(W.val.cpu().numpy() * u[ref.col]))
        assert (np.abs(r - 4.0) <= 1e-8 + 1e-12 * wu)[~isb].all()
        Wt = pkg.build_weights_batched([(3, 0)], Xd, None, ap, ai, pkg.PHS(3, poly_deg=3), hermite=herm,
                                       precision=precision, tune=1, tol=1e-11)[0]
        assert np.abs(Wt.apply(u)[~isb] - 4.0).max() < 1e-8
    # the apply bar is on the product itself: the oracle's SpMV over the same weights
    mine = orc.CSR(W.row_ptr.cpu().numpy(), W.col.cpu().numpy(), W.val.cpu().numpy()[None], None, W.shape)
    r_ref = orc.spmm(mine, u)
    assert np.abs(r - r_ref).max() <= APPLY_TOL * np.abs(r_ref).max()


def mixture_targets(n, seed):
    rng = np.random.default_rng(seed)
    half = n // 2
    centres = rng.uniform(0.1, 0.9, (8, 3))
    G = centres[rng.integers(0, 8, n - half)] + rng.normal(0, 0.05, (n - half, 3))
    return np.clip(np.concatenate([rng.uniform(0, 1, (half, 3)), G]), 0.0, 1.0)


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_regrid_mixture_32_fields(pkg, orc, precision):
    rng = np.random.default_rng(41)
    src = rng.uniform(0, 1, (30000, 3))
    tgt = mixture_targets(12000, seed=42)
    adjl = orc.knn(src, tgt, 20)
    assert np.array_equal(pkg.find_neighbors(src, tgt, 20), adjl)
    ref = orc.build(src, tgt, adjl, 3, 3, 1, [(orc.OP_IDENT, 0)])
    W = pkg.build_weights([(0, 0)], torch.from_numpy(src).cuda(), torch.from_numpy(tgt).cuda(),
                          torch.from_numpy(adjl).cuda(), pkg.PHS(3, poly_deg=1), precision=precision)[0]
    assert np.array_equal(W.row_ptr.cpu().numpy(), ref.row_ptr)
    assert np.array_equal(W.col.cpu().numpy(), ref.col)
    assert row_rel_err(ref.row_ptr, W.val.cpu().numpy(), ref.val[0]) <= W_TOL
    # 32 seeded Fourier fields (8 modes each), column-major like a Julia Matrix
    F = np.zeros((len(src), 32))
    for f in range(32):
        kv = rng.uniform(1, 4, (8, 3))
        a = rng.normal(0, 1, 8)
        F[:, f] = (a[None, :] * np.sin(src @ kv.T)).sum(1)
    Y = W.apply(torch.from_numpy(F).cuda()).cpu().numpy()
    mine = orc.CSR(W.row_ptr.cpu().numpy(), W.col.cpu().numpy(), W.val.cpu().numpy()[None], None, W.shape)
    for f in (0, 13, 31):
        y_ref = orc.spmm(mine, F[:, f])
        assert np.abs(Y[:, f] - y_ref).max() <= APPLY_TOL * np.abs(y_ref).max()
    # degree-1 regrid reproduces a linear field
    lin = 1.0 + src @ np.array([0.3, -1.2, 2.0])
    assert np.abs(W.apply(lin) - (1.0 + tgt @ np.array([0.3, -1.2, 2.0]))).max() < 1e-8


@pytest.mark.parametrize("path", ["fp64", "fp64_lu", "fp32_refined", "batched_fp64", "batched_fp32_refined"])
def test_disk_stencils_where_the_reference_arithmetic_loses_digits(pkg, path):
    """Six interior stencils of the full-size unit disk (2M points) next to the Neumann half of
    the circle, where the reference's raw-coordinate systems are ill-conditioned (the raw-frame
    oracle is 2e-6 .. 1e-5 off the 60-digit truth, tests/golden/disk_hermite_truth.npz).  Each
    is rebuilt as a 30-point cloud; every GPU path (one-size FP64 by symmetric indefinite and by
    LU, FP32-refined, the batched launch in both precisions) is within 1e-8 of the truth."""
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "disk_hermite_truth.npz"))
    basis = pkg.PHS(3, poly_deg=3)
    for t in range(len(z["truth"])):
        P = torch.from_numpy(z["points"][t]).cuda()
        pt = z["ptype"][t]
        b = pt > 0
        herm = dict(is_boundary=b, bc=[pkg.BoundaryCondition(x, y) for x, y in zip(z["alpha"][t][b], z["beta"][t][b])],
                    normals=z["normal"][t][b])
        adjl = torch.arange(30, dtype=torch.int32, device="cuda").repeat(30, 1)
        if path.startswith("batched"):
            ap, ai = pkg.ragged_stencils(adjl, torch.full((30,), 30, device="cuda"))
            W = pkg.build_weights_batched([(3, 0)], P, None, ap, ai, basis, hermite=herm,
                                          precision=path.split("_", 1)[1], tune=0)[0]
        else:
            W = pkg.build_weights([(3, 0)], P, None, adjl, basis, hermite=herm,
                                  precision="fp64" if path.startswith("fp64") else path,
                                  flags=4 if path == "fp64_lu" else 0)[0]
        w = W.val[:30].cpu().numpy()  # row 0: the stencil's eval point; columns 0..29 in stencil order
        assert np.array_equal(W.col[:30].cpu().numpy(), np.arange(30))
        truth = z["truth"][t]
        err = np.abs(w - truth).max() / np.abs(truth).max()
        assert err <= W_TOL, (path, t, err)
