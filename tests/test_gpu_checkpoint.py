"""Checkpoint and resume of built operators: a resumed operator applies bit-identically to the
one that was saved, and rebuilding it from its stored stencils gives the weights the original
build gave (the reference's update_weights!, src/operators/operators.jl:589-602)."""
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
    return np.random.default_rng(31).uniform(0.0, 1.0, (6000, 3))


def same_weights(a, b):
    return (torch.equal(a.row_ptr, b.row_ptr) and torch.equal(a.col, b.col) and torch.equal(a.val, b.val)
            and tuple(a.shape) == tuple(b.shape))


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_laplacian_resume(pkg, cloud, tmp_path, precision):
    op = pkg.laplacian(cloud, k=30, precision=precision)
    p = tmp_path / "lap.npz"
    pkg.save_operator(p, op)
    r = pkg.load_operator(p)
    assert same_weights(op.weights, r.weights) and r.valid_cache
    f = torch.from_numpy(np.sin(3 * cloud[:, 0]) + cloud[:, 1] * cloud[:, 2]).cuda()
    assert torch.equal(op(f), r(f))
    r.update_weights()  # rebuild from the stored stencils, points and basis
    assert same_weights(op.weights, r.weights)


def test_gradient_and_regrid_resume(pkg, cloud, tmp_path):
    g = pkg.gradient(cloud, k=20)
    pkg.save_operator(tmp_path / "g.npz", g)
    r = pkg.load_operator(tmp_path / "g.npz")
    assert isinstance(r.weights, tuple) and len(r.weights) == 3
    f = torch.from_numpy(cloud[:, 0] ** 2).cuda()
    assert torch.equal(g(f), r(f))
    r.invalidate_cache()
    r(f)  # an invalid cache rebuilds, as the original would
    assert all(same_weights(a, b) for a, b in zip(g.weights, r.weights))
    ev = np.random.default_rng(32).uniform(0.1, 0.9, (500, 3))
    rg = pkg.regrid(cloud, ev, k=20)
    pkg.save_operator(tmp_path / "rg.npz", rg)
    rr = pkg.load_operator(tmp_path / "rg.npz")
    assert rr.shape == (500, 6000) and torch.equal(rg(f), rr(f))


def test_boundary_operator_and_weights_file(pkg, cloud, tmp_path):
    X = cloud.copy()
    lo = X[:, 0] < 0.02
    X[lo, 0] = 0.0
    herm = dict(is_boundary=lo, bc=[pkg.BoundaryCondition(0.0, 1.0)] * int(lo.sum()),
                normals=np.tile([-1.0, 0.0, 0.0], (int(lo.sum()), 1)))
    op = pkg.laplacian(X, k=30, hermite=herm)
    pkg.save_operator(tmp_path / "h.npz", op)
    r = pkg.load_operator(tmp_path / "h.npz")
    r.update_weights()
    assert same_weights(op.weights, r.weights)
    pkg.save_weights(tmp_path / "w.npz", op.weights)
    assert same_weights(op.weights, pkg.load_weights(tmp_path / "w.npz"))


def test_derived_operator_is_apply_only(pkg, cloud, tmp_path):
    a = pkg.laplacian(cloud, k=20)
    b = pkg.partial(cloud, 2, 1, k=20, adjl=a.adjl)
    d = 2.0 * a - b
    pkg.save_operator(tmp_path / "d.npz", d)
    r = pkg.load_operator(tmp_path / "d.npz")
    f = torch.from_numpy(cloud[:, 2] ** 3).cuda()
    assert torch.equal(d(f), r(f))
    with pytest.raises(ValueError, match="operator algebra"):
        r.update_weights()


def test_surrogate_training_resumes_after_a_failure(pkg, tmp_path):
    """Training interrupted after its first epoch (an exception from the epoch callback) and
    resumed from the checkpoint reaches the weights of the uninterrupted run bit for bit; the
    resumed surrogate's checkpoint loads for prediction."""
    from importlib import import_module
    L = import_module(pkg.__name__ + ".learned")
    Xb, T = L.training_set(6000, 0, 20, 3, pkg.PHS(3, poly_deg=1), [(3, 0)], seed=3)
    kw = dict(hidden=(64, 64), epochs=3, batch=1024, lr=2e-3, seed=9)
    ref, hist = L.train_surrogate(Xb, T, 20, 3, **kw)

    class Crash(Exception):
        pass

    def crash(msg):
        raise Crash(msg)

    ck = tmp_path / "surrogate.npz"
    with pytest.raises(Crash):
        L.train_surrogate(Xb, T, 20, 3, checkpoint=ck, log=crash, **kw)
    got, hist2 = L.train_surrogate(Xb, T, 20, 3, checkpoint=ck, resume=ck, **kw)
    # the epoch losses are sums of float atomics: equal to rounding, the weights exactly
    assert np.allclose(hist2, hist, rtol=1e-5, atol=0.0)
    assert all(torch.equal(a, b) for a, b in zip(ref.W + ref.b + ref.m + ref.v, got.W + got.b + got.m + got.v))
    m = L.load_surrogate(ck)
    assert torch.equal(m.predict(Xb[:512]), ref.predict(Xb[:512]))
