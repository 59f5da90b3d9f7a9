"""The operator checkpoint's file format on the host (no GPU): what save_operator writes for an
operator whose weights are host arrays, and that load rejects a file of another format before it
touches a device."""
import json

import numpy as np
import pytest


@pytest.fixture(scope="module")
def pkg():
    import __graft_entry__ as g
    return g.load_package()


def fake_operator(pkg, L, nw, herm=None):
    rng = np.random.default_rng(5)
    X = rng.uniform(size=(40, 2))
    adjl = rng.integers(0, 40, size=(40, 6)).astype(np.int32)
    op = pkg.RadialBasisOperator.__new__(pkg.RadialBasisOperator)
    op.L, op.data, op.eval_points, op.adjl = L, X, X, adjl
    op.basis, op.k, op.hermite, op.precision, op.valid_cache = pkg.PHS(5, poly_deg=1), 6, herm, "fp32_refined", True
    rp = np.arange(0, 241, 6, dtype=np.int64)
    ws = tuple(pkg.WeightsCSR(rp, np.sort(adjl, 1).ravel(), rng.normal(size=240) + i, (40, 40), None)
               for i in range(nw))
    op.weights = ws if nw > 1 else ws[0]
    return op


def test_scalar_operator_file(pkg, tmp_path):
    op = fake_operator(pkg, pkg.Partial(2, 1), 1)
    p = tmp_path / "lap.npz"
    pkg.save_operator(p, op)
    z = np.load(p, allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    assert meta["op"] == {"kind": "partial", "order": 2, "dim": 1}
    assert meta["basis"] == {"order": 5, "poly_deg": 1} and meta["k"] == 6 and meta["precision"] == "fp32_refined"
    assert not meta["tuple"] and meta["nweights"] == 1
    assert "eval_points" not in z.files  # data = eval points is stored once
    assert np.array_equal(z["w0_val"], op.weights.val) and np.array_equal(z["w0_col"], op.weights.col)
    assert np.array_equal(z["adjl"], op.adjl) and z["w0_shape"].tolist() == [40, 40]


def test_tuple_operator_with_boundary(pkg, tmp_path):
    isb = np.zeros(40, dtype=bool)
    isb[:3] = True
    herm = dict(is_boundary=isb, bc=[pkg.BoundaryCondition(0.0, 1.0)] * 3, normals=np.tile([1.0, 0.0], (3, 1)))
    op = fake_operator(pkg, pkg.Operators(pkg.Jacobian(), pkg.Laplacian()), 3, herm)
    p = tmp_path / "ops.npz"
    pkg.save_operator(p, op)
    z = np.load(p, allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    assert meta["op"] == {"kind": "operators", "parts": [{"kind": "jacobian", "dim": None}, {"kind": "laplacian"}]}
    assert meta["tuple"] and meta["nweights"] == 3
    for i in range(3):
        assert np.array_equal(z[f"w{i}_val"], op.weights[i].val)
    assert z["is_boundary"].sum() == 3 and z["beta"].tolist() == [1.0] * 3 and z["normals"].shape == (3, 2)


def test_load_rejects_foreign_file(pkg, tmp_path):
    p = tmp_path / "other.npz"
    np.savez(p, format="something-else", meta="{}")
    with pytest.raises(ValueError, match="not an operator checkpoint"):
        pkg.load_operator(p)
    with pytest.raises(ValueError, match="not an operator checkpoint"):
        pkg.load_weights(p)


def test_path_without_extension(pkg, tmp_path):
    """np.savez appends .npz to a bare name; saving and loading under the same bare name meet."""
    op = fake_operator(pkg, pkg.Laplacian(), 1)
    bare = tmp_path / "lap"
    pkg.save_operator(bare, op)
    assert (tmp_path / "lap.npz").exists()
    z = np.load(str(bare) + ".npz", allow_pickle=False)
    assert np.array_equal(z["w0_val"], op.weights.val)
    np.savez(tmp_path / "foreign", format="something-else", meta="{}")
    with pytest.raises(ValueError, match="not an operator checkpoint"):
        pkg.load_operator(tmp_path / "foreign")  # found under its completed name, then rejected



def test_operator_kinds_round_trip(pkg):
    """Every operator kind the front ends build is stored by kind and parameters and restored to
    the same kind, parameters and right-hand sides (what update_weights rebuilds from)."""
    from importlib import import_module
    ck = import_module(pkg.__name__ + ".checkpoint")
    kinds = [pkg.Laplacian(), pkg.Partial(1, 2), pkg.Partial(2, 3), pkg.Jacobian(3), pkg.Regrid(),
             pkg.Operators(pkg.Jacobian(), pkg.Laplacian())]
    for L in kinds:
        spec = ck._op_spec(L)
        R = ck._op_from_spec(spec)
        assert type(R) is type(L) and ck._op_spec(R) == spec
        assert R.ops(3) == L.ops(3)
    v = np.array([0.6, 0.8, 0.0])
    D = ck._op_from_spec(ck._op_spec(pkg.Directional(v)), v)
    assert isinstance(D, pkg.Directional) and np.array_equal(D.v, v) and D.ops(3) == pkg.Directional(v).ops(3)
    C = ck._op_from_spec({"kind": "derived", "desc": "2.0 * Laplacian (∇²f)", "rank": 0})
    assert repr(C) == "2.0 * Laplacian (∇²f)" and C.rank == 0
