"""Checkpoint and resume of built operators.

The reference keeps a built operator in memory (its weights cache, invalidated by moved points
and rebuilt by update_weights!, src/operators/operators.jl:589-602).  A long simulation here
can write the operator to disk and resume from it in another process: the weights (CSR, one
array set per operator of a tuple), the stencils, the points, the basis, the Hermite boundary
and the operator kind, in one numpy .npz file.  A resumed operator applies its stored weights
at once and rebuilds them from its stored stencils when update_weights() is called, exactly as
the original would.  Operators made by operator algebra (sums, scalings) store their weights
only: they can be applied but not rebuilt after resume."""
from __future__ import annotations

import json
import os

import numpy as np

FORMAT = "rbffd-gb300-operator-1"


def _npz(path):
    """The file name numpy writes for path: np.savez appends .npz to a name without it, and
    np.load does not, so both directions use the completed name."""
    p = os.fspath(path)
    return p if p.endswith(".npz") else p + ".npz"


def _op_spec(L):
    from . import Directional, Jacobian, Laplacian, Operators, Partial, Regrid
    if isinstance(L, Laplacian):
        return {"kind": "laplacian"}
    if isinstance(L, Partial):
        return {"kind": "partial", "order": L.order, "dim": L.dim}
    if isinstance(L, Jacobian):
        return {"kind": "jacobian", "dim": L.dim}
    if isinstance(L, Regrid):
        return {"kind": "regrid"}
    if isinstance(L, Directional):
        return {"kind": "directional"}  # the direction is stored as an array
    if isinstance(L, Operators):
        return {"kind": "operators", "parts": [_op_spec(p) for p in L.parts]}
    return {"kind": "derived", "desc": repr(L), "rank": L.rank}


def _op_from_spec(spec, v=None):
    from . import Directional, Jacobian, Laplacian, Operators, Partial, Regrid, _Combined
    kind = spec["kind"]
    if kind == "laplacian":
        return Laplacian()
    if kind == "partial":
        return Partial(spec["order"], spec["dim"])
    if kind == "jacobian":
        return Jacobian(spec["dim"])
    if kind == "regrid":
        return Regrid()
    if kind == "directional":
        return Directional(v)
    if kind == "operators":
        return Operators(*[_op_from_spec(p) for p in spec["parts"]])
    return _Combined(spec["desc"], spec["rank"])


def _host(t):
    return t.detach().cpu().numpy() if hasattr(t, "detach") else np.asarray(t)


def save_weights(path, W):
    """One CSR operator (WeightsCSR) to an .npz file."""
    np.savez(_npz(path), format=FORMAT, row_ptr=_host(W.row_ptr), col=_host(W.col), val=_host(W.val),
             shape=np.asarray(W.shape, dtype=np.int64))


def load_weights(path, ctx=None):
    """A WeightsCSR from save_weights, on the context's GPU."""
    from . import Context, WeightsCSR, _torch
    z = np.load(_npz(path), allow_pickle=False)
    if str(z["format"]) != FORMAT:
        raise ValueError(f"{path}: not an operator checkpoint of this library (format {z['format']})")
    ctx = ctx or Context.default()
    dev = _torch().device("cuda", ctx.device)
    t = lambda a: _torch().from_numpy(np.ascontiguousarray(a)).to(dev)
    return WeightsCSR(t(z["row_ptr"]), t(z["col"]), t(z["val"]), tuple(int(s) for s in z["shape"]), ctx)


def save_operator(path, op):
    """A RadialBasisOperator (its current weights, stencils, points, basis, boundary) to .npz."""
    ws = op.weights if isinstance(op.weights, tuple) else (op.weights,)
    arrays = {"format": FORMAT, "data": _host(op.data), "adjl": _host(op.adjl)}
    if op.eval_points is not op.data:
        arrays["eval_points"] = _host(op.eval_points)
    for i, W in enumerate(ws):
        arrays[f"w{i}_row_ptr"], arrays[f"w{i}_col"], arrays[f"w{i}_val"] = _host(W.row_ptr), _host(W.col), \
            _host(W.val)
        arrays[f"w{i}_shape"] = np.asarray(W.shape, dtype=np.int64)
    from . import Directional, _hermite_arrays
    if isinstance(op.L, Directional):
        arrays["direction"] = np.asarray(_host(op.L.v), dtype=np.float64)
    herm = _hermite_arrays(op.hermite, op.data.shape[0], op.data.shape[1]) if op.hermite is not None else None
    if herm is not None:
        arrays["is_boundary"], arrays["alpha"], arrays["beta"], arrays["normals"] = herm
    meta = {"op": _op_spec(op.L), "basis": {"order": op.basis.order, "poly_deg": op.basis.poly_deg}, "k": int(op.k),
            "precision": op.precision, "tuple": isinstance(op.weights, tuple), "nweights": len(ws),
            "valid_cache": bool(op.valid_cache)}
    arrays["meta"] = json.dumps(meta)
    np.savez(_npz(path), **arrays)


def load_operator(path, ctx=None):
    """Resume a RadialBasisOperator from save_operator without rebuilding its weights."""
    from . import PHS, BoundaryCondition, Context, RadialBasisOperator, WeightsCSR, _torch
    z = np.load(_npz(path), allow_pickle=False)
    if str(z["format"]) != FORMAT:
        raise ValueError(f"{path}: not an operator checkpoint of this library (format {z['format']})")
    meta = json.loads(str(z["meta"]))
    ctx = ctx or Context.default()
    torch = _torch()
    dev = torch.device("cuda", ctx.device)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    op = RadialBasisOperator.__new__(RadialBasisOperator)
    op.L = _op_from_spec(meta["op"], z["direction"] if "direction" in z.files else None)
    op.ctx = ctx
    op.data = t(z["data"])
    op.eval_points = t(z["eval_points"]) if "eval_points" in z.files else op.data
    op.basis = PHS(meta["basis"]["order"], poly_deg=meta["basis"]["poly_deg"])
    op.k = meta["k"]
    op.adjl = t(z["adjl"])
    op.hermite = None
    if "is_boundary" in z.files:
        bc = [BoundaryCondition(a, b) for a, b in zip(z["alpha"], z["beta"])]
        op.hermite = dict(is_boundary=z["is_boundary"].astype(bool), bc=bc, normals=z["normals"])
    op.precision = meta["precision"]
    ws = tuple(WeightsCSR(t(z[f"w{i}_row_ptr"]), t(z[f"w{i}_col"]), t(z[f"w{i}_val"]),
                          tuple(int(s) for s in z[f"w{i}_shape"]), ctx) for i in range(meta["nweights"]))
    op.weights = ws if meta["tuple"] else ws[0]
    op.valid_cache = meta["valid_cache"]
    if meta["op"]["kind"] == "derived":
        def _no_rebuild():
            raise ValueError("an operator made by operator algebra was stored with its weights only and cannot "
                             "be rebuilt after resume")
        op._build = _no_rebuild
    return op
