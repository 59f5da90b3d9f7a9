"""Writes the golden fixtures under tests/golden/.

1. reference_known_answers.json -- the reference's own known-answer tests, restated as
   data (each block cites the reference test it comes from, RadialBasisFunctions.jl
   v0.7.0).  Values are the literal expressions of those tests evaluated in float64.
2. oracle_small_*.npz -- oracle outputs on small seeded inputs (stencils, CSR structure
   and weights) that the GPU parity tests compare against.  They are produced by the CPU
   oracle, itself pinned by tests/test_oracle_pins.py against (1) and against LAPACK.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

s5 = math.sqrt(5.0)


def known_answers():
    return {
        "source": "RadialBasisFunctions.jl v0.7.0 test suite",
        # test/basis/polyharmonic_spline.jl:22-245 : x1=(1,2), x2=(2,4), derivatives in dim 1
        "phs": [
            {"n": 1, "x1": [1.0, 2.0], "x2": [2.0, 4.0], "cite": "test/basis/polyharmonic_spline.jl:34-45",
             "values": {"phi": s5, "d1": -1 / s5, "grad": [-1 / s5, -2 / s5], "d2": 4 / (5 * s5)}},
            {"n": 3, "x1": [1.0, 2.0], "x2": [2.0, 4.0], "cite": "test/basis/polyharmonic_spline.jl:101-112",
             "values": {"phi": s5 ** 3, "d1": -3 * s5, "grad": [-3 * s5, -6 * s5], "d2": 18 / s5}},
            {"n": 5, "x1": [1.0, 2.0], "x2": [2.0, 4.0], "cite": "test/basis/polyharmonic_spline.jl:168-179",
             "values": {"phi": s5 ** 5, "d1": -25 * s5, "grad": [-25 * s5, -50 * s5], "d2": 40 * s5}},
            {"n": 7, "x1": [1.0, 2.0], "x2": [2.0, 4.0], "cite": "test/basis/polyharmonic_spline.jl:234-245",
             "values": {"phi": s5 ** 7, "d1": -175 * s5, "grad": [-175 * s5, -350 * s5], "d2": 350 * s5}},
        ],
        # test/basis/monomial.jl:105-190
        "monomial": [
            {"dim": 2, "deg": 2, "x": [2.0, 3.0], "cite": "test/basis/monomial.jl:105-121",
             "values": {"P": [1, 2, 3, 6, 4, 9], "d1_1": [0, 1, 0, 3, 4, 0], "d1_2": [0, 0, 1, 2, 0, 6],
                        "d2_1": [0, 0, 0, 0, 2, 0], "d2_2": [0, 0, 0, 0, 0, 2], "lap": [0, 0, 0, 0, 2, 2]}},
            {"dim": 2, "deg": 3, "x": [2.0, 3.0], "cite": "test/basis/monomial.jl:123-140",
             "values": {"P": [8, 12, 4, 18, 6, 2, 27, 9, 3, 1], "d1_1": [12, 12, 4, 9, 3, 1, 0, 0, 0, 0],
                        "d1_2": [0, 4, 0, 12, 2, 0, 27, 6, 1, 0], "d2_1": [12, 6, 2, 0, 0, 0, 0, 0, 0, 0],
                        "d2_2": [0, 0, 0, 4, 0, 0, 18, 2, 0, 0], "lap": [12, 6, 2, 4, 0, 0, 18, 2, 0, 0]}},
            {"dim": 3, "deg": 0, "x": [2.0, 3.0, 4.0], "cite": "test/basis/monomial.jl:142-158",
             "values": {"P": [1], "d1_1": [0], "d2_2": [0], "lap": [0]}},
            {"dim": 3, "deg": 1, "x": [2.0, 3.0, 4.0], "cite": "test/basis/monomial.jl:160-176",
             "values": {"P": [1, 2, 3, 4], "d1_1": [0, 1, 0, 0], "d1_2": [0, 0, 1, 0], "d1_3": [0, 0, 0, 1],
                        "d2_1": [0, 0, 0, 0], "lap": [0, 0, 0, 0]}},
            {"dim": 3, "deg": 2, "x": [2.0, 3.0, 4.0], "cite": "test/basis/monomial.jl:178-195",
             "values": {"P": [1, 2, 3, 4, 6, 8, 12, 4, 9, 16], "d1_1": [0, 1, 0, 0, 3, 4, 0, 4, 0, 0],
                        "d1_2": [0, 0, 1, 0, 2, 0, 4, 0, 6, 0], "d1_3": [0, 0, 0, 1, 0, 2, 3, 0, 0, 8],
                        "d2_1": [0, 0, 0, 0, 0, 0, 0, 2, 0, 0], "d2_2": [0, 0, 0, 0, 0, 0, 0, 0, 2, 0],
                        "d2_3": [0, 0, 0, 0, 0, 0, 0, 0, 0, 2], "lap": [0, 0, 0, 0, 0, 0, 0, 2, 2, 2]}},
        ],
        # test/solve/hermite_stencil.jl:108-158 (1D, points 0, 0.5, 1; MonomialBasis(1,1))
        "hermite_poly_rows": [
            {"cite": "test/solve/hermite_stencil.jl:131-145 (Neumann)", "points": [[0.0], [0.5], [1.0]],
             "ptype": [0, 1, 2], "alpha": [0.0, 1.0, 0.0], "beta": [0.0, 0.0, 1.0],
             "normals": [[0.0], [0.0], [1.0]], "rows": [[1.0, 0.0], [1.0, 0.5], [0.0, 1.0]]},
            {"cite": "test/solve/hermite_stencil.jl:147-157 (Robin 0.5,0.5)", "points": [[0.0], [0.5], [1.0]],
             "ptype": [0, 1, 2], "alpha": [0.0, 1.0, 0.5], "beta": [0.0, 0.0, 0.5],
             "normals": [[0.0], [0.0], [1.0]], "rows": [[1.0, 0.0], [1.0, 0.5], [0.5, 1.0]]},
        ],
        # test/solve.jl:7-47
        "collocation_3pt": {
            "cite": "test/solve.jl:7-47", "x": [[1.0, 2.0], [2.0, 1.0], [1.5, 0.0]], "eval_point": [0.0, 0.0],
            "rbf_pairs": [[0, 1], [0, 2], [1, 2]],
            "rbf_values": [math.sqrt(2.0) ** 3, math.sqrt(0.25 + 4.0) ** 3, math.sqrt(0.25 + 1.0) ** 3],
        },
        # test/hermite.jl:25-139: 12-point domain, PHS(3; poly_deg=2), default k = 12
        "hermite_12pt": {
            "cite": "test/hermite.jl:25-139",
            "points": [[0.0, 0.0], [0.15, 0.1], [0.2, 0.25], [0.3, 0.15], [0.4, 0.3], [0.5, 0.2],
                       [0.6, 0.35], [0.7, 0.25], [0.75, 0.15], [0.85, 0.3], [0.9, 0.2], [1.0, 0.0]],
            "is_boundary": [1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1],
            "normals": [[1.0, 0.0], [-1.0, 0.0]],
            "cases": {
                "dirichlet": {"alpha": [1.0, 1.0], "beta": [0.0, 0.0], "u": "x**2 + y**2", "lap": 4.0},
                "neumann": {"alpha": [0.0, 0.0], "beta": [1.0, 1.0], "u": "y**2", "lap": 2.0},
                "mixed": {"alpha": [1.0, 0.0], "beta": [0.0, 1.0], "u": "y**2", "lap": 2.0},
                "robin": {"alpha": [1.0, 2.0], "beta": [1.0, 3.0], "u": "y**2", "lap": 2.0},
            },
        },
    }


def oracle_fixtures():
    from oracle import oracle as O
    O.compile_oracle()
    out = {}
    # 2D PHS3 deg2 k=20 Laplacian (the CPU-runnable configuration, at 2,000 points)
    rng = np.random.default_rng(20260101)
    X = rng.uniform(0, 1, (2000, 2))
    adjl = O.knn(X, X, 20)
    W = O.build(X, X, adjl, 2, 3, 2, [(O.OP_LAP, 0)])
    np.savez_compressed(os.path.join(HERE, "oracle_small_lap2d.npz"), points=X, adjl=adjl,
                        row_ptr=W.row_ptr, col=W.col, val=W.val)
    # 3D PHS5 deg2 k=40, gradient + Laplacian on a jittered 12^3 lattice
    rng = np.random.default_rng(20260102)
    g = (np.stack(np.meshgrid(*[np.arange(12)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) / 12
    X = g + rng.uniform(-0.3, 0.3, g.shape) / 12
    adjl = O.knn(X, X, 40)
    ops = [(O.OP_D1, 0), (O.OP_D1, 1), (O.OP_D1, 2), (O.OP_LAP, 0)]
    W = O.build(X, X, adjl, 3, 5, 2, ops)
    np.savez_compressed(os.path.join(HERE, "oracle_small_grad_lap3d.npz"), points=X, adjl=adjl,
                        row_ptr=W.row_ptr, col=W.col, val=W.val)
    # 3D regrid PHS3 deg1 k=20
    rng = np.random.default_rng(20260103)
    S = rng.uniform(0, 1, (3000, 3))
    T = np.clip(np.concatenate([rng.uniform(0, 1, (500, 3)), 0.5 + 0.05 * rng.standard_normal((500, 3))]), 0, 1)
    adjl = O.knn(S, T, 20)
    W = O.build(S, T, adjl, 3, 3, 1, [(O.OP_IDENT, 0)])
    np.savez_compressed(os.path.join(HERE, "oracle_small_regrid3d.npz"), src=S, tgt=T, adjl=adjl,
                        row_ptr=W.row_ptr, col=W.col, val=W.val)


def _truth_d2(P, x0, phs, deg, dim):
    """Weights of d^2/dx_1^2 on one stencil with every entry evaluated in 80-digit arithmetic
    from the double coordinates (the exact answer the FP64 builds approximate)."""
    import mpmath
    from oracle import oracle as O
    mpmath.mp.dps = 80
    k = len(P)
    ex = O.monomial_exponents(dim, deg)
    nm = len(ex)
    n = k + nm
    Pm = [[mpmath.mpf(float(v)) for v in p] for p in P]
    x0m = [mpmath.mpf(float(v)) for v in x0]
    A = mpmath.zeros(n, n)
    b = mpmath.zeros(n, 1)
    r = lambda a, c: mpmath.sqrt(sum((a[d] - c[d]) ** 2 for d in range(dim)))
    for i in range(k):
        for j in range(k):
            A[i, j] = r(Pm[i], Pm[j]) ** phs
        for m in range(nm):
            v = mpmath.mpf(1)
            for d in range(dim):
                v *= Pm[i][d] ** int(ex[m][d])
            A[i, k + m] = v
            A[k + m, i] = v
    for i in range(k):
        rr = r(x0m, Pm[i])
        dx = x0m[0] - Pm[i][0]
        b[i] = phs * rr ** (phs - 2) + phs * (phs - 2) * rr ** (phs - 4) * dx ** 2 if rr != 0 else 0
    for m in range(nm):
        e = [int(v) for v in ex[m]]
        c = e[0] * (e[0] - 1)
        if c == 0:
            continue
        v = mpmath.mpf(c)
        for d in range(dim):
            v *= x0m[d] ** (e[d] - (2 if d == 0 else 0))
        b[k + m] = v
    x = mpmath.lu_solve(A, b)
    return np.array([float(x[i]) for i in range(k)])


def illcond_fixtures():
    """Stencils with near-coincident points (i.i.d. clouds), where the raw-coordinate
    reference arithmetic loses digits: the 4 stencils of each cloud where the oracle and a
    scaled-coordinate FP64 solve disagree most, with high-precision truth weights."""
    from oracle import oracle as O
    out = {}
    for name, (phs, deg, dim, k, n, seed) in {"d1_1d_phs3": (3, 2, 1, 7, 1500, 321),
                                              "d2_2d_phs7": (7, 2, 2, 20, 1500, 722)}.items():
        X = np.random.default_rng(seed).uniform(0, 1, (n, dim))
        adjl = O.knn(X, X, k)
        W = O.build(X, X, adjl, dim, phs, deg, [(O.OP_D2, 0)])
        dis = np.zeros(n)
        for e in range(n):
            P = X[adjl[e]]
            D = P - X[e]
            s = 2.0 ** np.ceil(np.log2(np.sqrt((D ** 2).sum(1)).max()))
            As, Bs, _ = O.assemble(dim, phs, deg, [(O.OP_D2, 0)], D / s, np.zeros(dim))
            S = np.triu(As) + np.triu(As, 1).T
            ws = np.linalg.solve(S, Bs[:, 0])[:k] / s ** 2
            wo = W.val[0, W.row_ptr[e]:W.row_ptr[e + 1]]
            dis[e] = np.abs(ws[np.argsort(adjl[e], kind="stable")] - wo).max() / np.abs(wo).max()
        rows = np.argsort(-dis)[:4]
        truth = np.zeros((4, k))
        for t, e in enumerate(rows):
            tw = _truth_d2(X[adjl[e]], X[e], phs, deg, dim)
            truth[t] = tw[np.argsort(adjl[e], kind="stable")]  # column-sorted like the CSR row
        out[name] = dict(points=X, adjl=adjl, rows=rows, truth=truth,
                         oracle=np.stack([W.val[0, W.row_ptr[e]:W.row_ptr[e + 1]] for e in rows]),
                         spec=np.array([phs, deg, dim, k]))
    np.savez_compressed(os.path.join(HERE, "illcond_truth.npz"),
                        **{f"{nm}__{key}": v for nm, d in out.items() for key, v in d.items()})


if __name__ == "__main__":
    with open(os.path.join(HERE, "reference_known_answers.json"), "w") as f:
        json.dump(known_answers(), f, indent=1)
    oracle_fixtures()
    illcond_fixtures()
    print("golden fixtures written")
