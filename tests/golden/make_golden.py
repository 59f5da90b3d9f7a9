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


def _truth_hermite_lap_phs3_2d(P, x0, ptype, alpha, beta, normal, exps):
    """60-digit weights of the reference's Hermite formulation (src/solve/assembly.jl:251-468)
    for PHS3 in 2D with the Laplacian, the reference's Laplacian coefficient 12 r: basis
    columns alpha phi - beta dphi/dn_j at Neumann/Robin points, the symmetric rules of
    herm_entry for the rows, alpha P + beta dP/dn in the polynomial block, the normal form
    -12 (n . (x0 - x_i)) / (r + avoid_inf) in the right-hand side."""
    import mpmath
    mpmath.mp.dps = 60
    k = len(P)
    n = k + len(exps)
    ai = mpmath.mpf(1e-16)
    Pm = [[mpmath.mpf(float(v)) for v in p] for p in P]
    x0m = [mpmath.mpf(float(v)) for v in x0]
    al = [mpmath.mpf(float(v)) for v in alpha]
    be = [mpmath.mpf(float(v)) for v in beta]
    nr = [[mpmath.mpf(float(v)) for v in q] for q in normal]
    A = mpmath.zeros(n, n)
    B = mpmath.zeros(n, 1)
    for i in range(k):
        for j in range(k):
            D = [Pm[i][0] - Pm[j][0], Pm[i][1] - Pm[j][1]]
            r = mpmath.sqrt(D[0] ** 2 + D[1] ** 2)
            phi = r ** 3
            g = [3 * r * D[0], 3 * r * D[1]]
            ti, tj = ptype[i], ptype[j]
            if ti != 2 and tj != 2:
                v = phi
            else:
                di = nr[i][0] * g[0] + nr[i][1] * g[1]
                dj = nr[j][0] * g[0] + nr[j][1] * g[1]
                if ti != 2:
                    v = al[j] * phi - be[j] * dj
                elif tj != 2:
                    v = al[i] * phi + be[i] * di
                else:
                    H = [[3 * ((1 if a == b else 0) * r + D[a] * D[b] / (r + ai)) for b in range(2)] for a in range(2)]
                    d2 = sum(nr[i][a] * sum(H[a][b] * nr[j][b] for b in range(2)) for a in range(2))
                    v = al[i] * al[j] * phi - al[i] * be[j] * dj + be[i] * al[j] * di + be[i] * be[j] * d2
            A[i, j] = v
    for i in range(k):
        x, y = Pm[i]
        for m, (ex, ey) in enumerate(exps):
            pv = x ** ex * y ** ey
            if ptype[i] == 2:
                dx = ex * x ** (ex - 1) * y ** ey if ex > 0 else 0
                dy = ey * x ** ex * y ** (ey - 1) if ey > 0 else 0
                pv = al[i] * pv + be[i] * (nr[i][0] * dx + nr[i][1] * dy)
            A[i, k + m] = pv
            A[k + m, i] = pv
        D = [x0m[0] - x, x0m[1] - y]
        r = mpmath.sqrt(D[0] ** 2 + D[1] ** 2)
        b = 12 * r
        if ptype[i] == 2:
            b = al[i] * b + be[i] * (-12 * (nr[i][0] * D[0] + nr[i][1] * D[1]) / (r + ai))
        B[i] = b
    x, y = x0m
    for m, (ex, ey) in enumerate(exps):
        v = 0
        if ex >= 2:
            v += ex * (ex - 1) * x ** (ex - 2) * y ** ey
        if ey >= 2:
            v += ey * (ey - 1) * x ** ex * y ** (ey - 2)
        B[k + m] = v
    w = mpmath.lu_solve(A, B)
    return np.array([float(w[i]) for i in range(k)])


def disk_hermite_fixtures():
    """The 2D unit-disk workload at full size (bench.unit_disk: 2M jittered interior points, 5,000
    boundary points, Dirichlet upper / Neumann lower half-circle; PHS3 degree 3, k = 30): its
    interior stencils near the circle are small against their distance from the origin, so the
    reference's raw-coordinate systems are ill-conditioned (condition numbers ~1e13).  The six
    stencils where the raw-frame oracle and the local-frame oracle differ most, each stored
    self-contained (points in stencil order, Hermite data), with 60-digit truth weights and the
    raw-frame oracle's weights (stencil order)."""
    from oracle import oracle as O
    import bench
    X, isb, nrm, al, be = bench.unit_disk(2_000_000, 5_000, 104)
    adjl = O.knn(X, X, 30)
    g2b = -np.ones(len(X), dtype=np.int64)
    g2b[np.nonzero(isb)[0]] = np.arange(int(isb.sum()))
    cand = np.nonzero((np.sqrt((X ** 2).sum(1)) > 0.985) & ~isb)[0]
    h = (isb.astype(np.uint8), al, be, nrm)
    raw = O.build(X, X[cand], adjl[cand], 2, 3, 3, [(O.OP_LAP, 0)], hermite=h)
    loc = O.build(X, X[cand], adjl[cand], 2, 3, 3, [(O.OP_LAP, 0)], hermite=h, frame="local")
    rows = np.repeat(np.arange(len(cand)), np.diff(raw.row_ptr))
    num = np.zeros(len(cand))
    den = np.zeros(len(cand))
    np.maximum.at(num, rows, np.abs(raw.val[0] - loc.val[0]))
    np.maximum.at(den, rows, np.abs(loc.val[0]))
    pick = cand[np.argsort(-(num / den))[:6]]
    exps = O.monomial_exponents(2, 3)
    out = dict(points=[], eval_index=[], ptype=[], alpha=[], beta=[], normal=[], truth=[], oracle_raw=[])
    for e in pick:
        ids = adjl[e]
        assert ids[0] == e  # interior eval point: itself first
        pt = np.zeros(30, dtype=np.int8)
        a = np.zeros(30)
        b = np.zeros(30)
        nv = np.zeros((30, 2))
        for i, g in enumerate(ids):
            if isb[g]:
                q = g2b[g]
                pt[i] = 1 if (al[q] == 1 and be[q] == 0) else 2
                a[i], b[i], nv[i] = al[q], be[q], nrm[q]
        tw = _truth_hermite_lap_phs3_2d(X[ids], X[e], pt, a, b, nv, exps)
        r1 = O.build(X, X[e:e + 1], adjl[e:e + 1], 2, 3, 3, [(O.OP_LAP, 0)], hermite=h)
        inv = np.argsort(np.argsort(ids, kind="stable"), kind="stable")  # column-sorted -> stencil order
        out["points"].append(X[ids])
        out["eval_index"].append(e)
        out["ptype"].append(pt)
        out["alpha"].append(a)
        out["beta"].append(b)
        out["normal"].append(nv)
        out["truth"].append(tw)
        out["oracle_raw"].append(r1.val[0][inv])
    np.savez_compressed(os.path.join(HERE, "disk_hermite_truth.npz"), **{k: np.array(v) for k, v in out.items()})


if __name__ == "__main__":
    with open(os.path.join(HERE, "reference_known_answers.json"), "w") as f:
        json.dump(known_answers(), f, indent=1)
    oracle_fixtures()
    illcond_fixtures()
    disk_hermite_fixtures()
    print("golden fixtures written")
