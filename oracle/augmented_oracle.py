"""CPU restatement of the normal-derivative-augmented Hermite stencils (test infrastructure: only
the tests and the benchmark's comparisons use it).

The reference's Hermite stencils (src/solve/assembly.jl:251-468) keep one unknown per stencil
point and replace a Neumann/Robin point's basis column by alpha phi + beta dphi/dn, so the
system stays (k + nmon) x (k + nmon).  The augmented formulation -- no counterpart in the
reference -- gives every Neumann/Robin stencil point two unknowns, the value u_j and the normal
derivative (du/dn)_j: a second basis function d/dn_j phi(x, x_j) and a normal-derivative
collocation condition at x_j, so a stencil with m such points has (k + m + nmon) unknowns
(Hermite-Birkhoff interpolation).  It is assembled from the reference's own pieces, the PHS
kernel, its gradient and Hessian, the operator's normal form (`(op::L)(x, xi, n)`,
polynomial_spline.jl) and the monomials' normal derivatives:

    A[i][l]       = phi(x_i - x_l)                         value rows, value columns
    A[i][k+j]     = -n_j . grad phi(x_i - x_j)             value rows, derivative columns
    A[k+m][k+j]   = -n_m^T Hess phi(x_m - x_j) n_j          derivative rows and columns
    P rows        = p(x_i); n_m . grad p(x_m)
    b             = (L phi)(x0 - x_i); L applied to d/dn_j phi at x0 (the normal form); L p(x0)

Dirichlet eval points keep the reference's identity row; every other eval point (interior and
Neumann/Robin) gets the operator's weights on u at its k stencil points and on du/dn at its m
Neumann/Robin points, the latter in the columns ns + b (b the point's boundary ordinal).  Each
stencil is assembled in its local frame (centred at the eval point, scaled by the power of two
above its radius: value weights scale by s^-q, derivative weights by s^(1-q)) and solved in
FP64.  PHS 3, 5 and 7 (phi = r has no normal derivative at r = 0).
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

ORDER = {O.OP_IDENT: 0, O.OP_D1: 1, O.OP_D2: 2, O.OP_LAP: 2}


def stencil_augmented(phs, deg, ops, X, x0, nr, normals):
    """Weights of one augmented stencil in its local frame.  X: k x dim stencil points (raw),
    x0: eval point, nr: stencil positions of the Neumann/Robin points, normals: their unit
    normals (len(nr) x dim).  Returns (value weights k x nops, derivative weights m x nops), both
    in raw units."""
    X = np.asarray(X, dtype=np.float64)
    k, dim = X.shape
    x0 = np.asarray(x0, dtype=np.float64)
    r2 = ((X - x0) ** 2).sum(1).max()
    es = int(np.frexp(np.sqrt(r2))[1]) if r2 > 0 else 0
    L = np.ldexp(X - x0, -es)
    z = np.zeros(dim)
    m = len(nr)
    e = O.monomial_exponents(dim, deg) if deg >= 0 else np.zeros((0, dim), dtype=np.int32)
    nmon = len(e)
    n = k + m + nmon
    A = np.zeros((n, n))
    B = np.zeros((n, len(ops)))
    for i in range(k):
        for l in range(k):
            A[i, l] = O.phs_phi(phs, L[i], L[l])
        for j, pj in enumerate(nr):
            v = -normals[j] @ O.phs_grad(phs, L[i], L[pj])
            A[i, k + j] = v
            A[k + j, i] = v
    for a, pa in enumerate(nr):
        for b, pb in enumerate(nr):
            A[k + a, k + b] = -normals[a] @ O.phs_hess(phs, L[pa], L[pb]) @ normals[b]
    if nmon:
        for i in range(k):
            A[i, k + m:] = O.mono_op(dim, deg, O.OP_IDENT, 0, L[i])
        for a, pa in enumerate(nr):
            A[k + a, k + m:] = O.mono_normal(dim, deg, normals[a], L[pa])
        A[k + m:, :k + m] = A[:k + m, k + m:].T
    for q, (op, od) in enumerate(ops):
        for i in range(k):
            B[i, q] = O.phs_op(phs, op, od, z, L[i])
        for j, pj in enumerate(nr):
            B[k + j, q] = O.phs_op_normal(phs, op, od, z, L[pj], normals[j])
        if nmon:
            B[k + m:, q] = O.mono_op(dim, deg, op, od, z)
    W = np.linalg.solve(A, B)
    sq = np.array([float(ORDER[op]) for op, _ in ops])
    return W[:k] * 2.0 ** (-es * sq), W[k:k + m] * 2.0 ** (es * (1 - sq))


def build_augmented(data, adjl, dim, phs, deg, ops, hermite, rows=None):
    """The augmented build on data points = eval points (rows: the eval rows to build, all by
    default).  hermite = (is_boundary per point, alpha, beta, normals per boundary point).
    Returns (row_ptr, col, val[nops][nnz]) with rows sorted by column: the value columns
    (data indices) then the derivative columns (ns + boundary ordinal)."""
    data = np.asarray(data, dtype=np.float64)
    adjl = np.asarray(adjl)
    ns = len(data)
    isb, al, be, nrm = hermite
    isb = np.asarray(isb).astype(bool)
    g2b = -np.ones(ns, dtype=np.int64)
    g2b[np.nonzero(isb)[0]] = np.arange(int(isb.sum()))
    dirichlet = np.zeros(ns, dtype=bool)
    dirichlet[isb] = (np.asarray(al) == 1.0) & (np.asarray(be) == 0.0)
    rows = np.arange(len(adjl)) if rows is None else np.asarray(rows)
    row_ptr = [0]
    cols, vals = [], []
    for e in rows:
        if dirichlet[e]:
            cols.append(np.array([e]))
            vals.append(np.ones((1, len(ops))))
            row_ptr.append(row_ptr[-1] + 1)
            continue
        ids = adjl[e]
        nr = [i for i, g in enumerate(ids) if isb[g] and not dirichlet[g]]
        normals = np.array([nrm[g2b[ids[i]]] for i in nr]).reshape(len(nr), dim)
        wv, wd = stencil_augmented(phs, deg, ops, data[ids], data[e], nr, normals)
        c = np.concatenate([ids, ns + g2b[ids[nr]]]) if nr else np.asarray(ids)
        v = np.concatenate([wv, wd]) if nr else wv
        o = np.argsort(c, kind="stable")
        cols.append(c[o])
        vals.append(v[o])
        row_ptr.append(row_ptr[-1] + len(c))
    return np.array(row_ptr, dtype=np.int64), np.concatenate(cols).astype(np.int32), np.concatenate(vals).T.copy()
