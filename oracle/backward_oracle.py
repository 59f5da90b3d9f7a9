"""CPU restatement of the pullback of the weight build (reverse-mode sensitivities of the
weights with respect to the point positions).

TEST INFRASTRUCTURE ONLY.  This is the checker the GPU adjoint (``rbf_build_backward``) is
compared against; only ``tests/`` may import it.

It follows RadialBasisFunctions.jl v0.7.0 in the reference's own global coordinates:
  - the stencil loop and cotangent extraction: src/solve/ad_shared.jl:63-127;
  - the implicit-function rule η = A⁻¹ [ΔW; 0], ΔA = -η λᵀ (summed over operators),
    Δb = η: src/solve/backward.jl:31-58;
  - the collocation rule (RBF pairs and the polynomial block): src/solve/backward.jl:85-160;
  - the right-hand side rule b_i = ℒφ(x0, x_i), with ∂/∂x0 and ∂/∂x_i = -∂/∂x0:
    src/solve/backward.jl:163-222; the gradients of the applied operators
    src/solve/operator_second_derivatives.jl (Hessian rows for ∂, the closed forms of
    ∇(∇²φ) per PHS order, PHS1 returning 0 below r = 1e-12);
  - the polynomial right-hand side ℒp_m(x0), which depends on x0 for a partial
    (_backward_partial_polynomial_section!, src/solve/backward.jl:223-363), written here
    for any degree by differentiating the monomials.
The identity (regrid) operator, which the reference's rules do not cover, uses ∇φ for its
right-hand side.  The stencil systems are assembled by the C oracle (``orc_assemble``) and
solved with numpy's LU; the weights and the adjoint are the same solutions the reference's
Bunch-Kaufman factorisation gives, up to rounding.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

AVOID_INF = 1.0e-16  # avoid_inf(Float64), src/RadialBasisFunctions.jl:111
PHS1_ZERO_R = 1.0e-12  # src/solve/operator_second_derivatives.jl, PHS1 rows at r = 0


def grad_phi(p, D):
    """∇φ(D) for φ = r^p (∇{PHS}, src/basis/polyharmonic_spline.jl:67-70, 153-156, ...)."""
    r = np.sqrt(D @ D)
    if p == 1:
        return D / (r + AVOID_INF)
    return p * r ** (p - 2) * D


def grad_applied(p, op, od, D):
    """∂/∂x of (ℒφ)(x, x_i) at D = x - x_i."""
    if op == O.OP_IDENT:
        return grad_phi(p, D)
    r = np.sqrt(D @ D)
    e = np.zeros_like(D)
    if op == O.OP_LAP:
        if p == 1:  # ∇²φ = 2/r
            return np.zeros_like(D) if r < PHS1_ZERO_R else -2.0 * D / r ** 3
        if p == 3:  # 12 r
            return 12.0 * D / (r + AVOID_INF)
        if p == 5:  # 30 r^3
            return 90.0 * r * D
        return 280.0 * r ** 3 * D  # 56 r^5
    # first partial along od: row od of the Hessian of φ
    e[od] = 1.0
    dd = D[od]
    if p == 1:
        if r < PHS1_ZERO_R:
            return np.zeros_like(D)
        return e / r - dd * D / r ** 3
    if p == 3:
        return 3.0 * (e * r + dd * D / (r + AVOID_INF))
    if p == 5:
        return 5.0 * (e * r ** 3 + 3.0 * dd * D * r)
    return 7.0 * (e * r ** 5 + 5.0 * dd * D * r ** 3)


def _mono_deriv(exps, alpha, x):
    """∂^alpha of every monomial (rows of exps) at x."""
    out = np.ones(len(exps))
    for m, e in enumerate(exps):
        v = 1.0
        for d in range(len(x)):
            if alpha[d] > e[d]:
                v = 0.0
                break
            c = 1
            for t in range(alpha[d]):
                c *= e[d] - t
            v *= c * x[d] ** (e[d] - alpha[d])
        out[m] = v
    return out


def _grad_applied_mono(exps, op, od, x0, dim):
    """∂/∂x0_d of ℒp_m(x0): rows d, columns m."""
    G = np.zeros((dim, len(exps)))
    for d in range(dim):
        a = np.zeros(dim, dtype=int)
        a[d] += 1
        if op == O.OP_IDENT:
            G[d] = _mono_deriv(exps, a, x0)
        elif op == O.OP_D1:
            a[od] += 1
            G[d] = _mono_deriv(exps, a, x0)
        elif op == O.OP_LAP:
            for c in range(dim):
                b = a.copy()
                b[c] += 2
                G[d] += _mono_deriv(exps, b, x0)
        else:
            raise ValueError("unsupported operator")
    return G


def build_backward(data, eval_points, adjl, dim, phs, poly_deg, ops, dW):
    """Gradients (ddata, deval) of L = sum_ops sum_e sum_i dW[op, e, i] * w[op, e, i], the
    weights w in stencil (adjl) order.  dW: (len(ops), ne, k)."""
    data = np.asarray(data, np.float64)
    eval_points = np.asarray(eval_points, np.float64)
    adjl = np.asarray(adjl)
    ns, ne, k = data.shape[0], eval_points.shape[0], adjl.shape[1]
    nops = len(ops)
    exps = O.monomial_exponents(dim, poly_deg) if poly_deg >= 0 else np.zeros((0, dim), int)
    nmon = len(exps)
    n = k + nmon
    ddata = np.zeros((ns, dim))
    deval = np.zeros((ne, dim))
    for e in range(ne):
        nb = adjl[e]
        X = data[nb]
        x0 = eval_points[e]
        Au, B, st = O.assemble(dim, phs, poly_deg, ops, X, x0)
        if st != 0:
            raise ValueError("assembly failed")
        A = np.triu(Au) + np.triu(Au, 1).T
        lam = np.linalg.solve(A, B)
        rhs = np.zeros((n, nops))
        rhs[:k] = np.asarray(dW[:, e, :]).T
        eta = np.linalg.solve(A, rhs)  # A is symmetric: A^T eta = rhs
        dA = -eta @ lam.T
        db = eta
        # collocation: RBF pairs and the polynomial block
        dX = np.zeros((k, dim))
        for j in range(k):
            for i in range(j):
                g = grad_phi(phs, X[i] - X[j])
                sc = dA[i, j] + dA[j, i]
                dX[i] += sc * g
                dX[j] -= sc * g
        for i in range(k):
            for d in range(dim):
                a = np.zeros(dim, dtype=int)
                a[d] = 1
                gp = _mono_deriv(exps, a, X[i])
                dX[i, d] += np.sum((dA[i, k:] + dA[k:, i]) * gp)
        # right-hand side: RBF section, then the polynomial section
        de = np.zeros(dim)
        for q, (op, od) in enumerate(ops):
            for i in range(k):
                g = grad_applied(phs, op, od, x0 - X[i])
                de += db[i, q] * g
                dX[i] -= db[i, q] * g
            if nmon:
                de += _grad_applied_mono(exps, op, od, x0, dim) @ db[k:, q]
        np.add.at(ddata, nb, dX)
        deval[e] += de
    return ddata, deval


def loss(data, eval_points, adjl, dim, phs, poly_deg, ops, dW):
    """L = <dW, w> through the C oracle's forward build (stencil order recovered from the
    sorted CSR rows)."""
    csr = O.build(data, eval_points, adjl, dim, phs, poly_deg, ops)
    w = csr_to_stencil_order(csr, adjl)
    return float(np.sum(np.asarray(dW) * w))


def csr_to_stencil_order(csr, adjl):
    """Values of a sorted-row CSR rearranged to (nops, ne, k) stencil (adjl) order."""
    adjl = np.asarray(adjl)
    ne, k = adjl.shape
    order = np.argsort(adjl, axis=1, kind="stable")  # rank of each stencil entry in its row
    rank = np.empty_like(order)
    np.put_along_axis(rank, order, np.arange(k)[None, :].repeat(ne, 0), axis=1)
    pos = csr.row_ptr[:-1, None] + rank
    return csr.val[:, pos]
