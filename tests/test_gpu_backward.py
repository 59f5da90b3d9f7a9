"""The adjoint of the weight build on the GPU (rbf_build_backward) against the oracle's
restatement of the reference's pullback (oracle/backward_oracle.py, itself pinned to finite
differences), on the reference's own AD test case (a 5 x 5 grid, k = 10, eval points = data,
loss sum(W.nzval .^ 2): test/extensions/ad_test_utils.jl, mooncake_ext.jl:82-125) and on 3D
clouds; at full size through exact invariances (translation: the gradients sum to zero;
scaling: sum_i x_i . g_i = -q L for an operator of order q)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

OP_IDENT, OP_D1, OP_D2, OP_LAP = 0, 1, 2, 3
TOL = 1e-9  # relative to the largest gradient component; FP64 solves on both sides


@pytest.fixture(scope="module")
def pkg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    return g.load_package()


@pytest.fixture(scope="module")
def bo(orc):
    from oracle import backward_oracle
    return backward_oracle


def grid_points():
    return np.array([[0.1 + 0.8 * i / 5, 0.1 + 0.8 * j / 5] for i in range(1, 6) for j in range(1, 6)])


def stencil_order(pkg, W, adjl):
    """(nops, ne, k) stencil-order copy of sorted CSR values."""
    adjl = np.asarray(adjl)
    ne, k = adjl.shape
    order = np.argsort(adjl, axis=1, kind="stable")
    rank = np.empty_like(order)
    np.put_along_axis(rank, order, np.arange(k)[None, :].repeat(ne, 0), axis=1)
    pos = W[0].row_ptr.cpu().numpy()[:-1, None] + rank
    return np.stack([w.val.cpu().numpy()[pos] for w in W])


def to_csr_order(adjl, x):
    """(nops, ne, k) stencil order -> (nops, nnz) sorted-row order."""
    adjl = np.asarray(adjl)
    ne, k = adjl.shape
    order = np.argsort(adjl, axis=1, kind="stable")
    return np.stack([np.take_along_axis(x[q], order, axis=1).reshape(-1) for q in range(x.shape[0])])


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
@pytest.mark.parametrize("phs,deg,op", [(3, 2, (OP_D1, 0)), (3, 2, (OP_LAP, 0)), (1, 1, (OP_D1, 0)),
                                        (3, 1, (OP_D1, 0)), (5, 1, (OP_D1, 0)), (7, 1, (OP_D1, 0)),
                                        (5, 2, (OP_LAP, 0)), (7, 2, (OP_LAP, 0)), (1, 1, (OP_LAP, 0)),
                                        (3, 2, (OP_D1, 1))])
def test_reference_grid_case(pkg, orc, bo, phs, deg, op, precision):
    X = grid_points()
    adjl = orc.knn(X, X, 10)
    basis = pkg.PHS(phs, poly_deg=deg)
    Xd = torch.from_numpy(X).cuda()
    W = pkg.build_weights([op], Xd, None, adjl, basis)
    w = stencil_order(pkg, W, adjl)
    dW = torch.from_numpy(2.0 * to_csr_order(adjl, w)).cuda()  # d/dW of sum(W.^2)
    gd, ge = pkg.build_weights_backward([op], Xd, None, adjl, basis, W[0].row_ptr, dW, precision=precision)
    got = (gd + ge).cpu().numpy()
    od, oe = bo.build_backward(X, X, adjl, 2, phs, deg, [op], 2.0 * w)
    want = od + oe
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()


def test_regrid_at_the_data_points(pkg, orc, bo):
    """Regrid onto the data points themselves gives the identity matrix whatever the
    positions: both gradients are rounding noise."""
    X = grid_points()
    adjl = orc.knn(X, X, 10)
    basis = pkg.PHS(5, poly_deg=2)
    Xd = torch.from_numpy(X).cuda()
    W = pkg.build_weights([(OP_IDENT, 0)], Xd, None, adjl, basis)
    gd, ge = pkg.build_weights_backward([(OP_IDENT, 0)], Xd, None, adjl, basis, W[0].row_ptr, 2.0 * W[0].val[None])
    assert float((gd + ge).abs().max()) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
@pytest.mark.parametrize("phs,ops", [(3, [(OP_LAP, 0)]), (5, [(OP_D1, 0), (OP_D1, 1), (OP_D1, 2)]),
                                     (7, [(OP_IDENT, 0)]), (3, [(OP_IDENT, 0), (OP_LAP, 0)]),
                                     (1, [(OP_D1, 2)])])
def test_cloud3d_separate_eval(pkg, orc, bo, phs, ops, precision):
    rng = np.random.default_rng(8)
    data = rng.uniform(0, 1, (400, 3))
    ev = rng.uniform(0.1, 0.9, (40, 3))
    k = 30
    adjl = orc.knn(data, ev, k)
    dW = rng.standard_normal((len(ops), len(ev), k))
    basis = pkg.PHS(phs, poly_deg=2)
    Xd, Ed = torch.from_numpy(data).cuda(), torch.from_numpy(ev).cuda()
    W = pkg.build_weights(ops, Xd, Ed, adjl, basis)
    gd, ge = pkg.build_weights_backward(ops, Xd, Ed, adjl, basis, W[0].row_ptr,
                                        torch.from_numpy(to_csr_order(adjl, dW)).cuda(), precision=precision)
    od, oe = bo.build_backward(data, ev, adjl, 3, phs, 2, ops, dW)
    assert np.abs(gd.cpu().numpy() - od).max() <= TOL * np.abs(od).max()
    assert np.abs(ge.cpu().numpy() - oe).max() <= TOL * np.abs(oe).max()


def test_stencil_order_and_local_units(pkg, orc, bo):
    """flags change the layout and units of dW the same way they change the forward values."""
    rng = np.random.default_rng(9)
    data = rng.uniform(0, 1, (300, 2))
    ev = rng.uniform(0.1, 0.9, (30, 2))
    k = 16
    adjl = orc.knn(data, ev, k)
    ops = [(OP_LAP, 0), (OP_D1, 1)]
    basis = pkg.PHS(3, poly_deg=2)
    dW = rng.standard_normal((2, len(ev), k))
    Xd, Ed = torch.from_numpy(data).cuda(), torch.from_numpy(ev).cuda()
    od, oe = bo.build_backward(data, ev, adjl, 2, 3, 2, ops, dW)
    # stencil order: dW given row by row in adjl order
    W = pkg.build_weights(ops, Xd, Ed, adjl, basis, flags=1)
    gd, ge = pkg.build_weights_backward(ops, Xd, Ed, adjl, basis, W[0].row_ptr,
                                        torch.from_numpy(dW.reshape(2, -1)).cuda(), flags=1)
    assert np.abs(gd.cpu().numpy() - od).max() <= TOL * np.abs(od).max()
    assert np.abs(ge.cpu().numpy() - oe).max() <= TOL * np.abs(oe).max()
    # local units: the values are w * 2^(es q), es the stencil's radius exponent
    r = np.sqrt(((data[adjl] - ev[:, None, :]) ** 2).sum(-1)).max(1)
    es = np.frexp(r)[1].astype(np.float64)
    order = np.array([2.0, 1.0])
    dW_glob = dW * np.exp2(es[None, :, None] * order[:, None, None])
    od2, oe2 = bo.build_backward(data, ev, adjl, 2, 3, 2, ops, dW_glob)
    W = pkg.build_weights(ops, Xd, Ed, adjl, basis, flags=3)
    gd, ge = pkg.build_weights_backward(ops, Xd, Ed, adjl, basis, W[0].row_ptr,
                                        torch.from_numpy(dW.reshape(2, -1)).cuda(), flags=3)
    assert np.abs(gd.cpu().numpy() - od2).max() <= TOL * np.abs(od2).max()
    assert np.abs(ge.cpu().numpy() - oe2).max() <= TOL * np.abs(oe2).max()


def test_autograd_function(pkg, orc):
    rng = np.random.default_rng(10)
    data = rng.uniform(0, 1, (500, 3))
    adjl = orc.knn(data, data, 20)
    basis = pkg.PHS(3, poly_deg=1)
    ops = [(OP_LAP, 0)]
    x = torch.from_numpy(data).cuda().requires_grad_(True)
    row_ptr, col, val = pkg.build_weights_differentiable(ops, x, None, adjl, basis)
    (val ** 2).sum().backward()
    W = pkg.build_weights(ops, x.detach(), None, adjl, basis)
    gd, ge = pkg.build_weights_backward(ops, x.detach(), None, adjl, basis, W[0].row_ptr, 2.0 * W[0].val[None])
    # the per-point sums are atomic (their order varies between launches)
    assert (x.grad - (gd + ge)).abs().max() <= 1e-12 * (gd + ge).abs().max()
    # separate eval points: one gradient per input
    e = torch.from_numpy(rng.uniform(0.2, 0.8, (50, 3))).cuda().requires_grad_(True)
    adj2 = orc.knn(data, e.detach().cpu().numpy(), 20)
    x.grad = None
    _, _, v2 = pkg.build_weights_differentiable([(OP_D1, 0)], x, e, adj2, basis)
    v2.sum().backward()
    assert x.grad is not None and e.grad is not None
    assert torch.isfinite(x.grad).all() and torch.isfinite(e.grad).all()


def test_rejects_unsupported(pkg, orc):
    X = torch.from_numpy(grid_points()).cuda()
    adjl = orc.knn(grid_points(), grid_points(), 10)
    basis = pkg.PHS(3, poly_deg=2)
    W = pkg.build_weights([(OP_D2, 0)], X, None, adjl, basis)
    with pytest.raises(Exception, match="adjoint"):
        pkg.build_weights_backward([(OP_D2, 0)], X, None, adjl, basis, W[0].row_ptr, W[0].val[None])
    with pytest.raises(ValueError):
        pkg.build_weights_backward([(OP_LAP, 0)], X, None, adjl, basis, W[0].row_ptr, W[0].val[None, :10])


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
@pytest.mark.parametrize("ops,q", [([(OP_LAP, 0)], 2), ([(OP_D1, 0), (OP_D1, 1), (OP_D1, 2)], 1)])
def test_invariances_full_size(pkg, ops, q, precision):
    """200k eval points in 3D, k = 30: the weights are unchanged by a translation of all
    points (sum of all gradients = 0) and scale as c^-q (sum_i x_i . g_i = -q L)."""
    g = torch.Generator(device="cuda").manual_seed(11)
    X = torch.rand((200_000, 3), generator=g, device="cuda", dtype=torch.float64)
    adjl = pkg.find_neighbors(X, 30)
    basis = pkg.PHS(3, poly_deg=2)
    W = pkg.build_weights(ops, X, None, adjl, basis)
    dW = torch.stack([torch.rand(w.val.shape, generator=g, device="cuda", dtype=torch.float64) - 0.5 for w in W])
    gd, ge = pkg.build_weights_backward(ops, X, None, adjl, basis, W[0].row_ptr, dW, precision=precision)
    G = gd + ge
    L = float(sum((dW[i] * W[i].val).sum() for i in range(len(W))))
    gscale = float((G.abs() * X.abs().max()).sum())
    assert float(G.sum(0).abs().max()) <= 1e-9 * float(G.abs().sum())
    assert abs(float((X * G).sum()) + q * L) <= 1e-9 * gscale
    if precision != "fp64":  # the refined adjoint against the FP64 one, point by point
        gd0, ge0 = pkg.build_weights_backward(ops, X, None, adjl, basis, W[0].row_ptr, dW, precision="fp64")
        assert float((G - (gd0 + ge0)).abs().max()) <= 1e-9 * float((gd0 + ge0).abs().max())


def test_apply_differentiable_field(pkg, orc):
    """d/dx <c, W x> = W^T c (one field and several), through the library's transposed apply."""
    rng = np.random.default_rng(13)
    data = rng.uniform(0, 1, (2000, 3))
    adjl = orc.knn(data, data, 20)
    X = torch.from_numpy(data).cuda()
    W = pkg.build_weights([(OP_LAP, 0)], X, None, adjl, pkg.PHS(3, poly_deg=1))[0]
    Ws = W.to_scipy()
    for shape in [(2000,), (2000, 3)]:
        x = torch.from_numpy(rng.standard_normal(shape)).cuda().requires_grad_(True)
        c = rng.standard_normal(shape)
        y = pkg.apply_differentiable(W, x)
        (y * torch.from_numpy(c).cuda()).sum().backward()
        want = Ws.T @ c
        assert np.abs(x.grad.cpu().numpy() - want).max() <= 1e-12 * np.abs(want).max()


def test_operator_application_differentiable_in_the_points(pkg, orc):
    """L(points) = sum((W(points) u)^2), u fixed: the autograd gradient through
    build_weights_differentiable and apply_differentiable against central differences of GPU
    builds (stencils fixed), as the reference's operator AD tests check against
    FiniteDifferences (test/extensions/mooncake_ext.jl:7-30)."""
    rng = np.random.default_rng(14)
    data = rng.uniform(0, 1, (300, 2))
    adjl = orc.knn(data, data, 15)
    basis = pkg.PHS(3, poly_deg=2)
    u = torch.from_numpy(np.sin(3 * data[:, 0]) * data[:, 1]).cuda()

    def loss(P, diff=False):
        if diff:
            rp, col, val = pkg.build_weights_differentiable([(OP_LAP, 0)], P, None, adjl, basis)
            Ws = pkg.WeightsCSR(rp, col, val[0].detach(), (300, 300), pkg.Context.default(0))
            y = pkg.apply_differentiable(Ws, u, val=val[0])
        else:
            y = pkg.build_weights([(OP_LAP, 0)], P, None, adjl, basis)[0].apply(u)
        return (y ** 2).sum()

    P = torch.from_numpy(data).cuda().requires_grad_(True)
    loss(P, True).backward()
    g = P.grad.cpu().numpy()
    h = 1e-6
    for idx in [(0, 0), (17, 1), (150, 0), (299, 1)]:
        Pp = torch.from_numpy(data).cuda()
        Pm = Pp.clone()
        Pp[idx] += h
        Pm[idx] -= h
        fd = (float(loss(Pp)) - float(loss(Pm))) / (2 * h)
        assert abs(g[idx] - fd) <= 1e-5 * np.abs(g).max(), (idx, g[idx], fd)
