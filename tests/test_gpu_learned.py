"""The learned surrogate: its hand-written training kernels against the CPU oracle, and the
learned + FP32-refined build against the plain FP64 build."""
import os

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
    p = g.load_package()
    from importlib import import_module
    p.learned = import_module(p.__name__ + ".learned")
    return p


def test_gradients_match_oracle(pkg):
    """Loss and every parameter gradient of one step (bf16 storage, FP32 accumulation) agree
    with the float64 restatement to 1e-2 relative (Frobenius) per tensor."""
    from oracle import mlp_oracle as MO
    L = pkg.learned
    model = L.StencilMLP(k=30, dim=3, hidden=(64, 64), seed=3)
    B = 256
    rng = np.random.default_rng(0)
    X = np.zeros((B, model.dims[0]), dtype=np.float32)
    X[:, :90] = rng.uniform(-1, 1, (B, 90))
    T = np.zeros((B, model.dims[-1]), dtype=np.float32)
    T[:, :30] = rng.standard_normal((B, 30))
    Xb = torch.from_numpy(X).cuda().to(torch.bfloat16)
    loss, gW, gb = model.gradients(Xb, torch.from_numpy(T).cuda())
    W = [w.cpu().numpy() for w in model.W]
    b = [v.cpu().numpy().astype(np.float64) for v in model.b]
    l_ref, y_ref, dW_ref, db_ref = MO.forward_backward(MO.bf16(X), W, b, T.astype(np.float64), 30)
    assert abs(float(loss) - l_ref) <= 2e-3 * l_ref
    y = model.forward(Xb).cpu().numpy()
    assert np.abs(y - y_ref).max() <= 2e-2 * np.abs(y_ref).max()
    for i in range(len(W)):
        g = gW[i].cpu().numpy()
        e = np.linalg.norm(g - dW_ref[i]) / np.linalg.norm(dW_ref[i])
        assert e < 1e-2, (i, e)
        gbv = gb[i].cpu().numpy()
        e = np.linalg.norm(gbv - db_ref[i]) / np.linalg.norm(db_ref[i])
        assert e < 1e-2, (i, e)


def test_gemm_exact_on_bf16_integers(pkg):
    """The tensor-core GEMM with small-integer operands (exact in bf16 and FP32) is exact."""
    L = pkg.learned
    model = L.StencilMLP(k=30, dim=3, hidden=(64,), seed=0)
    rng = np.random.default_rng(1)
    M, N, K = 200, 96, 160
    A = rng.integers(-4, 5, (M, K)).astype(np.float32)
    Bm = rng.integers(-4, 5, (N, K)).astype(np.float32)
    At = torch.from_numpy(A).cuda().to(torch.bfloat16)
    Bt = torch.from_numpy(Bm).cuda().to(torch.bfloat16)
    C = torch.empty((M, N), dtype=torch.float32, device="cuda")
    model._gemm(At, Bt, M, N, K, Cf=C)
    assert np.array_equal(C.cpu().numpy(), A @ Bm.T)


def test_features_check_indices(pkg):
    """Network inputs are the stencil offsets in local units; a neighbour index outside the
    data set is an argument error, not a device access."""
    L = pkg.learned
    X = L.sample_cloud(5000, 3, 2, device=torch.device("cuda"))
    adjl = pkg.find_neighbors(X, k=30)
    model = L.StencilMLP(30, 3, hidden=(32,), seed=0)
    F = model.features(X, None, adjl).float().cpu().numpy()
    Xh, a = X.cpu().numpy(), adjl.cpu().numpy()
    for e in (0, 17, 4999):
        off = Xh[a[e]] - Xh[e]
        s = 2.0 ** np.frexp(np.sqrt((off ** 2).sum(1).max()))[1]
        ref = (off / s).reshape(-1)
        assert np.allclose(F[e, :90], ref, rtol=2 ** -8, atol=0)
        assert not F[e, 90:].any()
    bad = adjl.clone()
    bad[7, 5] = 5000
    with pytest.raises(ValueError):
        model.features(X, None, bad)


def test_training_reduces_error(pkg):
    """Training on solver-generated stencils lowers the surrogate's weight error well below
    that of the untrained network (the gain of training)."""
    L = pkg.learned
    basis = pkg.PHS(3, poly_deg=2)
    Xb, T = L.training_set(40000, 20000, 30, 3, basis, [(3, 0)], seed=11)
    Xv, Tv = L.training_set(4000, 0, 30, 3, basis, [(3, 0)], seed=99)
    untrained = L.StencilMLP(30, 3, hidden=(256, 256, 256), seed=0, out_scale=float(T.std()))
    e0_max, e0_med = L.surrogate_error(untrained, Xv, Tv)
    model, hist = L.train_surrogate(Xb, T, 30, 3, epochs=8, batch=2048, lr=2e-3)
    e_max, e_med = L.surrogate_error(model, Xv, Tv)
    print(f"surrogate median row error: untrained {e0_med:.3e}, trained {e_med:.3e}; loss {hist[0]:.3e} -> {hist[-1]:.3e}")
    assert hist[-1] < 0.5 * hist[0]
    assert e_med < 0.5 * e0_med


def test_learned_build_equals_fp64(pkg):
    """Seeded by an (even untrained) surrogate, the refined build still meets the FP64 bar:
    the refinement, not the network, decides the weights."""
    L = pkg.learned
    basis = pkg.PHS(3, poly_deg=2)
    X = L.sample_cloud(60000, 3, 5, device=torch.device("cuda"))
    adjl = pkg.find_neighbors(X, k=30)
    W64 = pkg.build_weights([(3, 0)], X, None, adjl, basis, precision="fp64")[0]
    for trained in (False, True):
        if trained:
            Xb, T = L.training_set(30000, 10000, 30, 3, basis, [(3, 0)], seed=21)
            model, _ = L.train_surrogate(Xb, T, 30, 3, epochs=4, batch=2048)
        else:
            model = L.StencilMLP(30, 3, seed=1, out_scale=10.0)
        st = pkg._native.BuildStats()
        W, status = L.build_learned(model, [(3, 0)], X, adjl, basis, stats=st, return_status=True)
        W = W[0]
        assert torch.equal(W.col, W64.col)
        d = (W.val - W64.val).abs().reshape(-1, 30).amax(1) / W64.val.abs().reshape(-1, 30).amax(1)
        assert float(d.max()) <= 1e-8, (trained, float(d.max()))
        assert set(np.unique(status.cpu().numpy())) <= {0, 3}


@pytest.mark.parametrize("M,N,K", [(300, 256, 96), (128, 32, 256), (1000, 96, 32), (257, 64, 64), (100003, 256, 256)])
@pytest.mark.parametrize("gelu,bf16_out", [(False, False), (True, True)])
def test_tc_gemm_equals_mma_sync(pkg, M, N, K, gelu, bf16_out):
    """The tcgen05 GEMM (TMEM accumulators) equals the mma.sync GEMM bit for bit on operands
    whose products and sums are exact (small integers), incl. row/column tails, the bias and
    the GELU epilogue, several tiles per CTA (the persistent kernel's alternating
    accumulators and ring wrap-around), and it reports no pipeline timeout."""
    L = pkg.learned
    model = L.StencilMLP(k=30, dim=3, hidden=(64,), seed=0)
    rng = np.random.default_rng(M + N + K)
    A = torch.from_numpy(rng.integers(-4, 5, (M, K)).astype(np.float32)).cuda().to(torch.bfloat16)
    B = torch.from_numpy(rng.integers(-4, 5, (N, K)).astype(np.float32)).cuda().to(torch.bfloat16)
    bias = torch.from_numpy(rng.integers(-8, 9, N).astype(np.float32)).cuda()
    if bf16_out:
        C0 = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
        C1 = torch.empty_like(C0)
        model._gemm(A, B, M, N, K, bias=bias, epi=1 if gelu else 0, Cb=C0)
        model._gemm_tc(A, B, M, N, K, bias=bias, gelu=gelu, Cb=C1)
    else:
        C0 = torch.empty((M, N), dtype=torch.float32, device="cuda")
        C1 = torch.empty_like(C0)
        model._gemm(A, B, M, N, K, bias=bias, epi=1 if gelu else 0, Cf=C0)
        model._gemm_tc(A, B, M, N, K, bias=bias, gelu=gelu, Cf=C1)
    model.tc_status()
    assert torch.equal(C0, C1)


def test_predict_tensor_cores(pkg):
    """Inference on the tensor cores agrees with the mma.sync forward (bf16 activations)."""
    L = pkg.learned
    model = L.StencilMLP(k=30, dim=3, seed=4, out_scale=3.0)
    rng = np.random.default_rng(8)
    X = np.zeros((5000, model.dims[0]), dtype=np.float32)
    X[:, :90] = rng.uniform(-1, 1, (5000, 90))
    Xb = torch.from_numpy(X).cuda().to(torch.bfloat16)
    p_tc = model.predict(Xb)
    p_ms = model.predict(Xb, tensor_cores=False)
    assert float((p_tc - p_ms).abs().max() / p_ms.abs().max()) < 2e-2


def test_tc_gemm_wait_timeout_is_reported(pkg):
    """The tensor-core GEMM's waits are bounded: a launch whose producer issues no copy (the
    library's self-test, nothing in flight) gives up after a short wait limit, returns, and
    leaves the error flag that rbf_mlp_tc_status reports; the next GEMM on the same context
    runs normally and reports no failure."""
    import ctypes
    ctx = pkg.Context.default(0)
    failed = ctypes.c_int32(-1)
    assert ctx.lib.rbf_mlp_tc_selftest_timeout(ctx.h, ctypes.byref(failed)) == 0, ctx.lib.rbf_last_error(ctx.handle)
    assert failed.value == 1
    ok = ctypes.c_int32(-1)
    assert ctx.lib.rbf_mlp_tc_status(ctx.h, ctypes.byref(ok)) == 0
    assert ok.value == 0  # the self-test cleared what it set
    L = pkg.learned
    model = L.StencilMLP(k=30, dim=3, hidden=(64,), seed=0)
    rng = np.random.default_rng(2)
    M, N, K = 640, 64, 64
    A = torch.from_numpy(rng.integers(-4, 5, (M, K)).astype(np.float32)).cuda().to(torch.bfloat16)
    B = torch.from_numpy(rng.integers(-4, 5, (N, K)).astype(np.float32)).cuda().to(torch.bfloat16)
    C0 = torch.empty((M, N), dtype=torch.float32, device="cuda")
    C1 = torch.empty_like(C0)
    model._gemm(A, B, M, N, K, Cf=C0)
    model._gemm_tc(A, B, M, N, K, Cf=C1)
    assert ctx.lib.rbf_mlp_tc_status(ctx.h, ctypes.byref(ok)) == 0
    assert ok.value == 0
    assert torch.equal(C0, C1)
