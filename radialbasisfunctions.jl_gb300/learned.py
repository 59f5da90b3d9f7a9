"""Learned stencil surrogate: an MLP that predicts RBF-FD weights from a stencil's geometry.

Inputs: the k offsets of a stencil's points from its eval point, in stencil (distance) order,
divided by the power of two s >= the stencil radius (k*dim values).  Outputs: the k weights in
the same local units (w * s^q for an operator of order q).  Hidden layers use GELU; matrices
and activations are bf16 with FP32 accumulation on the tensor cores (`rbf_mlp_*` kernels of
librbffd_gb300.so).  The prediction seeds the FP32-factorised, FP64-refined build, which
accepts a stencil only once its FP64 residual says the weights are converged and otherwise
falls back to the plain FP64 solve, so the surrogate never decides the result.

Training data come from the plain FP64 solver on seeded clouds (the build with the
stencil-order / local-unit flags).  This module only orchestrates device buffers (torch) and
kernel launches; every arithmetic step is one of the library's kernels.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _native

RBF_FLAG_STENCIL_ORDER = 1
RBF_FLAG_LOCAL_UNITS = 2


def _torch():
    import torch
    return torch


def _pad(n, m=32):
    return (n + m - 1) // m * m


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class StencilMLP:
    """MLP k*dim -> hidden... -> k with GELU, trained and run on the library's kernels."""

    def __init__(self, k: int, dim: int, hidden=(256, 256, 256), ctx=None, seed: int = 0, out_scale: float = 1.0):
        torch = _torch()
        from . import Context
        self.ctx = ctx or Context.default(0)
        self.lib = self.ctx.lib
        self.dev = torch.device("cuda", self.ctx.device)
        self.k, self.dim = k, dim
        self.din, self.dout = k * dim, k
        self.dims = [_pad(self.din)] + list(hidden) + [_pad(self.dout)]
        self.out_scale = float(out_scale)
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.W, self.b, self.Wb = [], [], []
        for i in range(len(self.dims) - 1):
            fin, fout = self.dims[i], self.dims[i + 1]
            bound = math.sqrt(6.0 / fin) if i < len(self.dims) - 2 else math.sqrt(3.0 / fin)
            W = (torch.rand((fout, fin), generator=g, dtype=torch.float32) * 2 - 1) * bound
            if i == 0:
                W[:, self.din:] = 0.0
            self.W.append(W.to(self.dev).contiguous())
            self.b.append(torch.zeros(fout, dtype=torch.float32, device=self.dev))
            self.Wb.append(self.W[-1].to(torch.bfloat16).contiguous())
        self.m = [torch.zeros_like(t) for t in self.W + self.b]
        self.v = [torch.zeros_like(t) for t in self.W + self.b]
        self.t = 0

    # ------------------------------------------------------------------ kernels
    def _check(self, st):
        self.ctx.check(st)

    def _gemm(self, A, B, M, N, K, bias=None, epi=0, aux=None, Cf=None, Cb=None, Zf=None):
        lda = A.stride(0)
        ldb = B.stride(0)
        self._check(self.lib.rbf_mlp_gemm(self.ctx.h, M, N, K, _p(A), lda, _p(B), ldb, _p(bias), epi, _p(aux),
                                          aux.stride(0) if aux is not None else 0, _p(Cf),
                                          Cf.stride(0) if Cf is not None else 0, _p(Cb),
                                          Cb.stride(0) if Cb is not None else 0, _p(Zf),
                                          Zf.stride(0) if Zf is not None else 0))

    def _gemm_tc(self, A, B, M, N, K, bias=None, gelu=False, Cf=None, Cb=None):
        out = Cf if Cf is not None else Cb
        self._check(self.lib.rbf_mlp_gemm_tc(self.ctx.h, M, N, K, _p(A), A.stride(0), _p(B), B.stride(0), _p(bias),
                                             1 if gelu else 0, _p(Cf), _p(Cb), out.stride(0)))

    def tc_status(self):
        """Raise if a tensor-core GEMM gave up waiting on its pipeline (synchronises)."""
        f = ctypes.c_int32(0)
        self._check(self.lib.rbf_mlp_tc_status(self.ctx.h, ctypes.byref(f)))
        if f.value:
            raise RuntimeError("a tensor-core GEMM of the surrogate did not complete")

    def _transpose(self, X):
        torch = _torch()
        rows, cols = X.shape
        out = torch.empty((cols, rows), dtype=torch.bfloat16, device=self.dev)
        self._check(self.lib.rbf_mlp_transpose(self.ctx.h, rows, cols, _p(X), X.stride(0), _p(out), out.stride(0)))
        return out

    def features(self, data, eval_points, adjl):
        """bf16 network inputs (ne x pad(k*dim)) for stencils adjl over device points."""
        torch = _torch()
        ne = adjl.shape[0]
        out = torch.empty((ne, self.dims[0]), dtype=torch.bfloat16, device=self.dev)
        ev = data if eval_points is None else eval_points
        self._check(self.lib.rbf_mlp_features(self.ctx.h, _p(data), data.shape[0], _p(ev), self.dim, _p(adjl), ne, self.k,
                                              _p(out), out.stride(0)))
        return out

    # ------------------------------------------------------------------ forward / backward
    def forward(self, Xb, keep=False, tensor_cores=True):
        """Xb: bf16 inputs (B x pad(din)).  Returns FP32 outputs (B x pad(dout)) in network units;
        with keep=True also the pre-activations and activations needed by backward().  Without
        keep, the layers run on the tcgen05 GEMM (tensor_cores) or the mma.sync GEMM."""
        torch = _torch()
        B = Xb.shape[0]
        L = len(self.W)
        if not keep and tensor_cores:
            a = Xb
            for i in range(L):
                fout, fin = self.W[i].shape
                if i < L - 1:
                    h = torch.empty((B, fout), dtype=torch.bfloat16, device=self.dev)
                    self._gemm_tc(a, self.Wb[i], B, fout, fin, bias=self.b[i], gelu=True, Cb=h)
                    a = h
                else:
                    y = torch.empty((B, fout), dtype=torch.float32, device=self.dev)
                    self._gemm_tc(a, self.Wb[i], B, fout, fin, bias=self.b[i], gelu=False, Cf=y)
            return y
        acts, zs = [Xb], []
        a = Xb
        for i in range(L):
            fout, fin = self.W[i].shape
            if i < L - 1:
                z = torch.empty((B, fout), dtype=torch.float32, device=self.dev) if keep else None
                h = torch.empty((B, fout), dtype=torch.bfloat16, device=self.dev)
                self._gemm(a, self.Wb[i], B, fout, fin, bias=self.b[i], epi=1, Cb=h, Zf=z)
                zs.append(z)
                acts.append(h)
                a = h
            else:
                y = torch.empty((B, fout), dtype=torch.float32, device=self.dev)
                self._gemm(a, self.Wb[i], B, fout, fin, bias=self.b[i], epi=0, Cf=y)
        if keep:
            return y, zs, acts
        return y

    def gradients(self, Xb, T):
        """Loss and FP32 gradients (dW, db per layer) of the MSE between forward(Xb) and T
        (B x dout, network units)."""
        torch = _torch()
        B = Xb.shape[0]
        y, zs, acts = self.forward(Xb, keep=True)
        L = len(self.W)
        dz = torch.empty((B, self.dims[-1]), dtype=torch.bfloat16, device=self.dev)
        loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self._check(self.lib.rbf_mlp_mse(self.ctx.h, B, self.dout, _p(y), y.stride(0), _p(T), T.stride(0),
                                         _p(dz), dz.stride(0), self.dims[-1], _p(loss)))
        gW, gb = [None] * L, [None] * L
        for i in range(L - 1, -1, -1):
            fout, fin = self.W[i].shape
            dzT = self._transpose(dz)                # fout x B
            aT = self._transpose(acts[i])            # fin x B
            gW[i] = torch.empty((fout, fin), dtype=torch.float32, device=self.dev)
            self._gemm(dzT, aT, fout, fin, B, Cf=gW[i])
            gb[i] = torch.empty(fout, dtype=torch.float32, device=self.dev)
            self._check(self.lib.rbf_mlp_colsum(self.ctx.h, B, fout, _p(dz), dz.stride(0), _p(gb[i])))
            if i > 0:
                WT = self._transpose(self.Wb[i])     # fin x fout
                dprev = torch.empty((B, fin), dtype=torch.bfloat16, device=self.dev)
                self._gemm(dz, WT, B, fin, fout, epi=2, aux=zs[i - 1], Cb=dprev)
                dz = dprev
        return loss, gW, gb

    def train_step(self, Xb, T, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        loss, gW, gb = self.gradients(Xb, T)
        self.t += 1
        for j, (p, g) in enumerate(zip(self.W + self.b, gW + gb)):
            pb = self.Wb[j] if j < len(self.W) else None
            self._check(self.lib.rbf_mlp_adam(self.ctx.h, p.numel(), _p(p), _p(g), _p(self.m[j]), _p(self.v[j]),
                                              lr, b1, b2, eps, self.t, _p(pb)))
        return loss

    def predict(self, Xb, batch=1 << 20, tensor_cores=True):
        """Predicted weights (B x k, FP32, local units) for bf16 inputs, in chunks (tcgen05
        GEMMs by default; the call checks that they completed)."""
        torch = _torch()
        out = torch.empty((Xb.shape[0], self.dout), dtype=torch.float32, device=self.dev)
        for s in range(0, Xb.shape[0], batch):
            y = self.forward(Xb[s:s + batch], tensor_cores=tensor_cores)
            out[s:s + batch] = y[:, :self.dout] * self.out_scale
        if tensor_cores:
            self.tc_status()
        return out

    # ------------------------------------------------------------------ checkpoint
    def state_dict(self):
        """Everything training resumes from: the FP32 master weights and biases, their bf16
        copies, the Adam moments and step count (host tensors)."""
        return {"dims": list(self.dims), "k": self.k, "dim": self.dim, "out_scale": self.out_scale, "t": self.t,
                "W": [w.cpu() for w in self.W], "b": [b.cpu() for b in self.b], "Wb": [w.cpu() for w in self.Wb],
                "m": [t.cpu() for t in self.m], "v": [t.cpu() for t in self.v]}

    def load_state_dict(self, sd):
        torch = _torch()
        if list(sd["dims"]) != list(self.dims) or sd["k"] != self.k or sd["dim"] != self.dim:
            raise ValueError(f"state of a network with layers {sd['dims']} (k = {sd['k']}, dim = {sd['dim']}) "
                             f"does not fit this one ({self.dims}, k = {self.k}, dim = {self.dim})")
        self.out_scale = sd["out_scale"]
        self.t = sd["t"]
        self.W = [w.to(self.dev).contiguous() for w in sd["W"]]
        self.b = [b.to(self.dev).contiguous() for b in sd["b"]]
        self.Wb = ([w.to(self.dev).contiguous() for w in sd["Wb"]] if "Wb" in sd else
                   [w.to(torch.bfloat16).contiguous() for w in self.W])
        if "m" in sd:
            self.m = [t.to(self.dev).contiguous() for t in sd["m"]]
            self.v = [t.to(self.dev).contiguous() for t in sd["v"]]


SURROGATE_FORMAT = "rbffd-gb300-surrogate-1"


def save_surrogate(path, model, progress=None):
    """A StencilMLP (weights, Adam state) and optionally the training progress to one .npz:
    progress = {"epoch": epochs done, "hist": losses, "rng": generator state (uint8 tensor)}."""
    import json

    import numpy as np
    sd = model.state_dict()
    arrays = {"format": SURROGATE_FORMAT}
    nl = len(sd["W"])
    for name in ("W", "b", "m", "v"):
        for i, t in enumerate(sd[name]):
            arrays[f"{name}{i}"] = t.numpy()
    for i, t in enumerate(sd["Wb"]):  # bf16 bits
        arrays[f"Wb{i}"] = t.view(_torch().int16).numpy()
    meta = {"dims": sd["dims"], "k": sd["k"], "dim": sd["dim"], "out_scale": sd["out_scale"], "t": sd["t"],
            "layers": nl, "nmoments": len(sd["m"])}
    if progress is not None:
        meta["epoch"] = int(progress["epoch"])
        meta["hist"] = [float(h) for h in progress.get("hist", [])]
        if progress.get("rng") is not None:
            arrays["rng"] = progress["rng"].cpu().numpy()
    arrays["meta"] = json.dumps(meta)
    np.savez(path if str(path).endswith(".npz") else str(path) + ".npz", **arrays)


def load_surrogate(path, ctx=None, return_progress=False):
    """The StencilMLP of save_surrogate (and, with return_progress, its training progress)."""
    import json

    import numpy as np
    torch = _torch()
    z = np.load(path if str(path).endswith(".npz") else str(path) + ".npz", allow_pickle=False)
    if "format" not in z.files or str(z["format"]) != SURROGATE_FORMAT:
        raise ValueError(f"{path}: not a surrogate checkpoint of this library")
    meta = json.loads(str(z["meta"]))
    dims = meta["dims"]
    model = StencilMLP(meta["k"], meta["dim"], hidden=tuple(dims[1:-1]), ctx=ctx, out_scale=meta["out_scale"])
    nl, nm = meta["layers"], meta["nmoments"]
    sd = {"dims": dims, "k": meta["k"], "dim": meta["dim"], "out_scale": meta["out_scale"], "t": meta["t"],
          "W": [torch.from_numpy(z[f"W{i}"]) for i in range(nl)], "b": [torch.from_numpy(z[f"b{i}"]) for i in range(nl)],
          "Wb": [torch.from_numpy(z[f"Wb{i}"]).view(torch.bfloat16) for i in range(nl)],
          "m": [torch.from_numpy(z[f"m{i}"]) for i in range(nm)], "v": [torch.from_numpy(z[f"v{i}"]) for i in range(nm)]}
    model.load_state_dict(sd)
    if not return_progress:
        return model
    prog = None
    if "epoch" in meta:
        prog = {"epoch": meta["epoch"], "hist": meta["hist"],
                "rng": torch.from_numpy(z["rng"]) if "rng" in z.files else None}
    return model, prog


# ---------------------------------------------------------------------------- data
def sample_cloud(n, dim, seed, gradient=0.0, device=None):
    """n points in [0,1]^dim: uniform, or with density 1 + gradient*(2x_1 - 1) (a linear
    gradient of +/- gradient along the first axis), seeded."""
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(seed)
    if gradient == 0.0:
        X = torch.rand((n, dim), generator=g, dtype=torch.float64)
    else:
        parts, have = [], 0
        while have < n:
            Y = torch.rand((2 * n, dim), generator=g, dtype=torch.float64)
            acc = torch.rand(2 * n, generator=g, dtype=torch.float64) * (1 + gradient) < 1 + gradient * (2 * Y[:, 0] - 1)
            parts.append(Y[acc])
            have += int(acc.sum())
        X = torch.cat(parts)[:n]
    return X.to(device) if device is not None else X


def training_set(n_uniform, n_gradient, k, dim, basis, ops, seed=0, ctx=None, gradient=0.2, separate_eval=False):
    """Features and local-unit target weights of the plain FP64 solve on seeded clouds:
    n_uniform stencils of a uniform cloud and n_gradient of a cloud with a linear density
    gradient.  Every point of each cloud is an eval point, or, with separate_eval (regrid
    stencils, whose weights are trivial at the data points), an independent cloud of the same
    distribution and size holds the eval points."""
    torch = _torch()
    from . import Context, build_weights, find_neighbors
    ctx = ctx or Context.default(0)
    dev = torch.device("cuda", ctx.device)
    feats, targs = [], []
    mlp = StencilMLP(k, dim, hidden=(32,), ctx=ctx)  # only for its feature kernel
    for n, gr, sd in ((n_uniform, 0.0, seed), (n_gradient, gradient, seed + 1)):
        if n <= 0:
            continue
        X = sample_cloud(n, dim, sd, gr, dev)
        E = sample_cloud(n, dim, sd + 7919, gr, dev) if separate_eval else None
        adjl = find_neighbors(X, E, k=k, ctx=ctx)
        W = build_weights(ops, X, E, adjl, basis, precision="fp64", ctx=ctx,
                          flags=RBF_FLAG_STENCIL_ORDER | RBF_FLAG_LOCAL_UNITS)[0]
        feats.append(mlp.features(X, E, adjl))
        targs.append(W.val.reshape(n, k).to(torch.float32))
    return torch.cat(feats), torch.cat(targs)


def train_surrogate(Xb, T, k, dim, hidden=(256, 256, 256), epochs=20, batch=4096, lr=2e-3, ctx=None, seed=0,
                    log=None, checkpoint=None, resume=None):
    """Train a StencilMLP on bf16 features Xb and local-unit weights T (Adam, cosine decay).

    checkpoint: a path written at the end of every epoch (network, Adam state, epochs done,
    the shuffling generator's state); resume: such a path, from which training continues at the
    next epoch on the same Xb, T and arguments, reaching the weights an uninterrupted run gives."""
    torch = _torch()
    n = Xb.shape[0]
    g = None
    hist = []
    start = 0
    if resume is not None:
        model, prog = load_surrogate(resume, ctx=ctx, return_progress=True)
        if prog is None or list(model.dims[1:-1]) != list(hidden) or model.k != k or model.dim != dim:
            raise ValueError(f"{resume}: not a training checkpoint of this network")
        start, hist = prog["epoch"], list(prog["hist"])
        g = torch.Generator(device=model.dev)
        g.set_state(prog["rng"])
        scale = model.out_scale
    else:
        scale = float(T.std())
        model = StencilMLP(k, dim, hidden=hidden, ctx=ctx, seed=seed, out_scale=scale)
        g = torch.Generator(device=model.dev).manual_seed(seed)
    Tn = torch.zeros((n, model.dims[-1]), dtype=torch.float32, device=model.dev)
    Tn[:, :k] = T / scale
    steps = max(1, n // batch)
    total = epochs * steps
    it = start * steps
    for ep in range(start, epochs):
        perm = torch.randperm(n, device=model.dev, generator=g)
        acc = 0.0
        for s in range(steps):
            idx = perm[s * batch:(s + 1) * batch]
            cur = lr * 0.5 * (1 + math.cos(math.pi * it / total))
            loss = model.train_step(Xb[idx].contiguous(), Tn[idx].contiguous(), lr=cur)
            it += 1
            if s % 50 == 0:
                acc = float(loss)
        hist.append(acc)
        if checkpoint is not None:
            save_surrogate(checkpoint, model, {"epoch": ep + 1, "hist": hist, "rng": g.get_state()})
        if log:
            log(f"epoch {ep}: loss {acc:.4e}")
    return model, hist


def surrogate_error(model, Xb, T):
    """Max and median row-relative error of the predicted weights (local units)."""
    P = model.predict(Xb)
    err = (P - T).abs().amax(1) / T.abs().amax(1).clamp_min(1e-30)
    return float(err.max()), float(err.median())


def build_learned(model, ops, data, adjl, basis, ctx=None, stats=None, return_status=False, sell=False,
                  eval_points=None):
    """Learned + FP32-refined build: the surrogate's prediction seeds the refinement."""
    from . import build_weights
    feats = model.features(data, eval_points, adjl)
    seed = model.predict(feats)
    return build_weights(ops, data, eval_points, adjl, basis, precision="learned", ctx=ctx or model.ctx, stats=stats,
                         seed=seed, return_status=return_status, sell=sell)
