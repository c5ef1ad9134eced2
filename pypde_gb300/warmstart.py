"""Learned warm start of the stiff (Newton) space-time predictor.

Not in the reference: its predictor always starts from the plain guess
q = w (pypde solvers/dg/dg.cpp:187-199).  Here a per-cell MLP maps the WENO
coefficients of a cell and log10(dt/tau) to the correction qh - w of the
converged predictor; the solver's Newton iteration starts from w + that
correction, iterates to the same residual tolerance, and falls back to the
plain guess at the first iteration whose residual does not fall
(pypde_stats.pred_fallbacks).

Pieces:
  harvest()            (w, converged qh, dt) pairs sampled from plain runs,
                       by the library (pypde_harvest)
  features()/targets() the network's inputs and outputs, the recipe the
                       device kernel k_mlp_guess uses
  MLPFunction          a torch.autograd.Function whose forward and backward
                       passes are the library's BF16 tensor-core kernels
                       (pypde_mlp_gemm, pypde_mlp_silu_grad, pypde_mlp_colsum)
  WarmStartNet         the network, its normalisation and its training loop
  WarmStart            a trained network resident on the GPU, passed to
                       pde_solver(..., warm_start=...)
  train_warm_start()   harvest + train + upload in one call

torch is plumbing here (device memory, streams, the optimiser); every
forward and backward FLOP of the network runs in the library's kernels.
"""
import ctypes

import numpy as np

from . import _lib
from .callbacks import resolve_system
from .utils import nargs, parse_boundary_types

HIDDEN = 128


def shape(system, N):
    """(feat, k1, no) of the warm-start network for a system and order."""
    f, k, o = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _lib.check(_lib.lib().pypde_warm_start_shape(system.handle, N, f, k, o))
    return f.value, k.value, o.value


def features(w, dt, N, ndim, V, tau_var=-1):
    """Raw inputs of each cell, float32 (cells, V + N^ndim V + 1): the
    means of the V variables over the cell's N^ndim nodes, the deviations
    from them, and log10(dt) - mean[tau_var] (log10(dt) when tau_var < 0).
    WarmStartNet.inputs() normalises them and appends log10(r).
    w: (cells, N^ndim, V) or (cells N^ndim, V); dt a scalar or one value
    per cell.  Same operation order as k_mlp_guess."""
    Nd = N ** ndim
    w = np.asarray(w, dtype=np.float64).reshape(-1, Nd, V)
    s = w[:, 0, :].copy()
    for idx in range(1, Nd):
        s = s + w[:, idx, :]
    mean = s * (1.0 / Nd)
    dev = w - mean[:, None, :]
    lg = np.log10(np.broadcast_to(np.asarray(dt, dtype=np.float64), (w.shape[0],)))
    if tau_var >= 0:
        lg = lg - mean[:, tau_var]
    f = np.concatenate([mean, dev.reshape(w.shape[0], Nd * V), lg[:, None]], axis=1)
    return f.astype(np.float32)


def targets(w, qh, N, ndim, V):
    """Corrections qh - w at every space-time value, (cells, N^(ndim+1) V),
    output o = (t N^ndim + idx) V + v."""
    Nd = N ** ndim
    w = np.asarray(w, dtype=np.float64).reshape(-1, 1, Nd, V)
    qh = np.asarray(qh, dtype=np.float64).reshape(-1, N, Nd, V)
    return (qh - w).reshape(qh.shape[0], N * Nd * V)


def harvest(Q0, tf, L, F=None, B=None, S=None, boundaryTypes="periodic", cfl=0.9, order=2,
            steps=20, per_step=8192, device=0, newton_tol=None):
    """Run `steps` plain stiff steps from Q0 (not modified) and sample
    per_step reconstruction cells after every predictor.  Returns
    (w (n, N^ndim, V), qh (n, N^(ndim+1), V), dt (n,)) over the steps that
    ran."""
    nX = np.array(Q0.shape[:-1], dtype=np.int32)
    ndim, V, N = len(nX), Q0.shape[-1], order
    dX = np.array([L[i] / nX[i] for i in range(ndim)], dtype=np.float64)
    bt = parse_boundary_types(boundaryTypes, ndim)
    secondOrder = F is not None and nargs(F) == 3
    system = resolve_system(F, B, S, ndim, V, secondOrder)
    Cw = int(np.prod(nX + 2))
    per_step = min(per_step, Cw)
    stride = max(1, Cw // per_step)
    Nd = N ** ndim
    hw = np.zeros((steps * per_step, Nd, V))
    hq = np.zeros((steps * per_step, N * Nd, V))
    hdt = np.zeros(steps)
    u = np.ascontiguousarray(Q0, dtype=np.float64).copy()
    opt = _lib.Options()
    opt.device = device
    opt.newton_tol = float(newton_tol) if newton_tol else 0.0
    st = _lib.Stats()
    _lib.check(_lib.lib().pypde_harvest(
        system.handle, _lib.c_ptr(u), float(tf), _lib.c_ptr(nX), ndim, _lib.c_ptr(dX),
        float(cfl), _lib.c_ptr(bt), True, N, steps, per_step, stride, _lib.c_ptr(hw),
        _lib.c_ptr(hq), _lib.c_ptr(hdt), opt, st))
    ran = int(st.steps)
    n = ran * per_step
    return hw[:n], hq[:n], np.repeat(hdt[:ran], per_step)


# ---------------------------------------------------------------- kernels

def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def gemm(A, B, M, N, K, sam, sak, sbk, sbn, bias=None, act=False, splits=1, pre=True):
    """C = A B (BF16 operands, FP32 accumulation) through pypde_mlp_gemm;
    returns (C + bias, SiLU(C + bias) or None)."""
    import torch
    dev = A.device
    C = torch.empty((M, N), dtype=torch.float32, device=dev) if pre else None
    Aout = torch.empty((M, N), dtype=torch.float32, device=dev) if act else None
    work = torch.empty(splits * M * N, dtype=torch.float32, device=dev) if splits > 1 else None
    _lib.check(_lib.lib().pypde_mlp_gemm(
        _ptr(A), sam, sak, _ptr(B), sbk, sbn, _ptr(C) if C is not None else None, M, N, K,
        splits, _ptr(work) if work is not None else None,
        _ptr(bias) if bias is not None else None, _ptr(Aout) if Aout is not None else None,
        _stream()))
    return C, Aout


def _splits(K):
    return max(1, min(128, K // 512))


def _silu_grad(dA, Z):
    import torch
    dZ = torch.empty_like(Z)
    _lib.check(_lib.lib().pypde_mlp_silu_grad(_ptr(dA), _ptr(Z), _ptr(dZ), Z.numel(),
                                              _stream()))
    return dZ


def _colsum(X):
    import torch
    out = torch.empty(X.shape[1], dtype=torch.float32, device=X.device)
    _lib.check(_lib.lib().pypde_mlp_colsum(_ptr(X), X.shape[0], X.shape[1], _ptr(out),
                                           _stream()))
    return out


def _linear_grads(dZ, Xin, W, need_dx):
    """dW = dZ^T Xin, db = colsum(dZ), dX = dZ W (BF16 operands)."""
    M, n_out = dZ.shape
    n_in = Xin.shape[1]
    dW, _ = gemm(dZ, Xin, n_out, n_in, M, 1, n_out, n_in, 1, splits=_splits(M))
    db = _colsum(dZ)
    dX = None
    if need_dx:
        dX, _ = gemm(dZ, W, M, n_in, n_out, n_out, 1, n_in, 1)
    return dW, db, dX


def _make_function():
    import torch

    class MLPFunction(torch.autograd.Function):
        """y = W3 SiLU(W2 SiLU(W1 x + b1) + b2) + b3 on the library's
        kernels; x (M, k1) float32 on the GPU, weights row-major
        [out][in]."""

        @staticmethod
        def forward(ctx, x, W1, b1, W2, b2, W3, b3):
            x = x.contiguous()
            M, k1 = x.shape
            H, no = W1.shape[0], W3.shape[0]
            z1, a1 = gemm(x, W1, M, H, k1, k1, 1, 1, k1, bias=b1, act=True)
            z2, a2 = gemm(a1, W2, M, H, H, H, 1, 1, H, bias=b2, act=True)
            y, _ = gemm(a2, W3, M, no, H, H, 1, 1, H, bias=b3)
            ctx.save_for_backward(x, W1, W2, W3, z1, a1, z2, a2)
            return y

        @staticmethod
        def backward(ctx, dy):
            x, W1, W2, W3, z1, a1, z2, a2 = ctx.saved_tensors
            dy = dy.contiguous()
            dW3, db3, da2 = _linear_grads(dy, a2, W3, True)
            dz2 = _silu_grad(da2, z2)
            dW2, db2, da1 = _linear_grads(dz2, a1, W2, True)
            dz1 = _silu_grad(da1, z1)
            dW1, db1, dx = _linear_grads(dz1, x, W1, ctx.needs_input_grad[0])
            return dx, dW1, db1, dW2, db2, dW3, db3

    return MLPFunction


_MLP = None


def mlp(x, W1, b1, W2, b2, W3, b3):
    """The network on the library's kernels (differentiable)."""
    global _MLP
    if _MLP is None:
        _MLP = _make_function()
    return _MLP.apply(x, W1, b1, W2, b2, W3, b3)


# ---------------------------------------------------------------- network

class WarmStartNet:
    """The network with its input and output normalisation.  Parameters are
    FP32 master copies (torch tensors on the GPU); the kernels round them to
    BF16 in every GEMM."""

    def __init__(self, feat, k1, no, nout, V, seed=0, device="cuda"):
        import torch
        self.feat, self.k1, self.no, self.nout, self.V = feat, k1, no, nout, V
        g = torch.Generator(device="cpu").manual_seed(seed)

        def U(shape, fan_in):
            b = 1.0 / np.sqrt(fan_in)
            return ((torch.rand(shape, generator=g) * 2 - 1) * b).to(device).requires_grad_()

        self.params = [U((HIDDEN, k1), feat), U((HIDDEN,), feat), U((HIDDEN, HIDDEN), HIDDEN),
                       U((HIDDEN,), HIDDEN), U((no, HIDDEN), HIDDEN), U((no,), HIDDEN)]
        self.x_mean = np.zeros(k1, np.float32)
        self.x_scale = np.zeros(k1, np.float32)
        self.y_mean = np.zeros(no, np.float32)
        self.y_scale = np.zeros(no, np.float32)
        self.device = device
        self.history = []

    # raw feature layout: [means (V) | deviations (Nd V) | lg], then lr
    def _layout(self):
        nd_v = self.feat - 2 - self.V
        return self.V, self.V + nd_v            # deviations are [V, V + Nd V)

    def fit_normalisation(self, f, d):
        """Scales from training data.  Means and lg: centred and scaled by
        their standard deviation; deviations: scaled by their RMS (not
        centred, so that they stay homogeneous); lr: centred and scaled;
        outputs (correction / r): scaled by their RMS.  Constant columns
        get scale 0."""
        f = np.asarray(f, np.float32)
        d = np.asarray(d, np.float64)
        a, b = self._layout()
        f64 = f.astype(np.float64)
        xm = f64.mean(0)
        xs = f64.std(0)
        rms = np.sqrt((f64 ** 2).mean(0))
        self.x_mean[:] = 0
        self.x_scale[:] = 0
        for k in range(self.feat - 1):
            if a <= k < b:
                self.x_scale[k] = 1.0 / rms[k] if rms[k] > 1e-30 else 0.0
            else:
                self.x_mean[k] = xm[k]
                self.x_scale[k] = 1.0 / xs[k] if xs[k] > 1e-30 else 0.0
        _, r = self._normalise(f)
        lr = np.log10(r).astype(np.float64)
        k = self.feat - 1
        self.x_mean[k] = lr.mean()
        self.x_scale[k] = 1.0 / lr.std() if lr.std() > 1e-30 else 0.0
        yr = d / r.astype(np.float64)[:, None]
        ys = np.sqrt((yr ** 2).mean(0))
        self.y_mean[:] = 0
        self.y_scale[:] = 0
        self.y_scale[:self.nout] = np.where(ys > 1e-300, ys, 0.0)

    def _normalise(self, f):
        """The kernel's recipe in float32: x = (f - x_mean) x_scale over the
        raw features, r = RMS of the normalised deviations (>= 1e-30),
        deviations times 1/r.  Returns (x without lr, r)."""
        f = np.asarray(f, np.float32)
        a, b = self._layout()
        n = self.feat - 1
        x = (f[:, :n] - self.x_mean[:n]) * self.x_scale[:n]
        ss = np.zeros(f.shape[0], np.float32)
        for k in range(a, b):
            ss = ss + x[:, k] * x[:, k]
        r = np.maximum(np.sqrt(ss * (np.float32(1.0) / np.float32(b - a))), np.float32(1e-30))
        rr = np.float32(1.0) / r
        x[:, a:b] = x[:, a:b] * rr[:, None]
        return x, r

    def inputs(self, f):
        """Normalised, padded inputs (float32, (cells, k1)) and r, as the
        kernel forms them."""
        x0, r = self._normalise(f)
        x = np.zeros((x0.shape[0], self.k1), np.float32)
        n = self.feat - 1
        x[:, :n] = x0
        x[:, n] = (np.log10(r) - self.x_mean[n]) * self.x_scale[n]
        return x, r

    def outputs_normalised(self, d, r):
        y = np.zeros((d.shape[0], self.no), np.float32)
        s = self.y_scale[:self.nout].astype(np.float64)
        q = np.asarray(d, np.float64) / r.astype(np.float64)[:, None]
        y[:, :self.nout] = np.where(s > 0, q / np.where(s > 0, s, 1), 0.0)
        return y

    def correction(self, y, r):
        """De-normalised network output, as the kernel forms it (float32)."""
        n = self.nout
        return ((y[:, :n] * self.y_scale[:n] + self.y_mean[:n]) * r[:, None]).astype(np.float32)

    def forward(self, x):
        return mlp(x, *self.params)

    def train(self, f, d, iters=3000, batch=4096, lr=2e-3, seed=0, log_every=0):
        """Adam on the mean squared error of the normalised corrections."""
        import torch
        self.fit_normalisation(f, d)
        x, r = self.inputs(f)
        X = torch.from_numpy(x).to(self.device)
        Y = torch.from_numpy(self.outputs_normalised(d, r)).to(self.device)
        n = X.shape[0]
        opt = torch.optim.Adam(self.params, lr=lr)
        sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, iters, eta_min=lr * 0.02)
        gen = torch.Generator(device=self.device).manual_seed(seed)
        for it in range(iters):
            idx = torch.randint(0, n, (min(batch, n),), device=self.device, generator=gen)
            y = self.forward(X[idx])
            loss = ((y[:, :self.nout] - Y[idx, :self.nout]) ** 2).mean()
            opt.zero_grad()
            loss.backward()
            opt.step()
            sched.step()
            if log_every and (it % log_every == 0 or it == iters - 1):
                self.history.append((it, float(loss.detach())))
        return self

    def rms_error(self, f, d):
        """RMS of (prediction - target) / target scale over all outputs."""
        import torch
        x, r = self.inputs(f)
        X = torch.from_numpy(x).to(self.device)
        Y = self.outputs_normalised(d, r)
        with torch.no_grad():
            y = self.forward(X).cpu().numpy()
        return float(np.sqrt(((y[:, :self.nout] - Y[:, :self.nout]) ** 2).mean()))

    def arrays(self):
        """FP32 host copies (W1, b1, W2, b2, W3, b3)."""
        return [np.ascontiguousarray(p.detach().cpu().numpy(), dtype=np.float32)
                for p in self.params]


class WarmStart:
    """A trained network uploaded to the GPU for one (system, order)."""

    def __init__(self, system, N, net, tau_var=-1, device=0):
        feat, k1, no = shape(system, N)
        if (k1, no) != (net.k1, net.no):
            raise ValueError(f"network widths {(net.k1, net.no)} do not fit the system "
                             f"({(k1, no)})")
        arrs = net.arrays() + [net.x_mean, net.x_scale, net.y_mean, net.y_scale]
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in arrs]
        self._keep = arrs
        fps = [a.ctypes.data_as(_lib.fp) for a in arrs]
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pypde_warm_start_create(system.handle, N, device, *fps,
                                                      int(tau_var), ctypes.byref(h)))
        self.handle = h
        self.system, self.N, self.net, self.tau_var = system, N, net, tau_var
        self.active = True  # train_warm_start sets it from its validation

    def free(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            _lib.lib().pypde_warm_start_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def validate(ws, w, dt, dX, tol=1e-12):
    """Newton iterations of the stiff predictor over held-out cells (one
    harvested step's sample, w (cells, N^ndim, V), one dt), from the plain
    guess and from the network: {"cells", "iters_plain", "iters_learned",
    "fallbacks"}."""
    V = w.shape[-1]
    w2 = np.ascontiguousarray(np.asarray(w, dtype=np.float64).reshape(-1, V))
    dX = np.ascontiguousarray(dX, dtype=np.float64)
    qh = np.zeros((w2.shape[0] * ws.N, V))
    L = _lib.lib()
    sp, sl = _lib.Stats(), _lib.Stats()
    _lib.check(L.pypde_predictor(ws.system.handle, _lib.c_ptr(w2), w2.shape[0], _lib.c_ptr(dX),
                                 len(dX), ws.N, True, float(dt), tol, _lib.c_ptr(qh), sp))
    _lib.check(L.pypde_predictor_guess(ws.system.handle, _lib.c_ptr(w2), w2.shape[0],
                                       _lib.c_ptr(dX), len(dX), ws.N, float(dt), tol, None,
                                       ws.handle, _lib.c_ptr(qh), sl))
    return {"cells": int(w.shape[0]), "iters_plain": int(sp.pred_iters),
            "iters_learned": int(sl.pred_iters), "fallbacks": int(sl.pred_fallbacks)}


def train_warm_start(Q0, tf, L, F=None, B=None, S=None, boundaryTypes="periodic", cfl=0.9,
                     order=2, tau_var=-1, steps=20, per_step=8192, iters=3000, batch=4096,
                     lr=2e-3, seed=0, device=0, newton_tol=None):
    """Harvest `steps` plain steps from Q0, train the network on the
    library's kernels on all but the last step's sample, upload it, and
    validate it on that held-out sample: the Newton iterations it needs
    against the plain guess's (ws.validation).  A network that saves none
    is marked inactive (ws.active False), and pde_solver then keeps the
    plain guess (a guess that costs iterations is never used).  Returns a
    WarmStart for pde_solver(..., warm_start=...)."""
    import torch
    ndim, V, N = Q0.ndim - 1, Q0.shape[-1], order
    w, qh, dt = harvest(Q0, tf, L, F, B, S, boundaryTypes, cfl, order, steps, per_step,
                        device, newton_tol)
    nval = min(per_step, w.shape[0] // 2)  # the last harvested step is held out
    w_val, dt_val = w[-nval:], dt[-1]
    w, qh, dt = w[:-nval], qh[:-nval], dt[:-nval]
    f = features(w, dt, N, ndim, V, tau_var)
    d = targets(w, qh, N, ndim, V)
    secondOrder = F is not None and nargs(F) == 3
    system = resolve_system(F, B, S, ndim, V, secondOrder)
    feat, k1, no = shape(system, N)
    with torch.cuda.device(device):
        net = WarmStartNet(feat, k1, no, d.shape[1], V, seed=seed, device=f"cuda:{device}")
        net.train(f, d, iters=iters, batch=batch, lr=lr, seed=seed, log_every=max(1, iters // 20))
    ws = WarmStart(system, N, net, tau_var, device)
    ws.train_rms = net.rms_error(f[:65536], d[:65536])
    ws.samples = f.shape[0]
    nX = np.array(Q0.shape[:-1])
    dX = np.array([L[i] / nX[i] for i in range(ndim)], dtype=np.float64)
    with torch.cuda.device(device):
        ws.validation = validate(ws, w_val, dt_val, dX, newton_tol or 1e-12)
    ws.active = ws.validation["iters_learned"] < ws.validation["iters_plain"]
    return ws
