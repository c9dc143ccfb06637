"""Learned eigenvalue residual on top of a (coarse) trellis.

A ResidualModel predicts, per mode, the exact eigenvalue minus its plain
trellis interpolation.  It is trained on the GPU by the library's own
forward/backward/Adam kernels (brx_mlp_train_step) on exact samples of the
lattice-dynamics model that fills the trellis vertices, then attached to a
grid (brx_set_residual_model): every later query of that grid adds the
predicted residual to its interpolated eigenvalues inside the query
pipeline.  A predicted correction larger than `clip` is dropped, keeping the
plain interpolation for that q and mode.

The reference has no learned part; this module has no counterpart there.
Device memory and streams come from torch; every computation is a libbrx
kernel.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi
from ._lib import check, load

WIDTH = 128


def feature_width(n_modes):
    """Smallest legal input width (a multiple of 16) for n_modes eigenvalues."""
    return (16 + 9 * n_modes + 15) // 16 * 16


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("the learned residual needs a CUDA device")
    return torch


def locate_device(grid, Q, ir=True):
    """Locate records of device-resident Q (torch float64, n × 3) as a dict
    of torch tensors on the same device."""
    torch = _torch()
    n = Q.shape[0]
    dev = Q.device
    rec = dict(q_ir=torch.empty((n, 3), dtype=torch.float64, device=dev),
               tau=torch.empty((n, 3), dtype=torch.int32, device=dev),
               rot=torch.empty((n, 2), dtype=torch.int32, device=dev),
               node=torch.empty((n, 2), dtype=torch.int32, device=dev),
               n_weights=torch.empty(n, dtype=torch.int32, device=dev),
               vertex=torch.empty((n, 8), dtype=torch.int32, device=dev),
               weight=torch.empty((n, 8), dtype=torch.float64, device=dev),
               status=torch.empty(n, dtype=torch.int32, device=dev))
    lo = _records_struct(rec)
    h = grid._handle()
    check(load().brx_locate(h, Q.data_ptr(), n, 1 if ir else 0, 0, C.byref(lo), None), h)
    return rec


def _records_struct(rec):
    lo = _abi.LocateOut()
    for k, v in rec.items():
        setattr(lo, k, C.cast(C.c_void_p(v.data_ptr()), type(getattr(lo, k))))
    return lo


class ResidualModel:
    """MLP d_in → 128 → 128 → 128 → n_out (GELU), bf16 weights, FP32
    accumulation, predicting n_modes eigenvalue residuals."""

    def __init__(self, n_modes, *, n_out=None, d_in=None, seed=0, fp32_training=False):
        self.n_modes = int(n_modes)
        self.d_in = int(d_in or feature_width(n_modes))
        self.n_out = int(n_out or max(8, (n_modes + 7) // 8 * 8))
        flags = _abi.BRX_MLP_FP32 if fp32_training else 0
        self.dims = _abi.MlpDims(self.d_in, self.n_out, self.n_modes, flags)
        n = load().brx_mlp_param_count(C.byref(self.dims))
        if n < 0:
            raise ValueError(f"invalid model dimensions d_in={self.d_in} n_out={self.n_out} n_modes={n_modes}")
        self.n_params = int(n)
        self.params = self.init_params(seed)
        self.omega_scale = 1.0
        self.res_scale = 1.0
        self.clip = 0.0
        self.history = []

    # ----------------------------------------------------------- parameters
    def layout(self):
        """[(W offset, b offset, in, out)] of the four layers."""
        dims = [(self.d_in, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH), (WIDTH, self.n_out)]
        out, o = [], 0
        for i, n in dims:
            out.append((o, o + n * i, i, n))
            o += n * i + n
        assert o == self.n_params
        return out

    def init_params(self, seed):
        """Uniform ±1/√fan_in weights, zero biases."""
        rng = np.random.default_rng(seed)
        p = np.zeros(self.n_params, np.float32)
        for w, _, i, n in self.layout():
            lim = 1.0 / math.sqrt(i)
            p[w:w + n * i] = rng.uniform(-lim, lim, n * i).astype(np.float32)
        return p

    # ------------------------------------------------------------- features
    def features(self, grid, rec, omega_scale=None, stream=None):
        """(X n × d_in float32, base n × n_modes float32) on the device from
        locate records (locate_device)."""
        torch = _torch()
        n = rec["status"].shape[0]
        dev = rec["status"].device
        X = torch.empty((n, self.d_in), dtype=torch.float32, device=dev)
        base = torch.empty((n, self.n_modes), dtype=torch.float32, device=dev)
        lo = _records_struct(rec)
        h = grid._handle()
        om = float(omega_scale if omega_scale is not None else self.omega_scale)
        st = load().brx_mlp_features(h, C.byref(lo), n, C.byref(self.dims), om, X.data_ptr(), base.data_ptr(),
                                     stream)
        check(st, h)
        return X, base

    # ------------------------------------------------------------- training
    def fit(self, X, T, *, epochs=30, batch=4096, lr=2e-3, lr_min=2e-5, seed=0, stream=None, log=None):
        """Adam with a cosine learning-rate decay on (X, T) device tensors;
        T are residuals already divided by res_scale.  Returns the mean
        training loss per epoch."""
        torch = _torch()
        lib = load()
        dev = X.device
        n = X.shape[0]
        if n < batch:
            batch = n
        P = torch.from_numpy(self.params.copy()).to(dev)
        G = torch.zeros_like(P)
        m = torch.zeros_like(P)
        v = torch.zeros_like(P)
        ws = torch.empty(int(lib.brx_mlp_workspace_floats(C.byref(self.dims), batch)), dtype=torch.float32,
                         device=dev)
        loss = torch.zeros(1, dtype=torch.float32, device=dev)
        acc = torch.zeros(1, dtype=torch.float64, device=dev)
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        per_epoch = n // batch
        total = per_epoch * epochs
        step = 0
        hist = []
        for ep in range(epochs):
            perm = torch.randperm(n, device=dev, generator=gen)
            Xs = X[perm].contiguous()
            Ts = T[perm].contiguous()
            acc.zero_()
            for k in range(per_epoch):
                step += 1
                lr_t = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * (step - 1) / max(1, total - 1)))
                st = lib.brx_mlp_train_step(C.byref(self.dims), P.data_ptr(), G.data_ptr(), m.data_ptr(),
                                            v.data_ptr(), step, lr_t, Xs[k * batch:].data_ptr(),
                                            Ts[k * batch:].data_ptr(), batch, ws.data_ptr(), loss.data_ptr(), stream)
                check(st)
                acc += loss
            hist.append(float(acc.item()) / per_epoch)
            if log:
                log(f"[learned] epoch {ep + 1}/{epochs} loss {hist[-1]:.4e}")
        self.params = P.cpu().numpy()
        self.history.extend(hist)
        return hist

    def train_on(self, grid, Q, exact, **kw):
        """Locate Q (n × 3 r.l.u., host) on grid, build features, set the
        scales from the residuals and fit.  exact: n × n_modes eigenvalues of
        the exact model at Q.  Returns the fit history."""
        torch = _torch()
        dev = torch.device("cuda", grid.device)
        Qd = torch.from_numpy(np.ascontiguousarray(Q, dtype=np.float64)).to(dev)
        rec = locate_device(grid, Qd)
        vals = np.asarray(grid.values).reshape(len(grid.values), -1)
        self.omega_scale = float(max(1e-6, np.max(np.abs(vals))))
        X, base = self.features(grid, rec)
        E = torch.from_numpy(np.ascontiguousarray(exact, dtype=np.float64)).to(dev)
        R = E - base.double()
        ok = torch.isfinite(R).all(dim=1)
        R = R[ok]
        X = X[ok].contiguous()
        self.res_scale = float(max(1e-12, R.std().item()))
        self.clip = float(4.0 * R.abs().max().item())
        T = (R / self.res_scale).float().contiguous()
        return self.fit(X, T, **kw)

    def predict(self, X, stream=None):
        """Network outputs (batch × n_out, residual units) in training
        arithmetic, for checks."""
        torch = _torch()
        lib = load()
        n = X.shape[0]
        P = torch.from_numpy(self.params).to(X.device)
        ws = torch.empty(int(lib.brx_mlp_workspace_floats(C.byref(self.dims), n)), dtype=torch.float32,
                         device=X.device)
        Y = torch.empty((n, self.n_out), dtype=torch.float32, device=X.device)
        check(lib.brx_mlp_forward(C.byref(self.dims), P.data_ptr(), X.data_ptr(), n, Y.data_ptr(), ws.data_ptr(),
                                  stream))
        return Y

    # ------------------------------------------------------------ attaching
    def attach(self, grid):
        """Every later query of grid adds the predicted residual."""
        h = grid._handle()
        p = np.ascontiguousarray(self.params, np.float32)
        check(load().brx_set_residual_model(h, C.byref(self.dims), p.ctypes.data, self.omega_scale, self.res_scale,
                                            self.clip), h)

    @staticmethod
    def detach(grid):
        h = grid._handle()
        check(load().brx_set_residual_model(h, None, None, 1.0, 1.0, 0.0), h)

    # ----------------------------------------------------------- save/load
    def save(self, path):
        np.savez(path, params=self.params, dims=np.array([self.d_in, self.n_out, self.n_modes]),
                 scales=np.array([self.omega_scale, self.res_scale, self.clip]))

    @classmethod
    def load(cls, path):
        z = np.load(path)
        d_in, n_out, n_modes = (int(x) for x in z["dims"])
        m = cls(n_modes, n_out=n_out, d_in=d_in)
        m.params = z["params"].astype(np.float32)
        m.omega_scale, m.res_scale, m.clip = (float(x) for x in z["scales"])
        return m
