"""Batched queries over many grids in one launch per stage (brx_batch_*).

A BatchQuery is planned for fixed q counts per grid.  Every run is one
locate launch over all grids' q, one counting sort, one values gather and
one vectors gather; `capture()` records the run in a CUDA graph that
`launch()` replays, and `tune()` lets the library time its launch shapes on
the batch itself.  Q and outputs are device tensors (torch), with the same
shapes as each grid's own ir_interpolate_at.

The reference answers one grid per call; this batched entry point has no
counterpart there.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._lib import BrxError, load

_CONFIG_KEYS = ("locate_threads", "locate_ctas_per_sm", "q_per_tile", "values_smem_kb", "vectors_smem_kb",
                "values_ctas_per_sm", "vectors_ctas_per_sm", "tiles", "values_gather_warps", "vectors_gather_warps",
                "warp_min_groups", "small_q_per_group")


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("batched queries need a CUDA device")
    return torch


class BatchQuery:
    def __init__(self, grids, n_q, *, ir=True, out_f32=False, no_move=False):
        self.grids = list(grids)
        self.n_q = [int(x) for x in n_q]
        if len(self.n_q) != len(self.grids) or not self.grids:
            raise ValueError("one q count per grid is required")
        for g in self.grids:
            if g._fill is None:
                raise RuntimeError("The interpolation data must be filled before interpolating.")
        self.out_f32 = bool(out_f32)
        flags = (_abi.BRX_FLAG_OUT_F32 if out_f32 else 0) | (_abi.BRX_FLAG_NO_MOVE if no_move else 0)
        n = len(self.grids)
        hs = (C.c_void_p * n)(*[g._handle().value for g in self.grids])
        nq = (C.c_int64 * n)(*self.n_q)
        b = C.c_void_p()
        st = load().brx_batch_create(hs, n, nq, 1 if ir else 0, flags, C.byref(b))
        if st != 0:
            raise BrxError(st, f"brx_batch_create failed with status {st} (items must share device, storage and "
                               "element kinds)")
        self._b = b
        self._keep = None

    def __del__(self):
        try:
            if getattr(self, "_b", None) is not None and self._b.value:
                load().brx_batch_destroy(self._b)
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            raise BrxError(st, load().brx_batch_last_error(self._b).decode())

    # -------------------------------------------------------------- buffers
    def outputs(self, device=None):
        """Freshly allocated (values, vectors) device tensors, one per grid."""
        torch = _torch()
        vals, vecs = [], []
        for g, n in zip(self.grids, self.n_q):
            f = g._fill
            dev = device or torch.device("cuda", g.device)
            vdt = f["vdtype"]
            cdt = f["cdtype"]
            tv = _tdtype(torch, vdt, self.out_f32)
            vals.append(torch.empty((n,) + tuple(f["vshape"]), dtype=tv, device=dev))
            if f["cshape"] is not None:
                vecs.append(torch.empty((n,) + tuple(f["cshape"]), dtype=_tdtype(torch, cdt, self.out_f32),
                                        device=dev))
            else:
                vecs.append(None)
        return vals, vecs

    def set_io(self, Qs, values, vectors=None):
        n = len(self.grids)
        q = (C.c_void_p * n)(*[t.data_ptr() for t in Qs])
        v = (C.c_void_p * n)(*[t.data_ptr() for t in values])
        c = None
        if vectors is not None and any(x is not None for x in vectors):
            c = (C.c_void_p * n)(*[t.data_ptr() for t in vectors])
        self._keep = (Qs, values, vectors)
        self._check(load().brx_batch_set_io(self._b, q, v, c))

    # ----------------------------------------------------------------- runs
    def run(self, stream=None):
        self._check(load().brx_batch_run(self._b, stream))

    def capture(self, stream=None):
        self._check(load().brx_batch_capture(self._b, stream))

    def launch(self, stream=None):
        self._check(load().brx_batch_launch(self._b, stream))

    def sync(self, stream=None):
        item = C.c_int32(-1)
        st = load().brx_batch_sync(self._b, stream, C.byref(item))
        if st != 0:
            err = BrxError(st, load().brx_batch_last_error(self._b).decode())
            err.item = int(item.value)
            raise err

    def tune(self, stream=None, reps=2):
        self._check(load().brx_batch_tune(self._b, stream, int(reps)))
        return self.config()

    def set_config(self, cfg):
        """Apply launch shapes as config() returns them (a dict; derived
        entries are ignored) and re-plan; drops a captured graph."""
        v = (C.c_int32 * len(_CONFIG_KEYS))(*(int(cfg.get(k, 0)) for k in _CONFIG_KEYS))
        self._check(load().brx_batch_set_config(self._b, v, len(_CONFIG_KEYS)))
        return self.config()

    def config(self):
        cfg = (C.c_int32 * len(_CONFIG_KEYS))()
        self._check(load().brx_batch_config(self._b, cfg, len(_CONFIG_KEYS)))
        return dict(zip(_CONFIG_KEYS, (int(x) for x in cfg)))

    def launch_count(self):
        return int(load().brx_batch_launch_count(self._b))

    def query(self, Qs, stream=None):
        """Run the batch once on device Q tensors; returns the outputs."""
        vals, vecs = self.outputs()
        self.set_io(Qs, vals, vecs)
        self.run(stream)
        self.sync(stream)
        return vals, vecs


def _tdtype(torch, np_dtype, f32):
    if np.dtype(np_dtype) == np.complex128:
        return torch.complex64 if f32 else torch.complex128
    return torch.float32 if f32 else torch.float64
