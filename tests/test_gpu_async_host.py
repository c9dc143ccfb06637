"""Asynchronous queries with page-locked host Q and outputs.

Several calls are queued, on one stream per output buffer, into a ring of
two pinned buffers (each refilled after an event behind its previous call),
as a serving loop would stream results out; every call's outputs must equal the
synchronous call's, bit for bit.  Pageable host buffers with the flag fall
back to a synchronous call with the same results.
"""
import numpy as np
import pytest

from _cases import crystal_case
from brille_gb300 import BZTrellisQdc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_async_pinned_host_ring(storage, monkeypatch):
    monkeypatch.setenv("BRX_HOST_CHUNK_MB", "8")  # several staging chunks per call
    c = crystal_case("hex16")
    na = c["v"].shape[2]
    g = BZTrellisQdc(c["bz"], trellis=c["tr"])
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * na, 0, 2, 1], storage=storage)
    B = c["w"].shape[1]
    out_f32 = storage == "f32"
    fdt = torch.float32 if out_f32 else torch.float64
    cdt = torch.complex64 if out_f32 else torch.complex128
    n, calls = 3000, 5
    Qall = np.random.default_rng(41).uniform(-2, 2, size=(calls * n, 3))
    ref = [g.ir_interpolate_at(Qall[k * n:(k + 1) * n], out_f32=out_f32) for k in range(calls)]
    Qh = torch.from_numpy(Qall).pin_memory()
    vh = [torch.empty((n, B), dtype=fdt, pin_memory=True) for _ in range(2)]
    ch = [torch.empty((n, B, na, 3), dtype=cdt, pin_memory=True) for _ in range(2)]
    s = [torch.cuda.Stream(), torch.cuda.Stream()]  # one per output buffer
    done = [None, None]
    for k in range(calls):
        sl = k % 2
        if done[sl] is not None:
            done[sl].synchronize()
            v, e = ref[k - 2]
            assert np.array_equal(vh[sl].numpy(), v) and np.array_equal(ch[sl].numpy(), e), k - 2
        g.query_into(Qh[k * n:(k + 1) * n], n, vh[sl], ch[sl], out_f32=out_f32, async_=True,
                     stream=s[sl].cuda_stream)
        done[sl] = torch.cuda.Event()
        done[sl].record(s[sl])
    g.sync()
    for k in (calls - 2, calls - 1):
        v, e = ref[k]
        assert np.array_equal(vh[k % 2].numpy(), v) and np.array_equal(ch[k % 2].numpy(), e), k


def test_async_flag_with_pageable_host_buffers_is_synchronous():
    c = crystal_case("diamond8")
    na = c["v"].shape[2]
    g = BZTrellisQdc(c["bz"], trellis=c["tr"])
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * na, 0, 2, 1])
    Q = np.random.default_rng(42).uniform(-1, 1, size=(2000, 3))
    v0, e0 = g.ir_interpolate_at(Q)
    v = np.zeros_like(v0)
    e = np.zeros_like(e0)
    g.query_into(Q, len(Q), v, e, async_=True)
    assert np.array_equal(v, v0) and np.array_equal(e, e0)
    g.sync()
