"""Bounded device waits that run out, without faulting or hanging anything.

BRX_FLAG_TEST_TIMEOUT makes the first bounded wait of every warp of the FP32
vectors gather (and of every slot of the tensor-core residual network) wait
on an mbarrier that nothing completes.  The wait gives up after about a
millisecond; the kernels then take their real error path: the error flag,
the drain of the bulk copies still in flight (on its own long limit), and
for the tensor-core kernel the release of its tensor memory.  The call must
return BRX_ERR_TIMEOUT with its message, and the next call on the same
handle must be complete and equal to a query made before.
"""
import numpy as np
import pytest

from _cases import crystal_case
from brille_gb300 import BZTrellisQdc
from brille_gb300._lib import load
from brille_gb300.grid import BZTrellisQdd
from brille_gb300.learned import ResidualModel

pytestmark = pytest.mark.gpu

OUT_F32 = 0x2
TEST_TIMEOUT = 0x100  # BRX_FLAG_TEST_TIMEOUT in include/brx.h
ERR_TIMEOUT = 11      # BRX_ERR_TIMEOUT


def _expect_timeout(lib, h, Q, v, c):
    st = lib.brx_ir_interpolate_at(h, Q.ctypes.data, len(Q), v.ctypes.data, c.ctypes.data if c is not None else None,
                                   OUT_F32 | TEST_TIMEOUT, None)
    assert st == ERR_TIMEOUT, (st, lib.brx_last_error(h))
    assert b"bounded device-side wait ran out" in lib.brx_last_error(h)


def test_gather_wait_runs_out_and_handle_recovers():
    c = crystal_case("hex16")
    na = c["v"].shape[2]
    g = BZTrellisQdc(c["bz"], trellis=c["tr"])
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * na, 0, 2, 1], storage="f32")
    Q = np.random.default_rng(31).uniform(-2, 2, size=(20_000, 3))
    ref_v, ref_c = g.ir_interpolate_at(Q, out_f32=True)
    lib = load()
    h = g._handle()
    v = np.zeros_like(ref_v)
    e = np.zeros_like(ref_c)
    _expect_timeout(lib, h, Q, v, e)
    v2, c2 = g.ir_interpolate_at(Q, out_f32=True)
    assert np.array_equal(v2, ref_v) and np.array_equal(c2, ref_c)


def test_tensor_core_wait_runs_out_and_handle_recovers():
    c = crystal_case("diamond2", fraction=1 / 625)
    B = c["w"].shape[1]
    g = BZTrellisQdd(c["bz"], trellis=c["tr"])
    g.fill(c["w"][:, :, None], [1, 0, 0, 0, 3], storage="f32")
    m = ResidualModel(B, seed=3)
    m.attach(g)
    Q = np.random.default_rng(32).uniform(-1, 1, size=(50_000, 3))
    ref_v, _ = g.ir_interpolate_at(Q, out_f32=True)
    lib = load()
    h = g._handle()
    v = np.zeros_like(ref_v)
    _expect_timeout(lib, h, Q, v, None)
    v2, _ = g.ir_interpolate_at(Q, out_f32=True)
    assert np.array_equal(v2, ref_v)
