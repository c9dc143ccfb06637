"""brx_ir_interpolate_at_noalloc: the query entry point for callers that must
not allocate device memory while they run (a serving loop that cannot take
cudaMalloc's device-wide synchronisation inside a request, or a plugin whose
host's caching pool owns the device memory).

It is checked through the C ABI against the regular entry point on two
calls in a row with different q (FP32, the tolerance of the other FP32
parity tests), against the oracle at FP64 storage (eigenvalues bit-exact,
eigenvectors within 1e-12, as the regular path), and the second call must
leave the device's free memory unchanged.  This file is collected last on
purpose: a failure here comes after every other test has run.
"""
import numpy as np
import pytest

from _cases import crystal_case, values_vectors
from brille_gb300 import BZTrellisQdc
from brille_gb300._lib import load
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

MAX_Q = 65536  # BRX_NOALLOC_MAX_Q in include/brx.h
OUT_F32 = 0x2


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    c = crystal_case("hex16")
    g = BZTrellisQdc(c["bz"], trellis=c["tr"])
    na = c["v"].shape[2]
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * na, 0, 2, 1], storage="f32")
    B = c["w"].shape[1]
    lib = load()
    h = g._handle()
    dev = torch.device("cuda")
    rng = np.random.default_rng(17)
    for call, n in enumerate((5000, 20000)):
        Q = torch.from_numpy(rng.uniform(-2, 2, size=(n, 3))).to(dev)
        ref_v = torch.empty((n, B), dtype=torch.float32, device=dev)
        ref_c = torch.empty((n, B, na, 3), dtype=torch.complex64, device=dev)
        g.query_into(Q, n, ref_v, ref_c, out_f32=True)
        got_v = torch.full((n, B), float("nan"), dtype=torch.float32, device=dev)
        got_c = torch.full((n, B, na, 3), float("nan"), dtype=torch.complex64, device=dev)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        st = lib.brx_ir_interpolate_at_noalloc(h, Q.data_ptr(), n, got_v.data_ptr(), got_c.data_ptr(), OUT_F32, None)
        assert st == 0, lib.brx_last_error(h).decode()
        torch.cuda.synchronize()
        if call == 1:
            # the first call on the device did its set-up; this one may not
            # take any device memory
            assert torch.cuda.mem_get_info()[0] == free0
        rv, gv = ref_v.cpu().numpy(), got_v.cpu().numpy()
        rc, gc = ref_c.cpu().numpy(), got_c.cpu().numpy()
        assert np.isfinite(gv).all() and np.isfinite(gc).all(), call
        assert np.abs(gv - rv).max() <= 2e-5 * np.abs(rv).max(), call
        assert np.abs(gc - rc).max() <= 1e-5, call


def test_noalloc_fp64_matches_oracle():
    """FP64 storage and outputs: eigenvalues bit-exact with the oracle,
    eigenvectors within 1e-12 (the bars of the regular FP64 path)."""
    torch = pytest.importorskip("torch")
    c = crystal_case("diamond8")
    g = BZTrellisQdc(c["bz"], trellis=c["tr"])
    na = c["v"].shape[2]
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * na, 0, 2, 1])
    B = c["w"].shape[1]
    lib = load()
    h = g._handle()
    Qh = np.random.default_rng(23).uniform(-1, 1, size=(3000, 3))
    ov, oc, rc, _ = Oracle(c["tables"]).interpolate_at(Qh, *values_vectors(c))
    assert rc == 0
    Q = torch.from_numpy(Qh).cuda()
    for _ in range(2):
        v = torch.full((len(Qh), B), float("nan"), dtype=torch.float64, device="cuda")
        e = torch.full((len(Qh), B, na, 3), float("nan"), dtype=torch.complex128, device="cuda")
        st = lib.brx_ir_interpolate_at_noalloc(h, Q.data_ptr(), len(Qh), v.data_ptr(), e.data_ptr(), 0, None)
        assert st == 0, lib.brx_last_error(h).decode()
        torch.cuda.synchronize()
        assert np.array_equal(v.cpu().numpy(), ov[:, :, 0])
        assert np.abs(e.cpu().numpy().reshape(oc.shape) - oc).max() < 1e-12


def test_noalloc_rejects_oversized_and_host_buffers():
    torch = pytest.importorskip("torch")
    c = crystal_case("diamond2")
    g = BZTrellisQdc(c["bz"], trellis=c["tr"])
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 6, 0, 2, 1], storage="f32")
    lib = load()
    h = g._handle()
    n = MAX_Q + 1
    Q = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    v = torch.empty((n, 6), dtype=torch.float32, device="cuda")
    e = torch.empty((n, 6, 2, 3), dtype=torch.complex64, device="cuda")
    assert lib.brx_ir_interpolate_at_noalloc(h, Q.data_ptr(), n, v.data_ptr(), e.data_ptr(), OUT_F32, None) == 1
    assert b"at most" in lib.brx_last_error(h)
    Qh = np.zeros((4, 3))
    vh = np.zeros((4, 6), np.float32)
    eh = np.zeros((4, 6, 2, 3), np.complex64)
    assert lib.brx_ir_interpolate_at_noalloc(h, Qh.ctypes.data, 4, vh.ctypes.data, eh.ctypes.data, OUT_F32,
                                             None) == 1
    if torch.cuda.device_count() > 1:
        # device memory of another GPU is refused, not read as peer memory
        Q1 = torch.zeros((4, 3), dtype=torch.float64, device="cuda:1")
        v0 = torch.empty((4, 6), dtype=torch.float32, device="cuda:0")
        e0 = torch.empty((4, 6, 2, 3), dtype=torch.complex64, device="cuda:0")
        assert lib.brx_ir_interpolate_at_noalloc(h, Q1.data_ptr(), 4, v0.data_ptr(), e0.data_ptr(), OUT_F32,
                                                 None) == 1
