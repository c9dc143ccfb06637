"""The learned eigenvalue residual on the GPU, against the CPU oracle
(oracle/mlp_oracle.py).

Bars: feature rows bit-exact (same operation order in FP64, one FP32
rounding); gradients of the FP32 training mode within 1e-4 of the FP64
oracle (relative to the largest gradient of each layer); gradients of the
bf16 training mode within 2e-2 in relative L2 norm of the oracle evaluated on
the same bf16-rounded operands (accumulation order moves a few activations
across a bf16 rounding boundary); Adam within 1e-5 relative; the residual
the query pipeline adds within 2e-2 of the oracle's bf16 forward (relative
to the largest residual); and training makes the coarse trellis more
accurate against the exact lattice-dynamics model than it is without.
"""
import numpy as np
import pytest

from _cases import crystal_case
from brille_gb300.grid import BZTrellisQdd
from brille_gb300.learned import ResidualModel, locate_device
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def coarse():
    c = crystal_case("diamond2", fraction=1 / 625)
    g = BZTrellisQdd(c["bz"], trellis=c["tr"])
    g.fill(c["w"][:, :, None], [1, 0, 0, 0, 3])
    return c, g


def _dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def test_features_bit_exact(coarse):
    c, g = coarse
    B = c["w"].shape[1]
    rng = np.random.default_rng(0)
    Q = rng.uniform(-1, 1, (5000, 3))
    rec = locate_device(g, _dev(Q))
    m = ResidualModel(B)
    X, base = m.features(g, rec, omega_scale=37.5)
    host = {k: v.cpu().numpy() for k, v in rec.items()}
    Xo, bo = M.features(host, c["w"], c["tables"]["knots"], c["tables"]["outer_B"], B, m.d_in, 37.5)
    assert np.array_equal(X.cpu().numpy().view(np.uint32), Xo.view(np.uint32))
    assert np.array_equal(base.cpu().numpy(), bo, equal_nan=True)


def _grad_case(seed, fp32, n=3000):
    rng = np.random.default_rng(seed)
    m = ResidualModel(6, fp32_training=fp32, seed=seed)
    m.params = (m.params + rng.normal(scale=0.02, size=m.n_params)).astype(np.float32)
    X = rng.normal(size=(n, m.d_in)).astype(np.float32)
    X[:, 72:] = 0.0
    T = rng.normal(size=(n, 6)).astype(np.float32)
    return m, X, T


def _gpu_grads(m, X, T):
    import ctypes as C
    from brille_gb300._lib import check, load

    lib = load()
    n = X.shape[0]
    P = _dev(m.params)
    G = torch.zeros_like(P)
    ws = torch.empty(int(lib.brx_mlp_workspace_floats(C.byref(m.dims), n)), dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    Xd, Td = _dev(X), _dev(T)
    check(lib.brx_mlp_train_step(C.byref(m.dims), P.data_ptr(), G.data_ptr(), None, None, 0, 0.0, Xd.data_ptr(),
                                 Td.data_ptr(), n, ws.data_ptr(), loss.data_ptr(), None))
    torch.cuda.synchronize()
    return float(loss.item()), G.cpu().numpy()


def test_gradients_fp32_mode_match_oracle():
    m, X, T = _grad_case(1, fp32=True)
    loss, g = _gpu_grads(m, X, T)
    lo, go = M.loss_and_grads(m.params, X, T, m.d_in, m.n_out, 6, rounding=False)
    assert abs(loss - lo) <= 1e-5 * lo
    lay, _ = M.layout(m.d_in, m.n_out)
    for w, b, i, o in lay:
        for a, z in ((w, w + i * o), (b, b + o)):
            scale = np.max(np.abs(go[a:z]))
            assert np.max(np.abs(g[a:z] - go[a:z])) <= 1e-4 * scale, (a, z)


def test_gradients_bf16_mode_match_oracle():
    m, X, T = _grad_case(2, fp32=False)
    loss, g = _gpu_grads(m, X, T)
    lo, go = M.loss_and_grads(m.params, X, T, m.d_in, m.n_out, 6, rounding=True)
    assert abs(loss - lo) <= 1e-3 * lo
    lay, _ = M.layout(m.d_in, m.n_out)
    for w, b, i, o in lay:
        for a, z in ((w, w + i * o), (b, b + o)):
            err = np.linalg.norm(g[a:z] - go[a:z]) / np.linalg.norm(go[a:z])
            assert err <= 2e-2, (a, z, err)


def test_adam_step_matches_oracle():
    import ctypes as C
    from brille_gb300._lib import check, load

    lib = load()
    m, X, T = _grad_case(3, fp32=True, n=512)
    n = X.shape[0]
    P = _dev(m.params)
    G = torch.zeros_like(P)
    mm = torch.full_like(P, 0.01)
    vv = torch.full_like(P, 0.02)
    ws = torch.empty(int(lib.brx_mlp_workspace_floats(C.byref(m.dims), n)), dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    check(lib.brx_mlp_train_step(C.byref(m.dims), P.data_ptr(), G.data_ptr(), mm.data_ptr(), vv.data_ptr(), 3,
                                 1e-3, _dev(X).data_ptr(), _dev(T).data_ptr(), n, ws.data_ptr(), loss.data_ptr(),
                                 None))
    torch.cuda.synchronize()
    g = G.cpu().numpy()
    po, mo, vo = M.adam(m.params, g, np.full(m.n_params, 0.01, np.float32), np.full(m.n_params, 0.02, np.float32),
                        3, 1e-3)
    assert np.allclose(mm.cpu().numpy(), mo, rtol=1e-6, atol=0)
    assert np.allclose(vv.cpu().numpy(), vo, rtol=1e-6, atol=0)
    assert np.allclose(P.cpu().numpy(), po, rtol=1e-5, atol=1e-8)


def test_attached_residual_matches_oracle_forward(coarse):
    """The tensor-core inference inside the query adds res_scale·MLP(features)."""
    c, g = coarse
    B = c["w"].shape[1]
    rng = np.random.default_rng(5)
    m = ResidualModel(B, seed=7)
    m.params = (m.params + rng.normal(scale=0.05, size=m.n_params)).astype(np.float32)
    m.omega_scale, m.res_scale, m.clip = 40.0, 0.3, 0.0
    Q = rng.uniform(-1, 1, (3001, 3))
    plain, _ = g.ir_interpolate_at(Q)
    m.attach(g)
    try:
        corr, _ = g.ir_interpolate_at(Q)
    finally:
        ResidualModel.detach(g)
    again, _ = g.ir_interpolate_at(Q)
    assert np.array_equal(again, plain)
    rec = g.locate(Q)
    X, _ = M.features(rec, c["w"], c["tables"]["knots"], c["tables"]["outer_B"], B, m.d_in, m.omega_scale)
    _, _, Y = M.forward(m.params, X, m.d_in, m.n_out, rounding=True)
    want = Y[:, :B] * m.res_scale
    got = (corr - plain)[:, :, 0]
    scale = np.max(np.abs(want))
    assert scale > 0
    assert np.max(np.abs(got - want)) <= 2e-2 * scale


def test_clip_keeps_plain_interpolation(coarse):
    c, g = coarse
    B = c["w"].shape[1]
    m = ResidualModel(B, seed=8)
    m.omega_scale, m.res_scale, m.clip = 40.0, 1.0, 1e-30
    Q = np.random.default_rng(6).uniform(-1, 1, (500, 3))
    plain, _ = g.ir_interpolate_at(Q)
    m.attach(g)
    try:
        corr, _ = g.ir_interpolate_at(Q)
    finally:
        ResidualModel.detach(g)
    assert np.array_equal(corr, plain)


def test_training_beats_plain_coarse_interpolation(coarse):
    """Trained on exact samples, the corrected coarse trellis is closer to
    the exact model on held-out q than the plain coarse trellis."""
    c, g = coarse
    B = c["w"].shape[1]
    model = c["model"]
    rng = np.random.default_rng(9)
    Qt = rng.uniform(-1, 1, (200_000, 3))
    wt, _ = model.modes(Qt, chunk=8192)
    m = ResidualModel(B, seed=0)
    hist = m.train_on(g, Qt, wt, epochs=10, batch=1024, lr=2e-3)
    assert hist[-1] < 0.5 * hist[0]
    Qe = rng.uniform(-1, 1, (20_000, 3))
    we, _ = model.modes(Qe, chunk=8192)
    plain, _ = g.ir_interpolate_at(Qe)
    m.attach(g)
    try:
        corr, _ = g.ir_interpolate_at(Qe)
    finally:
        ResidualModel.detach(g)
    e_plain = np.sqrt(np.mean((plain[:, :, 0] - we) ** 2))
    e_corr = np.sqrt(np.mean((corr[:, :, 0] - we) ** 2))
    assert e_corr < 0.5 * e_plain, (e_plain, e_corr)
