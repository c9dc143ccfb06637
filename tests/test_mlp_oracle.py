"""The learned-residual oracle (oracle/mlp_oracle.py) pinned on the CPU:
bfloat16 rounding against torch's conversion, analytic gradients against
central finite differences, and the feature rows' plain-interpolation column
against the C oracle's own interpolated eigenvalues."""
import numpy as np
import pytest

from oracle import mlp_oracle as M


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(size=20000).astype(np.float32) * 10.0 ** rng.integers(-8, 8, 20000),
                        np.float32([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, -1 - 2 ** -8, 0.0, -0.0, 65504.0])])
    x = x.astype(np.float32)
    want = torch.from_numpy(x).to(torch.bfloat16).float().numpy()
    assert np.array_equal(M.bf16(x).view(np.uint32), want.view(np.uint32))


def test_layout_counts():
    lay, total = M.layout(80, 8)
    assert total == 128 * 80 + 128 + 2 * (128 * 128 + 128) + 8 * 128 + 8
    assert lay[3][2:] == (128, 8)
    assert M.feature_width(6) == 80 and M.feature_width(48) == 448 and M.feature_width(49) == 464


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(1)
    d_in, n_out, B, n = 16, 8, 6, 7
    p = M.init_params(d_in, n_out, seed=2).astype(np.float64)
    p += rng.normal(scale=0.05, size=p.size)  # non-zero biases
    X = rng.normal(size=(n, d_in))
    T = rng.normal(size=(n, B))
    loss, g = M.loss_and_grads(p, X, T, d_in, n_out, B, rounding=False)
    lay, _ = M.layout(d_in, n_out)
    idx = np.concatenate([rng.integers(w, w + i * o, 12) for w, _, i, o in lay] +
                         [rng.integers(b, b + o, 4) for _, b, _, o in lay])
    h = 1e-6
    for k in idx:
        pp = p.copy()
        pp[k] += h
        lp, _ = M.loss_and_grads(pp, X, T, d_in, n_out, B, rounding=False)
        pm = p.copy()
        pm[k] -= h
        lm, _ = M.loss_and_grads(pm, X, T, d_in, n_out, B, rounding=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-8, (k, fd, g[k])
    # padding outputs carry no gradient
    w3, b3, i3, o3 = lay[3]
    assert np.all(g[b3 + B:b3 + o3] == 0)


def test_adam_first_step_moves_by_lr():
    p = np.ones(5, np.float32)
    g = np.array([1, -2, 3, -4, 5], np.float32)
    q, m, v = M.adam(p, g, np.zeros(5, np.float32), np.zeros(5, np.float32), 1, 1e-2)
    assert np.allclose(q, p - 1e-2 * np.sign(g), rtol=0, atol=1e-6)


def test_feature_base_equals_oracle_interpolation():
    from _cases import crystal_case, values_vectors
    from oracle.oracle import Oracle

    c = crystal_case("diamond2", fraction=1 / 500)
    o = Oracle(c["tables"])
    rng = np.random.default_rng(4)
    Q = rng.uniform(-1, 1, (400, 3))
    rec = o.move_locate(Q)
    assert np.all(rec["status"] == 0)
    vals, _ = values_vectors(c)
    B = c["w"].shape[1]
    X, base = M.features(rec, c["w"], c["tables"]["knots"], c["tables"]["outer_B"], B, M.feature_width(B), 50.0)
    want, _, rc, st = o.interpolate_at(Q, vals)
    # the oracle interpolates FP64 values; the features use their FP32 copies
    assert np.allclose(base, want[:, :, 0], rtol=1e-6, atol=1e-5)
    assert np.all((X[:, 0:3] >= -1e-6) & (X[:, 0:3] <= 1 + 1e-6))
    assert np.allclose(X[:, 3:11].sum(axis=1), 1.0, atol=1e-5)
    assert np.allclose(X[:, 12 + 8 * B:12 + 9 * B] * 50.0, base, rtol=1e-6)
    box = X[:, 12 + 9 * B:15 + 9 * B]
    assert np.all((box >= -1e-6) & (box <= 1 + 1e-6))
    # distance to Γ: |q_ir| in Å⁻¹ over the longest side of the trellis box
    kn = c["tables"]["knots"]
    span = max(k[-1] - k[0] for k in kn)
    r = np.linalg.norm(rec["q_ir"] @ np.asarray(c["tables"]["outer_B"]).reshape(3, 3), axis=1)
    assert np.allclose(X[:, 15 + 9 * B], r / span, rtol=1e-5, atol=1e-7)
