"""CPU oracle for the learned eigenvalue residual: feature rows, the MLP's
forward pass, its gradients and one Adam update, in numpy.

Test infrastructure only.  This file is imported by tests/, by the package's
smoke check and by bench.py's CPU baseline, never by the product path.

The reference has no learned part, so there is no reference code to follow.
This file restates the network that include/brx.h defines (d_in → 128 → 128
→ 128 → n_out, GELU in its tanh form, mean squared error over the first
n_modes outputs; the device's inference evaluates tanh with the
special-function unit's approximation, about 2^-11 relative).  It is pinned two ways: its analytic gradients agree with central
finite differences in FP64 (tests/test_mlp_oracle.py), and its feature base
column equals the C oracle's own interpolated eigenvalues.

bfloat16 rounding is round-to-nearest-even on the top 16 bits of the float32
pattern, which is what __float2bfloat16_rn does for finite values.
"""
from __future__ import annotations

import numpy as np

WIDTH = 128


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even), as float32."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def feature_width(n_modes):
    """Smallest legal d_in (a multiple of 16) for n_modes eigenvalues."""
    need = 16 + 9 * n_modes
    return (need + 15) // 16 * 16


def layout(d_in, n_out):
    """[(W offset, b offset, in, out)] of the four layers in the flat vector."""
    dims = [(d_in, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH), (WIDTH, n_out)]
    out, o = [], 0
    for i, n in dims:
        out.append((o, o + n * i, i, n))
        o += n * i + n
    return out, o


def unpack(params, d_in, n_out):
    lay, total = layout(d_in, n_out)
    p = np.asarray(params)
    assert p.size == total
    return [(p[w:w + n * i].reshape(n, i), p[b:b + n]) for w, b, i, n in lay]


def init_params(d_in, n_out, seed=0):
    """Uniform ±1/√fan_in weights, zero biases (float32)."""
    rng = np.random.default_rng(seed)
    lay, total = layout(d_in, n_out)
    p = np.zeros(total, np.float32)
    for w, b, i, n in lay:
        lim = 1.0 / np.sqrt(i)
        p[w:w + n * i] = rng.uniform(-lim, lim, n * i).astype(np.float32)
    return p


GELU_C = np.sqrt(2.0 / np.pi)
GELU_A = 0.044715


def gelu(x):
    """GELU in its tanh form."""
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + GELU_A * x ** 3)))


def gelu_grad(x):
    t = np.tanh(GELU_C * (x + GELU_A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * x * x)


def forward(params, X, d_in, n_out, rounding=True):
    """FP64 forward pass on bf16-rounded operands (rounding=True, the GPU's
    arithmetic up to FP32 accumulation order) or on the FP64 values as given
    (rounding=False, for finite differences and the FP32 training mode).

    Returns (Z list, H list, Y): Z the pre-activations of the three hidden
    layers, H their activations (rounded like the GPU's), Y the outputs."""
    layers = unpack(np.asarray(params, np.float32 if rounding else np.float64), d_in, n_out)
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    H = r(X).astype(np.float64)
    Zs, Hs = [], []
    for l, (W, b) in enumerate(layers):
        Z = H @ r(W).astype(np.float64).T + r(b).astype(np.float64)
        if l < 3:
            Zs.append(Z)
            Hn = gelu(Z)
            H = r(Hn.astype(np.float32)).astype(np.float64) if rounding else Hn
            Hs.append(H)
        else:
            Y = Z
    return Zs, Hs, Y


def loss_and_grads(params, X, T, d_in, n_out, n_modes, rounding=True):
    """Mean squared error over the first n_modes outputs and its gradient
    (straight through the bf16 rounding), both FP64."""
    layers = unpack(np.asarray(params, np.float32 if rounding else np.float64), d_in, n_out)
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    Zs, Hs, Y = forward(params, X, d_in, n_out, rounding)
    M = X.shape[0]
    E = Y[:, :n_modes] - T
    loss = float(np.sum(E * E) / (M * n_modes))
    dZ = np.zeros_like(Y)
    dZ[:, :n_modes] = 2.0 * E / (M * n_modes)
    grads = []
    X64 = r(X).astype(np.float64)
    for l in range(3, -1, -1):
        Hprev = Hs[l - 1] if l > 0 else X64
        gW = dZ.T @ Hprev
        gb = dZ.sum(axis=0)
        grads.append((gW, gb))
        if l == 0:
            break
        W = r(layers[l][0]).astype(np.float64)
        dZ = (dZ @ W) * gelu_grad(Zs[l - 1])
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def adam(params, grads, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update in float32 (returns new params, m, v)."""
    p = np.asarray(params, np.float32)
    g = np.asarray(grads, np.float32)
    m = (np.float32(b1) * m + np.float32(1 - b1) * g).astype(np.float32)
    v = (np.float32(b2) * v + np.float32(1 - b2) * g * g).astype(np.float32)
    c1 = np.float32(1 - b1 ** step)
    c2 = np.float32(1 - b2 ** step)
    p = (p - np.float32(lr) * (m / c1) / (np.sqrt(v / c2) + np.float32(eps))).astype(np.float32)
    return p, m, v


def features(records, values, knots, outer_B, n_modes, d_in, omega_scale):
    """Feature rows (n × d_in float32) and plain interpolated eigenvalues
    (n × n_modes float32, NaN where the locate failed) from locate records
    (dict of q_ir, node, n_weights, vertex, weight, status), vertex
    eigenvalues (n_vertices × n_modes) and the trellis knots.  Every step is
    one IEEE float32 operation in the device code's order."""
    f32 = np.float32
    q = np.asarray(records["q_ir"], np.float64).astype(f32)
    n = q.shape[0]
    B = n_modes
    X = np.zeros((n, d_in), f32)
    base = np.full((n, B), np.nan, f32)
    ok = np.asarray(records["status"]) == 0
    vals32 = np.asarray(values).reshape(-1, B).astype(f32)
    inv = f32(1.0) / f32(omega_scale)
    Bm = np.asarray(outer_B, np.float64).reshape(3, 3).astype(f32)
    # x_d = (B0d q0 + B1d q1) + B2d q2
    x = np.stack([(Bm[0, d] * q[:, 0] + Bm[1, d] * q[:, 1]) + Bm[2, d] * q[:, 2] for d in range(3)], axis=1)
    node = np.asarray(records["node"]).reshape(n, 2)
    nx = len(knots[0]) - 1
    ny = len(knots[1]) - 1
    sub = np.stack([node[:, 0] % nx, (node[:, 0] // nx) % ny, node[:, 0] // (nx * ny)], axis=1)
    nw = np.minimum(np.asarray(records["n_weights"]), 8)
    vid = np.asarray(records["vertex"]).reshape(n, 8)
    w = np.asarray(records["weight"]).reshape(n, 8).astype(f32)
    kn = [np.asarray(k, np.float64).astype(f32) for k in knots]
    span = max(kn[d][-1] - kn[d][0] for d in range(3))
    for i in np.nonzero(ok)[0]:
        for d in range(3):
            lo, hi = kn[d][sub[i, d]], kn[d][sub[i, d] + 1]
            X[i, d] = (x[i, d] - lo) / (hi - lo)
            X[i, 12 + 9 * B + d] = (x[i, d] - kn[d][0]) / (kn[d][-1] - kn[d][0])
        # distance to Γ over the longest side of the trellis box
        r2 = (x[i, 0] * x[i, 0] + x[i, 1] * x[i, 1]) + x[i, 2] * x[i, 2]
        X[i, 15 + 9 * B] = np.sqrt(r2) / span
        X[i, 3:3 + nw[i]] = w[i, :nw[i]]
        X[i, 11] = 1.0 if node[i, 1] >= 0 else 0.0
        for b in range(B):
            s = f32(0.0)
            for k in range(nw[i]):
                ev = vals32[vid[i, k], b]
                X[i, 12 + k * B + b] = ev * inv
                s = f32(s + w[i, k] * ev)
            base[i, b] = s
            X[i, 12 + 8 * B + b] = s * inv
    return X, base
