"""The oracle's rotation back by R against a direct numpy restatement of the
reference's rules, at q spread over every operation of the point group.

Interpolator::rotate_in_place (src/interpolator.hpp:387-428) dispatches on
(LengthUnit, RotatesLike):

- real_lattice + vector, rip_real (src/interpolator_real.tpp:19-64):
  v → R·v, M → R·M·R⁻¹;
- reciprocal_lattice + vector, rip_recip (src/interpolator_recip.tpp:19-64):
  v → Rᵀ·v, M → Rᵀ·M·(R⁻¹)ᵀ;
- real_lattice + pseudovector, rip_axial (src/interpolator_axial.tpp:19-68):
  v → det(R)·R⁻¹·v, M → R⁻¹·M·R;

scalars are never rotated and q whose R is the identity are left alone.
The unrotated value is the weighted sum of the vertex rows the locate stage
chose (src/interpolator_at.tpp:92-127; real data take no antiphase).
"""
import numpy as np
import pytest

from _cases import crystal_case
from oracle.oracle import Oracle

# (RotatesLike, LengthUnit) of the three non-Γ rules
MODES = {"real": (0, 3), "recip": (0, 4), "axial": (1, 3)}
ELEMENTS = [1, 6, 9]  # one scalar, two 3-vectors, one 3×3 matrix per branch
CRYSTALS = ["hex16", "Im-3m", "R-3m"]


def rotation_data(case, B=3, seed=0, cplx=False):
    rng = np.random.default_rng(seed)
    nv = len(case["tr"].vertices)
    d = rng.normal(size=(nv, B, sum(ELEMENTS)))
    if cplx:
        d = d + 1j * rng.normal(size=d.shape)
    return np.ascontiguousarray(d)


def restated(case, Q, data, mode):
    """Weighted vertex sum, then the reference's rule for `mode`."""
    o = Oracle(case["tables"])
    rec = o.move_locate(Q)
    assert not rec["status"].any()
    ops = np.asarray(case["tables"]["ops"], dtype=np.float64).reshape(-1, 3, 3)
    n, B = len(Q), data.shape[1]
    out = np.zeros((n, B, data.shape[2]), dtype=data.dtype)
    for x in range(8):
        has = rec["n_weights"] > x
        out[has] += rec["weight"][has, x, None, None] * data[rec["vertex"][has, x]]
    r, ri = rec["rot"][:, 0], rec["rot"][:, 1]
    R, Ri = ops[r], ops[ri]
    ident = np.all(R == np.eye(3), axis=(1, 2))
    for q in np.nonzero(~ident)[0]:
        for b in range(B):
            row = out[q, b]
            for k in range(2):
                v = row[1 + 3 * k:4 + 3 * k].copy()
                if mode == "real":
                    v = R[q] @ v
                elif mode == "recip":
                    v = R[q].T @ v
                else:
                    v = np.linalg.det(R[q]) * (Ri[q] @ v)
                row[1 + 3 * k:4 + 3 * k] = v
            M = row[7:16].reshape(3, 3).copy()
            if mode == "real":
                M = R[q] @ (M @ Ri[q])
            elif mode == "recip":
                M = R[q].T @ (M @ Ri[q].T)
            else:
                M = Ri[q] @ (M @ R[q])
            row[7:16] = M.ravel()
    return out, ident


@pytest.mark.parametrize("name", CRYSTALS)
@pytest.mark.parametrize("mode", sorted(MODES))
def test_oracle_rotation_rules(name, mode):
    c = crystal_case(name)
    data = rotation_data(c)
    rl, lu = MODES[mode]
    Q = np.random.default_rng(5).uniform(-2, 2, size=(1500, 3))
    ov, _, rc, st = Oracle(c["tables"]).interpolate_at(Q, (data, ELEMENTS, rl, lu))
    assert rc == 0 and not st.any()
    ref, ident = restated(c, Q, data, mode)
    # most q land on a non-identity operation, so the rules are exercised
    assert (~ident).mean() > 0.5
    assert np.abs(ov - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
    # the scalar element is never rotated
    assert np.abs(ov[:, :, 0] - ref[:, :, 0]).max() < 1e-13


def test_oracle_rejects_unsupported_rotation_pairs():
    """rotate_in_place throws for reciprocal-lattice pseudovectors and for
    Å data that is not Γ-like (src/interpolator.hpp:407-426)."""
    c = crystal_case("Im-3m")
    data = rotation_data(c)
    Q = np.zeros((4, 3))
    for rl, lu in ((1, 4), (0, 1), (1, 1)):
        _, _, rc, _ = Oracle(c["tables"]).interpolate_at(Q, (data, ELEMENTS, rl, lu))
        assert rc != 0, (rl, lu)
