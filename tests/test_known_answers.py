"""The reference's analytic known answers for interpolate_at
(wrap/tests/test_4_interpolation.py:143-230), restated on the oracle with
this package's tables: a cubic reciprocal lattice with |b| = 1 and no
symmetry, a trellis of volume |BZ|/64, fields linear in Q — scalars, vectors
(also rotated), a matrix with Q on its diagonal and complex scalars — are
reproduced at Q = 0, (0.1, 0, 0), (0, 0.1, 0), (0, 0, 0.1) and at random Q
in the first zone."""
import numpy as np
import pytest

from brille_gb300.bz import BrillouinZone
from brille_gb300.crystal import Lattice
from brille_gb300.grid import BZTrellisQcc, BZTrellisQdd
from oracle.oracle import Oracle

TWO_PI = 2 * np.pi


def cubic_grid(cplx=False):
    lat = Lattice(((TWO_PI,) * 3, (90, 90, 90)))  # reciprocal basis: the unit vectors
    bz = BrillouinZone(lat)
    cls = BZTrellisQcc if cplx else BZTrellisQdd
    return cls(bz, bz.volume / 64)


def rot_z(Q, t):
    c, s = np.cos(t), np.sin(t)
    return np.stack([Q[:, 0] * c - Q[:, 1] * s, Q[:, 0] * s + Q[:, 1] * c, Q[:, 2]], axis=1)


def rot_x(Q, t):
    c, s = np.cos(t), np.sin(t)
    return np.stack([Q[:, 0], Q[:, 1] * c - Q[:, 2] * s, Q[:, 1] * s + Q[:, 2] * c], axis=1)


FIELDS = {
    "ones": (lambda Q: np.ones(len(Q))[:, None], (1, 0, 0)),
    "x": (lambda Q: Q[:, :1], (1, 0, 0)),
    "y": (lambda Q: Q[:, 1:2], (1, 0, 0)),
    "z": (lambda Q: Q[:, 2:], (1, 0, 0)),
    "xy": (lambda Q: Q[:, :1] + Q[:, 1:2], (1, 0, 0)),
    "xyz": (lambda Q: Q.sum(axis=1, keepdims=True), (1, 0, 0)),
    "vec": (lambda Q: Q, (0, 3, 0)),
    "vec_rotx": (lambda Q: rot_x(Q, np.pi / 3), (0, 3, 0)),
    "vec_rotz": (lambda Q: rot_z(Q, np.pi / 5), (0, 3, 0)),
    "mat_diag": (lambda Q: np.stack([np.diag(q).ravel() for q in Q]), (0, 0, 9)),
}


def points():
    Q = np.array([[0, 0, 0], [0.1, 0, 0], [0, 0.1, 0], [0, 0, 0.1]], float)
    return np.concatenate([Q, np.random.default_rng(0).uniform(-0.5, 0.5, (200, 3))])


@pytest.mark.parametrize("name", sorted(FIELDS))
def test_linear_fields_interpolate_at(name):
    f, el = FIELDS[name]
    g = cubic_grid()
    data = f(g.rlu)[:, None, :]  # one branch
    Q = points()
    vo, _, rc, st = Oracle(g.tables).interpolate_at(Q, (np.ascontiguousarray(data), list(el), 0, 4), None, ir=False)
    assert rc == 0 and (st == 0).all()
    assert np.abs(vo[:, 0, :] - f(Q)).max() < 1e-12


def test_complex_scalars_interpolate_at():
    g = cubic_grid(cplx=True)
    h = lambda Q: (Q[:, 0] - Q[:, 1]) + 1j * (Q[:, 2] + Q[:, 1])  # noqa: E731
    data = h(g.rlu)[:, None, None]
    Q = points()
    vo, co, rc, st = Oracle(g.tables).interpolate_at(Q, (np.ascontiguousarray(data), [1, 0, 0], 0, 4),
                                                     (np.ascontiguousarray(data), [1, 0, 0], 0, 4), ir=False)
    assert rc == 0 and (st == 0).all()
    # complex values keep their phase; complex vectors are phase-aligned to the pivot vertex
    assert np.abs(vo[:, 0, 0] - h(Q)).max() < 1e-12


def fe_dispersion(Q, J=-16.0, d=0.01):
    """Nearest-neighbour spin waves of bcc iron (wrap/tests/test_4_interpolation.py)."""
    return d + 8 * J * (1 - np.cos(np.pi * Q[:, 0]) * np.cos(np.pi * Q[:, 1]) * np.cos(np.pi * Q[:, 2]))


def fe_grid():
    from brille_gb300.crystal import spacegroup
    from brille_gb300.grid import BZTrellisQdc

    lat = Lattice(((2.87,) * 3, (90, 90, 90)), symmetry=spacegroup("Im-3m"))
    return BZTrellisQdc(BrillouinZone(lat), 0.125)


def test_iron_self_consistency():
    """test_4_interpolation.py:248-262: bcc Fe spin waves stored at the
    trellis vertices are returned at the vertices by ir_interpolate_at."""
    g = fe_grid()
    Q = g.rlu
    w = fe_dispersion(Q)
    vo, _, rc, st = Oracle(g.tables).interpolate_at(Q, (w[:, None, None].copy(), [1, 0, 0], 0, 3),
                                                    (np.ascontiguousarray(Q[:, None, :]).astype(complex), [0, 3, 0], 0, 3))
    assert rc == 0 and (st == 0).all()
    assert np.allclose(vo[:, 0, 0], w)
