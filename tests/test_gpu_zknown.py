"""The reference's analytic known answers for interpolate_at
(wrap/tests/test_4_interpolation.py:143-230) on the GPU, filled as the
reference's tests fill them: fields linear in Q on a cubic reciprocal
lattice with |b| = 1 and no symmetry are reproduced at Q = 0, (0.1, 0, 0),
(0, 0.1, 0), (0, 0, 0.1) and at random Q of the first zone."""
import numpy as np
import pytest

from tests.test_known_answers import FIELDS, cubic_grid, points

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(FIELDS))
def test_linear_fields_gpu(name):
    f, el = FIELDS[name]
    g = cubic_grid()
    g.fill(f(g.rlu), list(el), g.rlu, (0, 3))
    Q = points()
    vals, vecs = g.interpolate_at(Q)
    assert np.abs(vals.reshape(len(Q), -1) - f(Q)).max() < 1e-12
    assert np.abs(vecs.reshape(len(Q), 3) - Q).max() < 1e-12


def test_complex_scalars_gpu():
    g = cubic_grid(cplx=True)
    h = lambda Q: (Q[:, 0] - Q[:, 1]) + 1j * (Q[:, 2] + Q[:, 1])  # noqa: E731
    c = h(g.rlu)
    g.fill(c, (1,), c, (1,))
    Q = points()
    vals, _ = g.interpolate_at(Q)
    assert np.abs(np.squeeze(vals) - h(Q)).max() < 1e-12


def test_iron_self_consistency_gpu():
    """test_4_interpolation.py:248-262 on the GPU."""
    from tests.test_known_answers import fe_dispersion, fe_grid

    g = fe_grid()
    Q = g.rlu
    g.fill(fe_dispersion(Q), (1,), Q, (0, 3))
    vals, _ = g.ir_interpolate_at(Q, False, False)
    assert np.allclose(np.squeeze(vals), fe_dispersion(Q))
