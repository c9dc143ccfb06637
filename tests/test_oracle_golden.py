"""The oracle against the reference's only golden data for this path:
wrap/tests/test_5_gamma.py with its NaCl fixture (copied into
tests/golden/nacl_gamma.npz by tests/golden/make_golden.py)."""
import numpy as np
import pytest

from _cases import nacl
from oracle.oracle import Oracle


def _phase_fixed(ref, got):
    ph = np.exp(-1j * np.angle(np.einsum("qmij,qmij->qm", np.conj(ref), got)))
    return np.einsum("ab,abij->abij", ph, got)


def test_nacl_real_lattice_vectors():
    """test_5_gamma.py:test_nacl — eigenvectors in lattice components."""
    d, lat, bz, tr, t = nacl()
    o = Oracle(t)
    q, tau, rot, st = o.move(d["q_nu"])
    assert not st.any()
    assert np.allclose(q, d["grid_rlu"][4])
    vals = (d["grid_values"], [1, 0, 0], 0, 3)
    vecs = (d["grid_vectors"].reshape(29, 24, 24), [0, 24, 0], 2, 3)
    vo, co, rc, st = o.interpolate_at(d["q_nu"], vals, vecs)
    assert rc == 0
    vo = vo[:, :, 0]
    assert not np.any(np.isclose(np.diff(vo, axis=1), 0.0))
    assert np.allclose(np.diff(vo, axis=0), 0.0)
    assert np.allclose(vo, d["euphonic_values"])
    br = np.einsum("ba,ijkb->ijka", d["basis_vectors"], co.reshape(48, 24, 8, 3))
    assert np.allclose(_phase_fixed(d["euphonic_vectors"], br), d["euphonic_vectors"])
    assert np.abs(_phase_fixed(d["euphonic_vectors"], br) - d["euphonic_vectors"]).max() < 1e-12


def test_nacl_cartesian_vectors():
    """test_5_gamma.py:test_cartesian_eigenvector_interpolation."""
    d, lat, bz, tr, t = nacl()
    o = Oracle(t)
    gv = np.einsum("ba,ijkb->ijka", d["basis_vectors"], d["grid_vectors"]).reshape(29, 24, 24)
    vals = (d["grid_values"], [1, 0, 0], 0, 3)
    vo, co, rc, st = o.interpolate_at(d["q_nu"], vals, (gv, [0, 24, 0], 2, 1))
    assert rc == 0
    br = co.reshape(48, 24, 8, 3)
    assert np.abs(_phase_fixed(d["euphonic_vectors"], br) - d["euphonic_vectors"]).max() < 1e-12


@pytest.mark.parametrize("combo", [(0, 1), (1, 0), (2, 2), (2, 4)])
def test_nacl_unsupported_combinations(combo):
    """test_5_gamma.py:test_unsupported_rotateslike_lengthunit_combinations_error."""
    d, lat, bz, tr, t = nacl()
    o = Oracle(t)
    vals = (d["grid_values"], [1, 0, 0], 0, 3)
    vecs = (d["grid_vectors"].reshape(29, 24, 24), [0, 24, 0], *combo)
    vo, co, rc, st = o.interpolate_at(d["q_nu"], vals, vecs)
    assert rc == 8  # BRX_ERR_UNSUPPORTED
