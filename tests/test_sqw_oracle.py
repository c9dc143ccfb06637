"""The structure-factor oracle on cases with known answers."""
import numpy as np

from oracle.sqw_oracle import structure_factor


def test_single_atom_longitudinal():
    # one atom at the origin, weight 1, eigenvector along Q_c: S = |Q_c|²
    B = np.diag([1.0, 2.0, 3.0])
    Q = np.array([[0.5, 0.25, -1.0], [1.0, 0.0, 0.0]])
    Qc = Q @ B
    e = (Qc / np.linalg.norm(Qc, axis=1)[:, None])[:, None, None, :].astype(complex)
    S = structure_factor(Q, B, e, [1.0], [[0.0, 0.0, 0.0]])
    assert np.allclose(S[:, 0], np.sum(Qc ** 2, axis=1))


def test_two_atoms_interfere():
    # two equal atoms half a cell apart along x, in phase: F ∝ 1 + e^{iπ h}
    B = np.eye(3)
    pos = [[0, 0, 0], [0.5, 0, 0]]
    e = np.zeros((2, 1, 2, 3), complex)
    e[:, 0, :, 0] = 1.0
    Q = np.array([[1.0, 0, 0], [2.0, 0, 0]])
    S = structure_factor(Q, B, e, [1.0, 1.0], pos)
    assert np.allclose(S[:, 0], [0.0, 16.0], atol=1e-12)
