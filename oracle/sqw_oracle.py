"""Structure factor of interpolated modes — test infrastructure (the oracle
side of brx_ir_structure_factor; only tests/ use it).

The reference computes no structure factor; its downstream consumers
(brilleu, Euphonic) form the coherent one-phonon structure factor from the
eigenvectors brille interpolates.  This restates the textbook expression
per q and mode j,

    S_j(Q) = | Σ_k c_k exp(2πi Q·x_k) (Q_c · e_jk) |²,   Q_c = Q · B,

with Q in r.l.u., B the rows of the reciprocal basis (Å⁻¹), x_k fractional
atom positions, c_k = b_k / sqrt(m_k) and e_jk the Cartesian eigenvector of
atom k of mode j, in numpy FP64.
"""
import numpy as np


def structure_factor(Q, B, vectors, weights, positions):
    """Q: n × 3; B: 3 × 3 (rows b1, b2, b3); vectors: n × modes × atoms × 3
    complex; weights: atoms; positions: atoms × 3.  Returns n × modes."""
    Q = np.asarray(Q, float)
    Qc = Q @ np.asarray(B, float)                                   # n × 3
    ph = np.exp(2j * np.pi * (Q @ np.asarray(positions, float).T))  # n × atoms
    d = np.einsum("nc,nmkc->nmk", Qc, vectors)                      # Q_c · e_jk
    F = np.einsum("k,nk,nmk->nm", np.asarray(weights, float), ph, d)
    return np.abs(F) ** 2
