"""Where the reduced-precision eigenvector bars stop: the reference's own FP64
algorithm, not FP32 arithmetic.

The interpolated eigenvector of a (q, mode) aligns every vertex's row to the
pivot vertex's row by the antiphase of their Hermitian product
(utils::antiphase, src/utilities.tpp:544-580, called by interpolate_at_mix,
src/interpolator_at.tpp:38 and :112).  Where that product is small against the norms
(conditioned_modes: below 0.2), its phase is decided by rounding, so the
result is not a continuous function of the inputs.  This test runs the FP64
oracle twice, on the vertex eigenvectors as given and rounded to complex64
(a relative change of ~6e-8, what FP32 storage does): on conditioned pairs
the two agree to rounding, while on the others the FP64 algorithm itself
moves by O(1).  The GPU's FP32 and BF16 bars (test_gpu_parity) exclude the
same pairs; its FP64 path agrees with the oracle within 1e-12 on all pairs.
"""
import numpy as np
import pytest

from _cases import conditioned_modes, crystal_case, values_vectors
from oracle.oracle import Oracle


@pytest.mark.parametrize("name", ["diamond8", "hex16"])
def test_fp64_oracle_is_ill_conditioned_where_bars_exclude(name):
    c = crystal_case(name)
    Q = np.random.default_rng(21).uniform(-1, 1, size=(3000, 3))
    vals, vecs = values_vectors(c)
    o = Oracle(c["tables"])
    _, a, rc, _ = o.interpolate_at(Q, vals, vecs)
    assert rc == 0
    rounded = (vecs[0].astype(np.complex64).astype(np.complex128),) + tuple(vecs[1:])
    _, b, rc, _ = o.interpolate_at(Q, vals, rounded)
    assert rc == 0
    a = a.reshape(len(Q), a.shape[1], -1)
    b = b.reshape(a.shape)
    na, nb = np.linalg.norm(a, axis=-1), np.linalg.norm(b, axis=-1)
    loss = 1 - np.abs(np.einsum("qme,qme->qm", np.conj(a), b)) / np.maximum(na * nb, 1e-300)
    cond = conditioned_modes(c, Q)
    live = na > 1e-6
    ok, bad = cond & live, ~cond & live
    assert ok.mean() > 0.2 and bad.sum() > 1000
    # conditioned: second order in the 6e-8 input change
    assert loss[ok].max() < 1e-10
    # the rest: the FP64 algorithm's own output jumps by O(1) ...
    assert loss[bad].max() > 0.5
    # ... and every pair that moves at all is one of them
    assert not (ok & (loss > 1e-6)).any()
