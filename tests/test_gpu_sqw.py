"""The structure-factor form of the vectors gather (brx_ir_structure_factor)
against the numpy oracle applied to the oracle's interpolated eigenvectors.

Bar: S within 1e-4 of max S on the (q, mode) pairs whose antiphase is well
conditioned (elsewhere the interpolated vector itself takes its phase
pattern from rounding noise, as in the reference); values bit-identical to
ir_interpolate_at's.
"""
import numpy as np
import pytest

from _cases import boundary_q, conditioned_modes, crystal_case, values_vectors
from brille_gb300 import BZTrellisQdc
from brille_gb300._lib import BrxError
from oracle.oracle import Oracle
from oracle.sqw_oracle import structure_factor

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,storage", [("hex16", "f32"), ("P-1", "f32"), ("diamond2", "bf16")])
def test_structure_factor_matches_oracle(name, storage):
    c = crystal_case(name)
    g = BZTrellisQdc(c["bz"], trellis=c["tr"])
    na = c["model"].n_atoms
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * na, 0, 2, 1], storage=storage)
    rng = np.random.default_rng(31)
    Q = np.concatenate([rng.uniform(-2, 2, size=(3000, 3)), boundary_q(c, 1000, seed=32)])
    weights = rng.uniform(0.2, 1.0, na)
    pos = np.asarray(c["lat"].basis.positions, float)
    g.set_atoms(weights, pos)
    v, S = g.ir_structure_factor(Q)
    assert np.array_equal(v, g.ir_interpolate_at(Q, out_f32=True)[0])
    vals, vecs = values_vectors(c)
    ov, oc, rc, st = Oracle(c["tables"]).interpolate_at(Q, vals, vecs)
    assert rc == 0
    B = c["w"].shape[1]
    ref = structure_factor(Q, c["tables"]["outer_B"], oc.reshape(len(Q), B, na, 3), weights, pos)
    ok = conditioned_modes(c, Q)
    assert ok.mean() > 0.2
    tol = (1e-4 if storage == "f32" else 3e-2) * ref.max()
    assert np.abs(S - ref)[ok].max() <= tol


def test_structure_factor_needs_atoms_and_reduced_storage():
    c = crystal_case("diamond2")
    g = BZTrellisQdc(c["bz"], trellis=c["tr"])
    na = c["model"].n_atoms
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * na, 0, 2, 1], storage="f32")
    Q = np.zeros((4, 3))
    with pytest.raises(BrxError):
        g.ir_structure_factor(Q)  # no atoms yet
    with pytest.raises(ValueError):
        g.set_atoms(np.ones(na + 1), np.zeros((na, 3)))
    g.fill(c["w"], [1, 0, 0, 0, 3], c["v"], [0, 3 * na, 0, 2, 1], storage="f64")
    g.set_atoms(np.ones(na), np.asarray(c["lat"].basis.positions, float))
    with pytest.raises(BrxError):
        g.ir_structure_factor(Q)  # FP64 storage: the vectors gather keeps its reference order
