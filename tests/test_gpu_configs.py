"""Oracle parity at the benchmark's own configurations, through the C ABI.

- The small plain-method configuration: FCC Fd-3m, a = 4.96 Å, trellis at
  |BZ|/5000 (the 8-atom conventional diamond cell, 24 modes, and the 2-atom
  primitive cell, 6 modes), 1e5 q uniform in [-1, 1]³ r.l.u., plus 2e4 q
  within 1e-6 r.l.u. of trellis knots, tetrahedron faces and zone faces.
- The large plain-method configuration: P6₃/mmc, 16 atoms (48 modes), the
  199 272-vertex trellis of the benchmark, on a 2e4-q sample of q uniform
  in [-2, 2]³.

Bars as the other FP64 parity tests: every locate index and FP64 weight
bit-exact, FP64 eigenvalues bit-exact, FP64 eigenvectors within 1e-12.
"""
import numpy as np
import pytest

from _cases import boundary_q, crystal_case, values_vectors
from brille_gb300 import BZTrellisQdc
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

LOCATE_KEYS = ("status", "q_ir", "tau", "rot", "node", "n_weights", "vertex", "weight")


def _check(case, Q, atoms):
    g = BZTrellisQdc(case["bz"], trellis=case["tr"])
    o = Oracle(case["tables"])
    got = g.locate(Q)
    ref = o.move_locate(Q)
    for k in LOCATE_KEYS:
        assert np.array_equal(got[k], ref[k]), k
    assert not ref["status"].any()
    g.fill(case["w"], [1, 0, 0, 0, 3], case["v"], [0, 3 * atoms, 0, 2, 1])
    gv, gc = g.ir_interpolate_at(Q)
    ov, oc, rc, _ = o.interpolate_at(Q, *values_vectors(case))
    assert rc == 0
    assert np.array_equal(gv, ov[:, :, 0])
    err = np.abs(gc.reshape(oc.shape) - oc).max()
    assert err < 1e-12, err


@pytest.mark.parametrize("name", ["diamond8", "diamond2"])
def test_fcc_bz5000_1e5q(name):
    c = crystal_case(name, 1 / 5000)
    if name == "diamond8":
        assert len(c["tr"].vertices) == 333  # the reference's vertex count at |BZ|/5000
    Q = np.concatenate([np.random.default_rng(0).uniform(-1, 1, size=(100_000, 3)),
                        boundary_q(c, 20_000, seed=1)])
    _check(c, Q, c["v"].shape[2])


def test_hex16_199k_vertices_sample():
    c = crystal_case("hex16", 2.4e-7)
    assert len(c["tr"].vertices) == 199_272
    Q = np.random.default_rng(2).uniform(-2, 2, size=(20_000, 3))
    _check(c, Q, 16)
