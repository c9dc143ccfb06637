"""Real-lattice, reciprocal-lattice and axial data rotated back by R on the
GPU, against the oracle (rip_real, rip_recip and rip_axial:
src/interpolator_real.tpp:19-64, src/interpolator_recip.tpp:19-64,
src/interpolator_axial.tpp:19-68), at q spread over every operation.

Each branch holds one scalar, two 3-vectors and one 3×3 matrix.  Bars:
FP64 storage within 1e-12 of the oracle (the gather sums with FMAs, the
oracle in the reference's order); complex data as well (their antiphase
comes from the handle's FP64 antiphase table); FP32 storage of vector data
(the warp-independent kernel) within 1e-5 relative.
"""
import numpy as np
import pytest

from _cases import crystal_case
from brille_gb300 import BZTrellisQdc
from brille_gb300.grid import BZTrellisQdd
from oracle.oracle import Oracle
from test_rotations import CRYSTALS, ELEMENTS, MODES, rotation_data

pytestmark = pytest.mark.gpu


def _scalars(c, B):
    return np.ones((len(c["tr"].vertices), B, 1))


@pytest.mark.parametrize("name", CRYSTALS)
@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("cplx", [False, True])
def test_rotated_data_fp64(name, mode, cplx):
    c = crystal_case(name)
    data = rotation_data(c, cplx=cplx)
    B = data.shape[1]
    rl, lu = MODES[mode]
    g = (BZTrellisQdc if cplx else BZTrellisQdd)(c["bz"], trellis=c["tr"])
    g.fill(_scalars(c, B), [1, 0, 0, 0, 3], data, ELEMENTS + [rl, lu])
    Q = np.random.default_rng(5).uniform(-2, 2, size=(3000, 3))
    _, gc = g.ir_interpolate_at(Q)
    o = Oracle(c["tables"])
    _, oc, rc, st = o.interpolate_at(Q, (_scalars(c, B), [1, 0, 0], 0, 3), (data, ELEMENTS, rl, lu))
    assert rc == 0 and not st.any()
    rec = o.move_locate(Q)
    ops = np.asarray(c["tables"]["ops"]).reshape(-1, 3, 3)
    assert (~np.all(ops[rec["rot"][:, 0]] == np.eye(3, dtype=ops.dtype), axis=(1, 2))).mean() > 0.5
    err = np.abs(gc.reshape(oc.shape) - oc).max()
    assert err < 1e-12 * max(1.0, np.abs(oc).max()), err


@pytest.mark.parametrize("mode", sorted(MODES))
def test_rotated_vectors_fp32(mode):
    c = crystal_case("hex16")
    data = rotation_data(c)[:, :, :7]  # the scalar and the two vectors
    B = data.shape[1]
    rl, lu = MODES[mode]
    g = BZTrellisQdd(c["bz"], trellis=c["tr"])
    g.fill(_scalars(c, B), [1, 0, 0, 0, 3], data, [1, 6, 0, rl, lu], storage="f32")
    Q = np.random.default_rng(6).uniform(-2, 2, size=(3000, 3))
    _, gc = g.ir_interpolate_at(Q, out_f32=True)
    _, oc, rc, _ = Oracle(c["tables"]).interpolate_at(Q, (_scalars(c, B), [1, 0, 0], 0, 3),
                                                      (np.ascontiguousarray(data), [1, 6, 0], rl, lu))
    assert rc == 0
    assert np.abs(gc.reshape(oc.shape) - oc).max() < 1e-5 * np.abs(oc).max()
