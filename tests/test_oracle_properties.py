"""Known-answer and property tests of the oracle, modelled on the
reference's own tests:

* src/tests/brillouinzone_test.cpp:114-169 — moveinto gives Q = q + τ with
  q inside the first zone, for random Q in [-5, 5]³;
* wrap/tests/test_4_interpolation.py:143-263 and
  src/tests/trellis_test.cpp:76-137 — linear fields are reproduced exactly;
* src/tests/trellis_test.cpp:351-372 — points near node boundaries locate.
"""
import numpy as np
import pytest

from _cases import boundary_q, crystal_case
from oracle.oracle import Oracle


@pytest.mark.parametrize("name", ["diamond2", "diamond8", "hex16", "P-1", "Im-3m", "R-3m"])
def test_moveinto_q_plus_tau(name):
    c = crystal_case(name)
    o = Oracle(c["tables"])
    Q = np.random.default_rng(0).uniform(-5, 5, size=(2000, 3))
    q, tau, rot, st = o.move(Q, ir=False)
    assert not st.any()
    assert np.allclose(q + tau, Q, atol=1e-12)
    assert c["bz"].isinside(q).all()


@pytest.mark.parametrize("name", ["diamond2", "diamond8", "hex16", "P-1", "Im-3m", "R-3m"])
def test_ir_moveinto_symmetry(name):
    """Q = Rᵀ q_ir + τ with q_ir in the irreducible wedge."""
    c = crystal_case(name)
    o = Oracle(c["tables"])
    Q = np.random.default_rng(1).uniform(-3, 3, size=(2000, 3))
    q, tau, rot, st = o.move(Q, ir=True)
    assert not st.any()
    W = c["bz"].pointgroup.W
    # q_ir = W_j^T q_1st with j = rot[:,1]; so q_1st = (W_j^T)^-1 q_ir = W_R^T q_ir for R = rot[:,0]
    q1 = np.einsum("nji,nj->ni", W[rot[:, 0]], q)
    assert np.allclose(q1 + tau, Q, atol=1e-12)
    x = q @ c["lat"].B
    assert (x @ c["bz"].wedge_normal.T >= -1e-9).all()


@pytest.mark.parametrize("name", ["diamond2", "hex16", "P-1"])
def test_linear_field_exact(name):
    """A field linear in Q is reproduced exactly (interpolate_at, no
    rotation), as in test_4_interpolation.py's known answers."""
    c = crystal_case(name)
    o = Oracle(c["tables"])
    lat, tr = c["lat"], c["tr"]
    rlu = tr.vertices @ np.linalg.inv(lat.B)
    coef = np.array([[1.0, -2.0, 0.5], [0.3, 0.2, -0.7]])
    f = (rlu @ coef.T)[:, :, None]  # two branches, one scalar
    # points inside the irreducible polyhedron: sample trellis tetrahedra and cubes
    rng = np.random.default_rng(2)
    t = tr.tet_vertices[rng.integers(0, len(tr.tet_vertices), 500)]
    x = np.einsum("nk,nkd->nd", rng.dirichlet([1, 1, 1, 1], 500), tr.vertices[t])
    Q = x @ np.linalg.inv(lat.B)
    vo, _, rc, st = o.interpolate_at(Q, (f, [1, 0, 0], 0, 3), None, ir=False, no_move=True)
    assert rc == 0
    assert np.abs(vo[:, :, 0] - Q @ coef.T).max() < 1e-12


def test_vector_field_rotation_exact():
    """trellis_test.cpp:76-137: f(Q) = Q_xyz as a reciprocal-lattice vector
    field is reproduced at Q after the wedge rotation (|err| < 2e-10)."""
    c = crystal_case("diamond8")
    o = Oracle(c["tables"])
    lat, tr = c["lat"], c["tr"]
    rlu = tr.vertices @ np.linalg.inv(lat.B)
    vec = rlu[:, None, :]  # one branch, one vector, reciprocal_lattice components
    Q = np.random.default_rng(4).uniform(-0.6, 0.6, size=(2000, 3))
    q1, tau, _, st = o.move(Q, ir=False)
    vals = (np.ones((len(rlu), 1, 1)), [1, 0, 0], 0, 3)
    vo, co, rc, st = o.interpolate_at(Q, vals, (vec.astype(np.complex128), [0, 3, 0], 0, 4))
    assert rc == 0
    assert np.abs(co[:, 0, :].real - q1).max() < 2e-10


@pytest.mark.parametrize("name", ["diamond8", "hex16"])
def test_locate_near_boundaries(name):
    c = crystal_case(name)
    o = Oracle(c["tables"])
    q = boundary_q(c, 3000)
    qq, tau, rot, st = o.move(q, ir=True)
    assert not st.any()
    node, nw, vi, w, st2 = o.locate(qq @ c["lat"].B)
    assert not st2.any()
    assert (nw >= 1).all()
    s = np.array([w[i, :nw[i]].sum() for i in range(len(nw))])
    assert np.abs(s - 1).max() < 1e-9


def test_empty_query():
    c = crystal_case("diamond2")
    o = Oracle(c["tables"])
    vals = (np.ascontiguousarray(c["w"][:, :, None]), [1, 0, 0], 0, 3)
    vo, co, rc, st = o.interpolate_at(np.zeros((0, 3)), vals)
    assert rc == 0 and vo.shape[0] == 0
