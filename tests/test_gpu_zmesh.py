"""BZMeshQ / BZNestQ on the GPU against the oracle, through the C ABI.

The mesh grids hand the trellis kernels tables with poly nodes only (every
tetrahedron listed in each knot cell its bounding box touches).  Bars as for
the trellis: locate indices and FP64 weights bit-exact, FP64 eigenvalues
bit-exact, FP64 eigenvectors within 1e-12; sort() permutations equal to the
oracle's where the optimum is unique.
"""
import numpy as np
import pytest

from brille_gb300 import workloads as W
from brille_gb300.bz import BrillouinZone
from brille_gb300.grid import BZMeshQdc, BZNestQdc
from oracle import oracle as O
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _grid(kind, name):
    lat, masses = {"diamond2": W.diamond_primitive, "hex16": W.hexagonal16}[name]()
    bz = BrillouinZone(lat)
    g = BZMeshQdc(bz, bz.ir_volume / 300) if kind == "mesh" else BZNestQdc(bz, 300)
    model = W.bvk_for(lat, masses)
    w, v = model.modes(g.trellis.vertices @ np.linalg.inv(lat.B))
    return g, lat, w, v


def _queries(g, lat, n=4000, seed=0):
    rng = np.random.default_rng(seed)
    Q = rng.uniform(-2, 2, (n, 3))
    # points on mesh tetrahedron faces and at vertices, in r.l.u.
    m = g.trellis
    t = m.mesh_tetrahedra[rng.integers(0, len(m.mesh_tetrahedra), n // 4)]
    bc = rng.dirichlet([1, 1, 1], size=len(t))
    face = np.einsum("nk,nkd->nd", bc, m.vertices[t[:, :3]])
    vert = m.vertices[rng.integers(0, len(m.vertices), n // 4)]
    return np.concatenate([Q, face @ np.linalg.inv(lat.B), vert @ np.linalg.inv(lat.B)])


@pytest.mark.parametrize("kind", ["mesh", "nest"])
@pytest.mark.parametrize("name", ["diamond2", "hex16"])
def test_mesh_locate_bit_exact(kind, name):
    g, lat, _, _ = _grid(kind, name)
    Q = _queries(g, lat)
    got = g.locate(Q, ir=True)
    ref = Oracle(g.tables).move_locate(Q, ir=True)
    for k in ("status", "q_ir", "tau", "rot", "node", "n_weights", "vertex", "weight"):
        assert np.array_equal(got[k], ref[k]), k
    assert not got["status"].any()


@pytest.mark.parametrize("kind", ["mesh", "nest"])
def test_mesh_ir_interpolate_fp64(kind):
    g, lat, w, v = _grid(kind, "diamond2")
    nv, B = w.shape
    g.fill(w, [1, 0, 0, 0, 3], v, [0, 3 * v.shape[2], 0, 2, 1])
    Q = _queries(g, lat, seed=2)
    gv, gc = g.ir_interpolate_at(Q)
    ov, oc, rc, st = Oracle(g.tables).interpolate_at(Q, (w[:, :, None], [1, 0, 0], 0, 3),
                                                     (v.reshape(nv, B, -1), [0, 3 * v.shape[2], 0], 2, 1))
    assert rc == 0 and (st == 0).all()
    assert np.array_equal(gv, ov[:, :, 0])
    assert np.abs(gc.reshape(oc.shape) - oc).max() < 1e-12


def test_mesh_sort():
    g, lat, w, v = _grid("mesh", "diamond2")
    nv, B = w.shape
    g.fill(w, [1, 0, 0, 0, 3], v, [0, 3 * v.shape[2], 0, 2, 1], sort=True)
    keys, perms = g.permutation_table()
    assert np.array_equal(keys, g.trellis.permutation_keys())
    ref, costs = O.sort_permutations((w[:, :, None], (1, 0, 0), 0, (1, 1, 1)),
                                     (v.reshape(nv, B, -1), (0, 3 * v.shape[2], 0), 0, (1, 1, 1)), keys,
                                     return_costs=True)
    diff = np.nonzero((perms != ref).any(axis=1))[0]
    for k in diff:
        i, j = keys[k] // nv, keys[k] % nv
        kk = k if i < j else np.searchsorted(keys, j * nv + i)
        c = costs[kk]
        opt = c[np.arange(B), ref[kk]].sum()
        assert c[np.arange(B), perms[kk]].sum() <= opt + 1e-9 * (1 + abs(opt))
    assert len(diff) <= max(2, len(keys) // 100)


def test_nb_vector_field_nest_known_answer_gpu():
    """src/tests/nest_test.cpp:45-150 on the GPU: Nb (Im-3m), leaf volume
    0.01 Å⁻³, f = Q stored as a reciprocal-lattice 3-vector, returned to
    2e-14 at irreducible points with and without the move."""
    from brille_gb300.crystal import Basis, Lattice, spacegroup
    from brille_gb300.grid import BZNestQdd

    a = 3.2598
    lat = Lattice(((a, a, a), (90, 90, 90)), symmetry=spacegroup("Im-3m"), basis=Basis([[0, 0, 0]], [0]))
    bz = BrillouinZone(lat)
    g = BZNestQdd(bz, 0.01, 5)
    xyz = g.trellis.vertices
    rng = np.random.default_rng(11)
    lo, hi = bz.ir_vertices_invA.min(axis=0), bz.ir_vertices_invA.max(axis=0)
    x = rng.uniform(lo, hi, (20000, 3))
    hs = bz.ir_halfspaces
    x = x[np.all(x @ hs[:, :3].T + hs[:, 3] < -1e-6, axis=1)][:200]
    Q = x @ np.linalg.inv(lat.B)
    g.fill(np.ones(len(xyz)), [1, 0, 0, 0, 3], np.ascontiguousarray(xyz[:, None, :]), [0, 3, 0, 0, 4])
    for no_move in (True, False):
        _, vecs = g.ir_interpolate_at(Q, do_not_move_points=no_move)
        assert np.abs(vecs.reshape(len(Q), 3) - x).max() < 2e-14


def test_nb_vector_field_along_face_gpu():
    """src/tests/nest_test.cpp:223-290 on the GPU: 99 points along the
    diagonal of the irreducible polyhedron's bounding box return Q to 2e-10."""
    from brille_gb300.crystal import Basis, Lattice, spacegroup
    from brille_gb300.grid import BZNestQdd

    a = 3.2598
    lat = Lattice(((a, a, a), (90, 90, 90)), symmetry=spacegroup("Im-3m"), basis=Basis([[0, 0, 0]], [0]))
    bz = BrillouinZone(lat)
    g = BZNestQdd(bz, 0.01)
    xyz = g.trellis.vertices
    rlu = bz.ir_vertices_invA @ np.linalg.inv(lat.B)
    v_min, v_del = rlu.min(axis=0), rlu.max(axis=0) - rlu.min(axis=0)
    Q = np.array([v_min + v_del * (i + 1) * (0.64 / 99) for i in range(99)])
    g.fill(np.ones(len(xyz)), [1, 0, 0, 0, 3], np.ascontiguousarray(xyz[:, None, :]), [0, 3, 0, 0, 4])
    _, vecs = g.ir_interpolate_at(Q)
    assert np.abs(vecs.reshape(len(Q), 3) - Q @ lat.B).max() < 2e-10


def test_node_containing_type():
    """node_containing_type (wrap/_trellis.hpp:88-94) on a trellis and a mesh
    grid: the type of the node the oracle's locate finds for each point."""
    from brille_gb300.grid import BZTrellisQdc, NodeType, node_type

    lat, _ = W.diamond_primitive()
    bz = BrillouinZone(lat)
    for g in (BZTrellisQdc(bz, bz.ir_volume / 300), BZMeshQdc(bz, bz.ir_volume / 300)):
        Q = Oracle(g.tables).move(np.random.default_rng(3).uniform(-1, 1, (500, 3)), ir=True)[0]
        got = g.node_containing_type(Q)
        node = Oracle(g.tables).move_locate(Q, ir=False, no_move=True)["node"][:, 0]
        want = [node_type(g.trellis.node_type[n]) if n >= 0 else NodeType.null for n in node]
        assert got == want
        assert all(t != NodeType.null for t in got)
