"""BZMeshQ / BZNestQ tables on the CPU: the mesh, its bucketing into trellis
form, and the oracle's answers on it.

The mesh grids reuse the trellis query path: their tetrahedra are listed in
poly nodes of a knot grid (brille_gb300.mesh.MeshTrellis).  These tests pin
the tables: the mesh covers the irreducible polyhedron exactly with
positively oriented tetrahedra within the volume limit; every point of the
polyhedron is located in a tetrahedron that contains it; a linear field is
reproduced exactly (the reference's known-answer test for its grids,
wrap/tests/test_4_interpolation.py:143-263); the permutation keys are the
mesh's tetrahedron edges (TetTriLayer::collect_keys,
src/triangulation_layers.hpp:242-258).
"""
import numpy as np
import pytest

from brille_gb300 import workloads as W
from brille_gb300.bz import BrillouinZone
from brille_gb300.mesh import MeshTrellis, delaunay_mesh
from brille_gb300.tables import geometry_tables
from oracle.oracle import Oracle


def _bz(name):
    lat, _ = {"diamond2": W.diamond_primitive, "hex16": W.hexagonal16}[name]()
    return BrillouinZone(lat)


@pytest.mark.parametrize("name", ["diamond2", "hex16"])
def test_mesh_covers_polyhedron(name):
    bz = _bz(name)
    vmax = bz.ir_volume / 400
    m = MeshTrellis(bz.ir_vertices_invA, vmax)
    T, v = m.mesh_tetrahedra, m.vertices
    q = v[T]
    o = np.einsum("ij,ij->i", q[:, 0] - q[:, 3], np.cross(q[:, 1] - q[:, 3], q[:, 2] - q[:, 3]))
    assert (o > 0).all()
    assert np.isclose(np.sum(o) / 6, bz.ir_volume, rtol=1e-9)
    assert (o / 6 <= vmax * (1 + 1e-12)).all()
    # every listed entry is one mesh tetrahedron with its own sphere and volume
    assert np.array_equal(m.tet_vertices, T[m.tet_mesh_index])
    assert np.allclose(m.tet_volume, o[m.tet_mesh_index] / 6)
    assert m.node_type.size == np.prod(m.shape)


def test_max_points_stops_refinement():
    bz = _bz("diamond2")
    v, t, vol = delaunay_mesh(bz.ir_vertices_invA, bz.ir_volume / 5000, max_points=200)
    assert len(v) <= 200 + len(t)  # the last round may add up to one point per tetrahedron it split
    v2, _, _ = delaunay_mesh(bz.ir_vertices_invA, -1)
    assert len(v2) == len(np.unique(bz.ir_vertices_invA, axis=0))


@pytest.mark.parametrize("name", ["diamond2", "hex16"])
def test_oracle_locates_every_point(name):
    bz = _bz(name)
    m = MeshTrellis(bz.ir_vertices_invA, bz.ir_volume / 300)
    t = geometry_tables(bz, m)
    rng = np.random.default_rng(3)
    Q = rng.uniform(-1.5, 1.5, (3000, 3))
    rec = Oracle(t).move_locate(Q, ir=True)
    assert (rec["status"] == 0).all()
    tet = rec["node"][:, 1]
    assert (tet >= 0).all()
    x = rec["q_ir"] @ bz.lattice.B
    # barycentric coordinates of x in the located mesh tetrahedron
    p = m.vertices[m.tet_vertices[tet]]
    M = np.stack([p[:, 0] - p[:, 3], p[:, 1] - p[:, 3], p[:, 2] - p[:, 3]], axis=-1)
    lam = np.linalg.solve(M, (x - p[:, 3])[..., None])[..., 0]
    lam = np.concatenate([lam, 1 - lam.sum(axis=1, keepdims=True)], axis=1)
    assert lam.min() > -1e-9
    assert np.allclose(rec["weight"].sum(axis=1), 1.0)


@pytest.mark.parametrize("cls", ["mesh", "nest"])
def test_linear_field_exact(cls):
    """Values f = a·x + c at the vertices interpolate to f(q_ir) exactly (up
    to rounding) anywhere in the polyhedron."""
    from brille_gb300.grid import BZMeshQdd, BZNestQdd

    bz = _bz("diamond2")
    grid = BZMeshQdd(bz, bz.ir_volume / 200) if cls == "mesh" else BZNestQdd(bz, 200)
    t = grid.tables
    a, c = np.array([0.3, -1.2, 2.5]), 0.7
    f = grid.trellis.vertices @ a + c
    rng = np.random.default_rng(5)
    Q = rng.uniform(-1, 1, (2000, 3))
    vo, _, rc, st = Oracle(t).interpolate_at(Q, (f[:, None, None].copy(), [1, 0, 0], 0, 3), None, ir=True)
    assert rc == 0 and (st == 0).all()
    q_ir = Oracle(t).move(Q, ir=True)[0]
    want = (q_ir @ bz.lattice.B) @ a + c
    assert np.abs(vo[:, 0, 0] - want).max() < 1e-12 * (1 + np.abs(want).max())


def test_nest_density_and_volume():
    from brille_gb300.grid import BZNestQdc

    bz = _bz("diamond2")
    by_density = BZNestQdc(bz, 100)
    by_volume = BZNestQdc(bz, bz.ir_volume / 100)
    assert np.array_equal(by_density.invA, by_volume.invA)
    assert np.array_equal(by_density.tetrahedra, by_volume.tetrahedra)
    assert by_density.all_rlu.shape == by_density.rlu.shape
    assert by_density.bytes_per_point > 0
    with pytest.raises(ValueError):
        BZNestQdc(bz, 0)


def test_mesh_permutation_keys():
    bz = _bz("diamond2")
    m = MeshTrellis(bz.ir_vertices_invA, bz.ir_volume / 100)
    n = len(m.vertices)
    want = set()
    for tet in m.mesh_tetrahedra:
        for a in tet:
            for b in tet:
                if a != b:
                    want.add(int(a) * n + int(b))
    assert np.array_equal(m.permutation_keys(), np.array(sorted(want), np.int64))


@pytest.mark.parametrize("cls", ["nest", "mesh"])
def test_nb_vector_field_nest_known_answer(cls):
    """src/tests/nest_test.cpp:45-150: Nb (Im-3m, a = 3.2598 Å), leaf volume
    0.01 Å⁻³, the vector field f = Q (Cartesian) stored as one branch of a
    3-vector; at random points of the irreducible polyhedron interpolation
    returns Q to 2e-14, with and without the move (the points are already
    irreducible, so R is the identity and τ = 0)."""
    from brille_gb300.crystal import Basis, Lattice, spacegroup
    from brille_gb300.grid import BZMeshQdd, BZNestQdd

    a = 3.2598
    lat = Lattice(((a, a, a), (90, 90, 90)), symmetry=spacegroup("Im-3m"), basis=Basis([[0, 0, 0]], [0]))
    bz = BrillouinZone(lat)
    g = BZNestQdd(bz, 0.01, 5) if cls == "nest" else BZMeshQdd(bz, 0.01)
    xyz = g.trellis.vertices
    o = Oracle(g.tables)
    rng = np.random.default_rng(11)
    # random points of the irreducible polyhedron (rejection from its box),
    # kept off its surface so that rounding cannot move them out
    lo, hi = bz.ir_vertices_invA.min(axis=0), bz.ir_vertices_invA.max(axis=0)
    x = rng.uniform(lo, hi, (20000, 3))
    hs = bz.ir_halfspaces
    inside = np.all(x @ hs[:, :3].T + hs[:, 3] < -1e-6, axis=1)
    x = x[inside][:200]
    Q = x @ np.linalg.inv(lat.B)
    vals = (np.ones((len(xyz), 1, 1)), [1, 0, 0], 0, 3)
    vecs = (np.ascontiguousarray(xyz[:, None, :]), [0, 3, 0], 0, 4)
    for no_move in (True, False):
        _, co, rc, st = o.interpolate_at(Q, vals, vecs, ir=True, no_move=no_move)
        assert rc == 0 and (st == 0).all()
        assert np.abs(co[:, 0, :] - x).max() < 2e-14


@pytest.mark.parametrize("cls", ["nest", "mesh"])
def test_nb_vector_field_along_face(cls):
    """src/tests/nest_test.cpp:223-290: the same Nb field at 99 points along
    the diagonal of the irreducible polyhedron's bounding box in r.l.u. (a
    line on one of its faces), moved and rotated as needed, returns Q to
    2e-10."""
    from brille_gb300.crystal import Basis, Lattice, spacegroup
    from brille_gb300.grid import BZMeshQdd, BZNestQdd

    a = 3.2598
    lat = Lattice(((a, a, a), (90, 90, 90)), symmetry=spacegroup("Im-3m"), basis=Basis([[0, 0, 0]], [0]))
    bz = BrillouinZone(lat)
    g = BZNestQdd(bz, 0.01) if cls == "nest" else BZMeshQdd(bz, 0.01)
    xyz = g.trellis.vertices
    rlu = bz.ir_vertices_invA @ np.linalg.inv(lat.B)
    v_min, v_del = rlu.min(axis=0), rlu.max(axis=0) - rlu.min(axis=0)
    step = 0.64 / 99
    Q = np.array([v_min + v_del * (i + 1) * step for i in range(99)])
    vals = (np.ones((len(xyz), 1, 1)), [1, 0, 0], 0, 3)
    vecs = (np.ascontiguousarray(xyz[:, None, :]), [0, 3, 0], 0, 4)
    _, co, rc, st = Oracle(g.tables).interpolate_at(Q, vals, vecs, ir=True)
    assert rc == 0 and (st == 0).all()
    assert np.abs(co[:, 0, :] - Q @ lat.B).max() < 2e-10


def test_trellis_accessors():
    """The reference's BZTrellisQ accessors (wrap/_trellis.hpp:36-98):
    node_volume_fraction (the maximum node volume in Å⁻³), inner/outer
    vertices, node types."""
    from brille_gb300.grid import BZTrellisQdc, node_type

    bz = _bz("diamond2")
    g = BZTrellisQdc(bz, node_volume_fraction=bz.ir_volume / 100)
    t = g.trellis
    assert len(g.all_node_types()) == t.node_type.size
    nx, ny, _ = t.shape
    for lin in (0, t.node_type.size // 2, t.node_type.size - 1):
        sub = (lin % nx, (lin // nx) % ny, lin // (nx * ny))
        assert g.node_at_type(sub) == node_type(t.node_type[lin])
    with pytest.raises(IndexError):
        g.node_at_type(t.shape)
    assert set(map(tuple, g.inner_invA)) == set(map(tuple, t.vertices[np.unique(t.cube_vertices)]))
    assert np.allclose(g.outer_rlu @ bz.lattice.B, g.outer_invA)
    with pytest.raises(ValueError):
        BZTrellisQdc(bz, 0.0)


def test_approx_config():
    """ApproxConfig and the global tolerances (wrap/_approx.cpp:7-40) reach
    the grid's device tables."""
    import brille_gb300 as b
    from brille_gb300.grid import BZTrellisQdd

    c = b.ApproxConfig()
    assert (c.digits, c.real_space_tolerance, c.reciprocal_space_tolerance) == (1000, 1e-10, 1e-10)
    bz = _bz("diamond2")
    g = BZTrellisQdd(bz, bz.ir_volume / 50, False, b.ApproxConfig(100, 1e-9, 1e-8))
    assert g.tables["float_tolerance"] == 1e-8 and g.tables["digit"] == 100
    assert b.reciprocal_space_tolerance() == 1e-12
    b.reciprocal_space_tolerance(3e-12)
    try:
        g2 = BZTrellisQdd(bz, bz.ir_volume / 50)
        assert g2.tables["float_tolerance"] == 3e-12 and g2.tables["digit"] == 1000
    finally:
        b.reciprocal_space_tolerance(1e-12)
    with pytest.raises(ValueError):
        b.ApproxConfig(0)


def test_brillouin_zone_arguments():
    """BrillouinZone takes the reference's arguments (wrap/_bz.cpp:156-203)."""
    lat, _ = W.hexagonal16()
    a = BrillouinZone(lat)
    b = BrillouinZone(lat, True, 1, False, True, True)
    assert np.array_equal(a.ir_vertices_invA, b.ir_vertices_invA)
    c = BrillouinZone(lat, time_reversal_symmetry=True)
    d = BrillouinZone(lat, time_reversal=True)
    assert c.time_reversal and d.time_reversal
    assert c.pointgroup.size == d.pointgroup.size
    with pytest.raises(ValueError):
        BrillouinZone(lat, use_primitive=False)


def test_brillouin_zone_approx_config_overload():
    import brille_gb300 as b

    lat, _ = W.diamond_primitive()
    cfg = b.ApproxConfig(1000, 1e-12, 1e-12)
    z = BrillouinZone(lat, cfg)
    assert z.approx_config is cfg and not z.time_reversal and z.wedge_search
    z2 = BrillouinZone(lat, cfg, True, 1, True)
    assert z2.time_reversal
    with pytest.raises(TypeError):
        BrillouinZone(lat, nonsense=1)


@pytest.mark.parametrize("kind", ["mesh", "nest"])
@pytest.mark.parametrize("name", ["diamond2", "hex16"])
def test_mesh_boundary_points_locate(kind, name):
    """Points at the irreducible polyhedron's vertices, on its faces and
    within 1e-9 r.l.u. of them locate without error (the trellis bar of
    src/tests/trellis_test.cpp:351-372, on the mesh tables)."""
    from brille_gb300.grid import BZMeshQdd, BZNestQdd

    bz = _bz(name)
    g = BZMeshQdd(bz, bz.ir_volume / 300) if kind == "mesh" else BZNestQdd(bz, 300)
    rng = np.random.default_rng(8)
    v = bz.ir_vertices_invA
    pts = [v]
    for f in bz.ir_faces:
        ring = v[list(f)]
        w = rng.dirichlet(np.ones(len(ring)), 20)
        pts.append(w @ ring)
    x = np.concatenate(pts)
    x = np.concatenate([x, x + rng.uniform(-1e-9, 1e-9, x.shape)])
    Q = x @ np.linalg.inv(bz.lattice.B)
    rec = Oracle(g.tables).move_locate(Q, ir=True)
    assert (rec["status"] == 0).all()
    assert np.allclose(rec["weight"].sum(axis=1), 1.0)


def test_fill_arguments():
    """fill() takes the reference's positional forms and keyword names
    (wrap/_common_grid.hpp:26-47, 127-147)."""
    from brille_gb300.grid import _fill_arguments as fa

    a = fa(("v", "ve", "c", "ce"), {})
    assert (a["vectors_data"], a["vectors_elements"], a["sort"]) == ("c", "ce", False)
    a = fa(("v", "ve", "c", "ce", True), {})
    assert a["sort"] is True
    a = fa(("v", "ve", "vw", "c", "ce", "cw", True), {})
    assert (a["values_weights"], a["vectors_weights"], a["sort"]) == ("vw", "cw", True)
    a = fa((), dict(values_data="v", values_elements="ve", vectors_data="c", vectors_elements="ce", sort=1))
    assert a["vectors_data"] == "c" and a["sort"] is True
    a = fa(("v", "ve"), {})
    assert a["vectors_data"] is None
    a = fa(("v", "ve", "c", "ce"), dict(sort=True, values_weights=(2, 1, 1)))
    assert a["sort"] and a["values_weights"] == (2, 1, 1)
    for args, kw in ((("v", "ve", "c"), {}), (("v", "ve", "c", "ce", True), dict(sort=True)),
                     (("v",), {}), (("v", "ve"), dict(bogus=1)), (("v", "ve"), dict(vectors_data="c"))):
        with pytest.raises(TypeError):
            fa(args, kw)


def test_lattice_reference_forms():
    """The reference's Python Lattice forms (brille/lattice.py:10-120)."""
    from brille_gb300.crystal import Basis, Lattice, spacegroup

    a = Lattice(((2.87,) * 3, (90, 90, 90)), symmetry=spacegroup("Im-3m"))
    b = Lattice(((2.87,) * 3, np.pi / 2 * np.ones(3)), spacegroup="Im-3m")   # radians, by keyword
    c = Lattice(((2.87,) * 3, (90, 90, 90)), "Im-3m")                       # by position
    for x in (b, c):
        assert np.allclose(x.A, a.A) and x.pointgroup.size == a.pointgroup.size
    r = Lattice(((1, 1, 1), (90, 90, 90)), real_space=False)
    assert np.allclose(r.B, np.eye(3))
    h = Lattice(((3.2, 3.2, 5.2), (90, 90, 120)), spacegroup="P 6_3/m m c")
    assert h.pointgroup.size == 24
    s = Lattice(np.diag([3.0, 4.0, 5.0]), symmetry=(np.eye(3, dtype=int)[None], np.zeros((1, 3))),
                basis=([[0, 0, 0]], [0]))
    assert isinstance(s.basis, Basis) and s.pointgroup.size == 1
    with pytest.raises(ValueError):
        Lattice(((3,) * 3, (90,) * 3), spacegroup="Ia-3d")


def test_brillouin_zone_accessors():
    """Reference units: vertices in r.l.u., *_invA in Å⁻¹ (wrap/_bz.cpp:237-372)."""
    bz = _bz("hex16")
    B = bz.lattice.B
    assert np.allclose(bz.ir_vertices @ B, bz.ir_vertices_invA)
    assert np.allclose(bz.vertices @ B, bz.vertices_invA)
    assert np.allclose(bz.points @ B, bz.points_invA)
    assert np.allclose(np.linalg.norm(bz.normals_invA, axis=1), 1)
    assert np.allclose(bz.wedge_normals @ B, bz.wedge_normals_invA)
    # the face centres are on the faces: n·p = |τ|/2
    assert np.allclose(np.einsum("ij,ij->i", bz.normals_invA, bz.points_invA), bz.face_tau_len / 2)


def test_create_bz_and_grid():
    """create_bz / create_grid (brille/utils.py:63-356) argument forms."""
    from brille_gb300 import grid as G
    from brille_gb300.utils import create_bz, create_grid

    a = create_bz(2.87, 2.87, 2.87, 90, 90, 90, "Im-3m")
    b = create_bz([2.87] * 3, [90] * 3, "Im-3m")
    c = create_bz(np.eye(3) * 2.87, "Im-3m")
    d = create_bz(lens=[2.87] * 3, angs=[np.pi / 2] * 3, spacegroup="Im-3m")
    for z in (b, c, d):
        assert np.allclose(z.ir_vertices_invA, a.ir_vertices_invA)
    r = create_bz([1, 1, 1], [90, 90, 90], "P1", is_reciprocal=True)
    assert np.allclose(r.lattice.B, np.eye(3))
    with pytest.raises(ValueError):
        create_bz([2.87] * 3, [90] * 3)
    g = create_grid(a, node_volume_fraction=a.ir_volume / 50)
    assert type(g) is G.BZTrellisQdd
    assert type(create_grid(a, complex_vectors=True, mesh=True, max_size=a.ir_volume / 20)) is G.BZMeshQdc
    assert type(create_grid(a, True, True, nest=True, number_density=20)) is G.BZNestQcc
    for kw in (dict(mesh=True, nest=True), dict(nest=True), dict(max_size=1.0), dict(nest=True, num_levels=2)):
        with pytest.raises(ValueError):
            create_grid(a, **kw)
