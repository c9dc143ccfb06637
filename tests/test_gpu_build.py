"""Trellis construction on the GPU (brx_trellis_cells_build) against the host
builder, and queries on the GPU-built tables against the oracle.

Both builders must give the same knots, node types, cube nodes and vertex
set (the points are the same: knot points of cube corners and the corners of
cell ∩ polyhedron); the cut cells' tetrahedra differ (a fan over the facets
instead of Delaunay) but must tile the same polytopes: per poly node the
tetrahedra's volumes sum to the host's within 1e-9 of the cell volume, and
every tetrahedron is positively oriented.  A query through GPU-built tables
must match the oracle on those tables as on any (locate indices and FP64
weights bit-exact, FP64 eigenvalues bit-exact, eigenvectors within 1e-12).
"""
import numpy as np
import pytest
from scipy.spatial import cKDTree

from _cases import CRYSTALS, values_vectors
from brille_gb300 import BZTrellisQdc
from brille_gb300 import workloads as W
from brille_gb300.bz import BrillouinZone
from brille_gb300.tables import geometry_tables
from brille_gb300.trellis import NODE_CUBE, NODE_POLY, TrellisBuild, orient_many
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

CASES = [("diamond2", 1 / 2000), ("diamond8", 1 / 2000), ("diamond8", 1 / 5000), ("hex16", 1 / 2000), ("P-1", 1 / 2000),
         ("R-3m", 1 / 2000), ("Im-3m", 1 / 2000), ("hex16", 1 / 20000)]


def _crystal(name):
    return CRYSTALS[name]() if name in CRYSTALS else W.random_crystal(name, 2, seed=3)


def _both(name, frac, always_triangulate=False):
    lat, _ = _crystal(name)
    bz = BrillouinZone(lat)
    args = (bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * frac, always_triangulate)
    return bz, TrellisBuild(*args), TrellisBuild(*args, backend="gpu")


def _node_volumes(t):
    vol = np.zeros(t.node_type.size)
    poly = np.nonzero(t.node_type == NODE_POLY)[0]
    for n in poly:
        k = t.node_index[n]
        vol[n] = t.tet_volume[t.poly_tet_offset[k]:t.poly_tet_offset[k + 1]].sum()
    return vol


@pytest.mark.parametrize("name,frac", CASES)
def test_gpu_build_matches_host(name, frac):
    bz, h, g = _both(name, frac)
    for d in range(3):
        assert np.array_equal(h.knots[d], g.knots[d])
    assert h.shape == g.shape
    # cube nodes: the same cells with the same corner coordinates
    assert np.array_equal(h.node_type == NODE_CUBE, g.node_type == NODE_CUBE)
    assert np.array_equal(h.vertices[h.cube_vertices], g.vertices[g.cube_vertices])
    # the same vertex set
    scale = float(np.max(np.abs(bz.ir_vertices_invA)))
    assert len(h.vertices) == len(g.vertices)
    dist, _ = cKDTree(h.vertices).query(g.vertices)
    assert dist.max() <= 1e-9 * scale
    # the same cut polytopes: poly nodes and their volumes
    kx, ky, kz = h.knots
    cell = (kx[1] - kx[0]) * (ky[1] - ky[0]) * (kz[1] - kz[0])
    vh, vg = _node_volumes(h), _node_volumes(g)
    assert np.abs(vh - vg).max() <= 1e-9 * cell
    both = (h.node_type == NODE_POLY) & (g.node_type == NODE_POLY)
    only = (h.node_type == NODE_POLY) ^ (g.node_type == NODE_POLY)
    assert both.sum() > 0
    assert np.all(np.maximum(vh, vg)[only] <= 1e-9 * cell)
    # tetrahedra positively oriented, indices in range
    assert g.tet_vertices.min() >= 0 and g.tet_vertices.max() < len(g.vertices)
    assert np.all(orient_many(g.vertices[g.tet_vertices]) > 0)
    assert np.all(g.tet_volume > 0)


@pytest.mark.parametrize("name", ["diamond8", "hex16", "R-3m"])
def test_query_on_gpu_built_trellis_matches_oracle(name):
    lat, masses = _crystal(name)
    bz = BrillouinZone(lat)
    tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume / 2000, backend="gpu")
    model = W.bvk_for(lat, masses)
    w, v = model.modes(tr.vertices @ np.linalg.inv(lat.B))
    case = dict(tables=geometry_tables(bz, tr), w=w, v=v)
    Q = np.random.default_rng(8).uniform(-2, 2, size=(4000, 3))
    g = BZTrellisQdc(bz, trellis=tr)
    o = Oracle(case["tables"])
    got, ref = g.locate(Q), o.move_locate(Q)
    for k in ("status", "q_ir", "tau", "rot", "node", "n_weights", "vertex", "weight"):
        assert np.array_equal(got[k], ref[k]), k
    assert not ref["status"].any()
    g.fill(w, [1, 0, 0, 0, 3], v, [0, 3 * v.shape[2], 0, 2, 1])
    gv, gc = g.ir_interpolate_at(Q)
    ov, oc, rc, _ = o.interpolate_at(Q, *values_vectors(case))
    assert rc == 0
    assert np.array_equal(gv, ov[:, :, 0])
    assert np.abs(gc.reshape(oc.shape) - oc).max() < 1e-12


@pytest.mark.parametrize("name", ["diamond2", "hex16"])
def test_gpu_build_always_triangulate(name):
    """always_triangulate: every non-null cell is a poly node on both
    builders, with the same per-node volumes and vertex set."""
    bz, h, g = _both(name, 1 / 2000, always_triangulate=True)
    assert not (h.node_type == NODE_CUBE).any() and not (g.node_type == NODE_CUBE).any()
    assert np.array_equal(h.node_type == NODE_POLY, g.node_type == NODE_POLY)
    kx, ky, kz = h.knots
    cell = (kx[1] - kx[0]) * (ky[1] - ky[0]) * (kz[1] - kz[0])
    assert np.abs(_node_volumes(h) - _node_volumes(g)).max() <= 1e-9 * cell
    scale = float(np.max(np.abs(bz.ir_vertices_invA)))
    dist, _ = cKDTree(h.vertices).query(g.vertices)
    assert len(h.vertices) == len(g.vertices) and dist.max() <= 1e-9 * scale
    assert np.all(orient_many(g.vertices[g.tet_vertices]) > 0)


def test_grid_constructor_builds_on_the_gpu():
    """BZTrellisQdc(..., trellis_backend="gpu") builds its trellis on the
    device, like TrellisBuild(backend="gpu"), and answers queries."""
    lat, masses = _crystal("diamond8")
    bz = BrillouinZone(lat)
    g = BZTrellisQdc(bz, bz.volume / 2000, trellis_backend="gpu")
    ref = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume / 2000, backend="gpu")
    assert g.trellis.summary() == ref.summary()
    model = W.bvk_for(lat, masses)
    w, v = model.modes(g.trellis.vertices @ np.linalg.inv(lat.B))
    g.fill(w, [1, 0, 0, 0, 3], v, [0, 3 * v.shape[2], 0, 2, 1])
    Q = np.random.default_rng(2).uniform(-1, 1, size=(500, 3))
    vals, _ = g.ir_interpolate_at(Q)
    assert np.isfinite(vals).all() and vals.shape == (500, w.shape[1])

