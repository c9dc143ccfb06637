"""The host half of the GPU trellis build (TrellisBuild._assemble: cube
corners from the knots, the global merge of cut-cell corners, node tables),
fed on the CPU with the per-cell results of the host builder in the layout
brx_trellis_cells_build returns: it must give back the host trellis."""
import numpy as np
import pytest
from scipy.spatial import cKDTree

from _cases import CRYSTALS
from brille_gb300 import workloads as W
from brille_gb300.bz import BrillouinZone
from brille_gb300.trellis import NODE_CUBE, NODE_POLY, TrellisBuild


def _cells_of(h):
    """Per poly node: the points its tetrahedra use and the tetrahedra as
    local indices, concatenated with offsets (brx_trellis_cells layout)."""
    poly_node = np.nonzero(h.node_type == NODE_POLY)[0]
    poff, toff, pts, local = [0], [0], [], []
    for n in poly_node:
        k = h.node_index[n]
        tv = h.tet_vertices[h.poly_tet_offset[k]:h.poly_tet_offset[k + 1]]
        ids, loc = np.unique(tv, return_inverse=True)
        pts.append(h.vertices[ids])
        local.append(loc.reshape(-1, 4))
        poff.append(poff[-1] + len(ids))
        toff.append(toff[-1] + len(tv))
    return (h.node_type.copy(), poly_node, np.array(poff), np.array(toff), np.concatenate(pts),
            np.concatenate(local))


@pytest.mark.parametrize("name,frac", [("diamond2", 1 / 2000), ("hex16", 1 / 2000), ("R-3m", 1 / 2000)])
def test_assemble_rebuilds_the_host_trellis(name, frac):
    lat, _ = CRYSTALS[name]() if name in CRYSTALS else W.random_crystal(name, 2, seed=3)
    bz = BrillouinZone(lat)
    h = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * frac)
    a = TrellisBuild.__new__(TrellisBuild)
    a.knots = h.knots
    scale = float(np.max(np.abs(bz.ir_vertices_invA)))
    a._assemble(*_cells_of(h), 1e-10 * scale)
    assert a.shape == h.shape
    assert np.array_equal(a.node_type, h.node_type)
    assert np.array_equal(a.node_index, h.node_index)
    # cube corners: the same coordinates in the same order
    assert np.array_equal(a.vertices[a.cube_vertices], h.vertices[h.cube_vertices])
    # the vertices in use are the same points
    used_h = np.unique(np.concatenate([h.cube_vertices.ravel(), h.tet_vertices.ravel()]))
    assert len(a.vertices) == len(used_h)
    d, _ = cKDTree(h.vertices[used_h]).query(a.vertices)
    assert d.max() == 0.0
    # the same tetrahedra, node by node, positively oriented
    assert np.array_equal(a.poly_tet_offset, h.poly_tet_offset)
    assert len(a.tet_vertices) == len(h.tet_vertices)
    assert np.allclose(a.tet_volume, h.tet_volume, rtol=1e-12, atol=0)
    got = np.sort(a.vertices[a.tet_vertices].reshape(len(a.tet_vertices), -1), axis=1)
    want = np.sort(h.vertices[h.tet_vertices].reshape(len(h.tet_vertices), -1), axis=1)
    assert np.array_equal(got, want)
