"""Tetrahedral meshes of the irreducible polyhedron for BZMeshQ and BZNestQ.

Set-up code (host).  The reference offers two grids besides the trellis:

* ``BrillouinZoneMesh3`` (``src/bz_mesh.hpp``, ``src/mesh.hpp``) meshes the
  irreducible polyhedron with TetGen in layers of decreasing maximum
  tetrahedron volume (``triangulate``, ``src/triangulation_layers.hpp:633-670``)
  and locates a point by walking the layers down to the finest one, where it
  takes the first tetrahedron that contains the point and keeps the
  barycentric weights that are not ≈ 0 (``unsafe_locate``, :169-180);
* ``BrillouinZoneNest3`` (``src/bz_nest.hpp``, ``src/nest.hpp``) refines a root
  tetrahedralisation into a tree of branches down to a maximum leaf volume
  (``Nest::construct``; the volume is given, or the polyhedron's volume over a
  number density, :312-320) and locates a point by descending the tree to the
  leaf that contains it.

Either way the answer is the finest-level tetrahedron that contains q and its
barycentric weights; the coarser levels only speed the search.  Here the
finest level is built directly and bucketed for the GPU instead: the
tetrahedra are listed in every cell of a regular knot grid that they may meet,
so that the trellis tables (``include/brx.h``) describe the mesh
with poly nodes only and the trellis locate kernel answers the query (cell
from the knots, then the first listed tetrahedron that contains q).

The mesh: Delaunay tetrahedralisation (Qhull) of the polyhedron's vertices,
refined by inserting a point into every tetrahedron larger than the maximum
volume (its circumcentre where that lies well inside, its projection onto
the boundary where it lies outside, else its centroid) until none is (or
``max_points`` is reached).  The polyhedron is convex, so the Delaunay mesh
of points inside it covers it exactly.  It is not the
reference's TetGen mesh: grids built here are compared with the oracle on
the same tables.
"""
from __future__ import annotations

import numpy as np
from scipy.spatial import Delaunay

from .trellis import NODE_POLY, TrellisBuild, _orient, circumspheres


def _circumcentres(q):
    """Circumcentres of tetrahedra q (n, 4, 3)."""
    a = q[:, 1:] - q[:, :1]
    rhs = 0.5 * np.sum(a * a, axis=2)
    det = np.linalg.det(a)
    ok = np.abs(det) > 1e-300
    c = np.zeros((len(q), 3))
    c[ok] = np.linalg.solve(a[ok], rhs[ok][..., None])[..., 0]
    return q[:, 0] + c, ok


def delaunay_mesh(points, max_volume=-1.0, max_points=-1, max_rounds=200):
    """(vertices, tetrahedra, volumes) of the convex hull of points, every
    tetrahedron positively oriented and, when max_volume > 0, no larger than
    max_volume (unless max_points stops the refinement first).  Refinement
    inserts the circumcentre of each tetrahedron above the limit where it
    lies well inside the hull (Delaunay refinement, which removes the
    worst-shaped tetrahedra first), its projection onto the hull face it
    crosses where that lies on the hull, and its centroid otherwise; never a
    point next to an existing one."""
    from scipy.spatial import ConvexHull, cKDTree

    p = np.unique(np.asarray(points, float), axis=0)
    eq = ConvexHull(p).equations if len(p) >= 4 else None
    for _ in range(max_rounds):
        tri = Delaunay(p, qhull_options="Qbb Qc Qz Q12 Qt")
        s = tri.simplices
        q = p[s]
        o = np.einsum("ij,ij->i", q[:, 0] - q[:, 3], np.cross(q[:, 1] - q[:, 3], q[:, 2] - q[:, 3]))
        span = float(np.max(np.ptp(p, axis=0)))
        keep = np.abs(o) > 1e-12 * span ** 3
        s, o = s[keep], o[keep]
        flip = o < 0
        s[flip] = s[flip][:, [0, 2, 1, 3]]
        vol = np.abs(o) / 6.0
        if max_volume is None or max_volume <= 0:
            break
        big = np.nonzero(vol > max_volume)[0]
        if big.size == 0:
            break
        room = (max_points - len(p)) if max_points and max_points > 0 else big.size
        if room <= 0:
            break
        big = big[np.argsort(-vol[big], kind="stable")][:room]
        q = p[s[big]]
        new = q.mean(axis=1)
        cc, ok = _circumcentres(q)
        edge = np.cbrt(vol[big])
        d = cc @ eq[:, :3].T + eq[:, 3]  # signed distances to the hull planes, < 0 inside
        inside = np.all(d < -0.25 * edge[:, None], axis=1)
        # a circumcentre outside or next to the boundary goes onto the plane
        # it violates most, when that point lies on the hull
        f = np.argmax(d, axis=1)
        proj = cc - d[np.arange(len(cc)), f][:, None] * eq[f, :3]
        on_face = ~inside & np.all(proj @ eq[:, :3].T + eq[:, 3] < 1e-12 * span, axis=1)
        cand = np.where(inside[:, None], cc, proj)
        use = ok & (inside | on_face) & (cKDTree(p).query(cand)[0] > 0.5 * edge)
        new[use] = cand[use]
        new = new[np.unique(np.round(new / (1e-6 * span)), axis=0, return_index=True)[1]]
        p = np.vstack([p, new])
    return p, s.astype(np.int32), vol


class MeshTrellis(TrellisBuild):
    """A tetrahedral mesh of the irreducible polyhedron in trellis form: a
    knot grid whose non-empty cells are poly nodes listing every tetrahedron
    that may meet the cell (its bounding box touches the cell and none of its
    face planes separates the two; a tetrahedron appears once per such cell,
    ``mesh_tetrahedra`` holds each once).  Cells are cell_factor times
    the cube root of the mean tetrahedron volume on a side."""

    def __init__(self, ir_vertices, max_volume=-1.0, max_points=-1, cell_factor=2.0):  # noqa: D401
        verts, tets, vol = delaunay_mesh(ir_vertices, max_volume, max_points)
        self.vertices = verts
        self.mesh_tetrahedra = tets
        self.cube_vertices = np.zeros((0, 8), np.int32)
        lo, hi = verts.min(axis=0), verts.max(axis=0)
        ext = hi - lo
        pad = 1e-9 * max(float(np.max(ext)), 1e-30)
        lo, hi = lo - pad, hi + pad
        ext = hi - lo
        h = cell_factor * np.cbrt(float(np.mean(vol)))
        n = np.maximum(1, np.ceil(ext / h).astype(int))
        while np.prod(n) > 4_000_000:
            n = np.maximum(1, n // 2)
        self.knots = [np.linspace(lo[d], hi[d], n[d] + 1) for d in range(3)]
        nx, ny, nz = (int(x) for x in n)
        # cells touched by each tetrahedron's bounding box (closed, so that a
        # point on a knot plane finds its tetrahedron from either side)
        tmin = verts[tets].min(axis=1)
        tmax = verts[tets].max(axis=1)
        eps = 1e-9 * float(np.max(ext))
        c0 = np.empty((len(tets), 3), np.int64)
        c1 = np.empty((len(tets), 3), np.int64)
        for d in range(3):
            k = self.knots[d]
            c0[:, d] = np.clip(np.searchsorted(k, tmin[:, d] - eps, side="right") - 1, 0, n[d] - 1)
            c1[:, d] = np.clip(np.searchsorted(k, tmax[:, d] + eps, side="left") - 1, 0, n[d] - 1)
        span = c1 - c0 + 1
        count = np.prod(span, axis=1)
        tet_of = np.repeat(np.arange(len(tets)), count)
        local = np.arange(count.sum()) - np.repeat(np.cumsum(count) - count, count)
        sx, sy = np.repeat(span[:, 0], count), np.repeat(span[:, 1], count)
        ci = np.repeat(c0[:, 0], count) + local % sx
        cj = np.repeat(c0[:, 1], count) + (local // sx) % sy
        ck = np.repeat(c0[:, 2], count) + local // (sx * sy)
        # drop the cells that one face plane of the tetrahedron separates from
        # it (all eight box corners strictly beyond the plane): a sound test,
        # it never drops a cell the tetrahedron meets
        keep = np.ones(len(tet_of), bool)
        kx, ky, kz = self.knots
        corners = np.stack(np.meshgrid([0, 1], [0, 1], [0, 1], indexing="ij"), axis=-1).reshape(8, 3)
        for f, opp in ((0, 3), (1, 2), (2, 1), (3, 0)):
            face = [a for a in range(4) if a != opp]
            a, b, c = (verts[tets[:, x]] for x in face)
            nrm = np.cross(b - a, c - a)
            # orient outward: away from the opposite vertex
            sgn = np.sign(np.einsum("ij,ij->i", nrm, verts[tets[:, opp]] - a))
            nrm = -nrm * sgn[:, None]
            nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
            off = np.einsum("ij,ij->i", nrm, a)
            n_e, o_e = nrm[tet_of], off[tet_of]
            dmin = np.full(len(tet_of), np.inf)
            for cc in corners:
                x = np.stack([kx[ci + cc[0]], ky[cj + cc[1]], kz[ck + cc[2]]], axis=1)
                dmin = np.minimum(dmin, np.einsum("ij,ij->i", n_e, x) - o_e)
            keep &= ~(dmin > eps)
        ci, cj, ck, tet_of = ci[keep], cj[keep], ck[keep], tet_of[keep]
        cell = ci + nx * (cj + ny * ck)
        order = np.lexsort((tet_of, cell))
        cell, tet_of = cell[order], tet_of[order]
        cells, first = np.unique(cell, return_index=True)
        node_type = np.zeros(nx * ny * nz, np.int32)
        node_index = np.full(nx * ny * nz, -1, np.int32)
        node_type[cells] = NODE_POLY
        node_index[cells] = np.arange(len(cells), dtype=np.int32)
        self.node_type = node_type
        self.node_index = node_index
        self.poly_tet_offset = np.append(first, len(cell)).astype(np.int32)
        self.tet_mesh_index = tet_of.astype(np.int32)  # mesh tetrahedron of each listed entry
        self.tet_vertices = tets[tet_of]
        c, r = circumspheres(verts[tets])
        self.tet_sphere = np.concatenate([c, r[:, None]], axis=1)[tet_of]
        self.tet_volume = vol[tet_of]
        self.shape = (nx, ny, nz)

    @property
    def total_volume(self):
        return float(np.sum(self.tet_volume[np.unique(self.tet_mesh_index, return_index=True)[1]]))


def _check_orientation(verts, tets):
    """True when every tetrahedron is positively oriented."""
    return all(_orient(*verts[t]) > 0 for t in tets)
