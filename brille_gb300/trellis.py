"""Hybrid cube / tetrahedron trellis over the irreducible polyhedron.

Set-up code (host).  The reference builds its ``PolyTrellis`` in
``src/trellis_poly_parallel.tpp:74-482`` with TetGen for the cut cells; that
construction is outside the GPU query path.  This module builds a trellis with
the same structure and the same node semantics from scipy's Qhull:

* knots along x, y, z from the polyhedron's bounding box with spacing
  ``L / ceil(L / cbrt(max_volume))``, appended until the last knot reaches the
  maximum (reference ``trellis_poly_parallel.tpp:88-101``);
* a cell wholly inside the polyhedron is a cube node whose eight vertex
  indices are ordered (000)(100)(110)(010)(101)(001)(011)(111), so entries i
  and 7-i are body-diagonal partners (``src/trellis_node.hpp:127-131``);
* a cell cut by the polyhedron surface is a poly node: the convex cut cell is
  tetrahedralised (Delaunay), each tetrahedron stored with its four vertex
  indices (positively oriented), circumsphere and volume
  (``src/trellis_node.hpp:216-364``);
* any other cell is a null node.

Node linear index is ``i + nx*(j + ny*k)`` (``trellis_poly.hpp:557-562``).
"""
from __future__ import annotations

import numpy as np
from scipy.spatial import Delaunay, cKDTree

NODE_NULL, NODE_CUBE, NODE_POLY = 0, 1, 2

# corner order of a cube node: (000)(100)(110)(010)(101)(001)(011)(111)
CUBE_CORNERS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                         [1, 0, 1], [0, 0, 1], [0, 1, 1], [1, 1, 1]])
_BOX_EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (5, 4), (4, 7), (7, 6), (6, 5),
              (0, 5), (1, 4), (2, 7), (3, 6)]


def make_knots(vmin, vmax, max_volume):
    lengths = vmax - vmin
    step = lengths / np.ceil(lengths / np.cbrt(max_volume))
    knots = []
    for i in range(3):
        k = [vmin[i]]
        while k[-1] < vmax[i]:
            k.append(k[-1] + step[i])
        knots.append(np.array(k))
    return knots


def _poly_edges(verts, halfspaces, tol):
    A, b = halfspaces[:, :3], halfspaces[:, 3]
    nrm = np.linalg.norm(A, axis=1)
    on = np.abs((verts @ A.T + b) / nrm) < tol  # (nv, nh)
    edges = []
    for i in range(len(verts)):
        for j in range(i + 1, len(verts)):
            if np.count_nonzero(on[i] & on[j]) >= 2:
                edges.append((i, j))
    return np.array(edges, dtype=int).reshape(-1, 2)


def circumsphere(p):
    """Centre and radius of the sphere through four points (4, 3)."""
    a = p[1:] - p[0]
    rhs = 0.5 * np.sum(a * a, axis=1)
    c = np.linalg.solve(a, rhs)
    return p[0] + c, np.linalg.norm(c)


def _orient(p0, p1, p2, p3):
    return np.dot(p0 - p3, np.cross(p1 - p3, p2 - p3))


def orient_many(q):
    """orient3d of tetrahedra q (n, 4, 3): six times the signed volume."""
    return np.einsum("ij,ij->i", q[:, 0] - q[:, 3], np.cross(q[:, 1] - q[:, 3], q[:, 2] - q[:, 3]))


def circumspheres(q):
    """Centres (n, 3) and radii (n,) of the spheres through tetrahedra q (n, 4, 3)."""
    a = q[:, 1:] - q[:, :1]
    rhs = 0.5 * np.sum(a * a, axis=2)
    c = np.linalg.solve(a, rhs[..., None])[..., 0]
    return q[:, 0] + c, np.linalg.norm(c, axis=1)


def oriented_tets(points, tets):
    """tets (n, 4) reordered to positive orientation, with their circumsphere
    rows (centre x, y, z, radius) and volumes."""
    tets = np.array(tets, dtype=np.int64).reshape(-1, 4)
    if len(tets) == 0:
        return tets.astype(np.int32), np.zeros((0, 4)), np.zeros(0)
    o = orient_many(points[tets])
    flip = o < 0
    tets[flip] = tets[flip][:, [0, 2, 1, 3]]
    c, r = circumspheres(points[tets])
    return tets.astype(np.int32), np.concatenate([c, r[:, None]], axis=1), np.abs(o) / 6.0


class TrellisBuild:
    """Flat trellis tables (numpy) ready for the query-path C ABI.

    backend "host" builds every node here (cut cells tetrahedralised by
    Delaunay); "gpu" classifies the cells and splits the cut cells into
    tetrahedra on the GPU (``brx_trellis_cells_build``) and only merges the
    vertices here.  Both give the same knots, node types, vertices and cube
    nodes; the cut cells' tetrahedra differ (a fan over the facets instead
    of a Delaunay tetrahedralisation) and tile the same polytopes."""

    def __init__(self, ir_vertices, ir_halfspaces, max_volume, always_triangulate=False, backend="host",
                 device=0):
        verts = np.asarray(ir_vertices, float)
        hs = np.asarray(ir_halfspaces, float)
        scale = float(np.max(np.abs(verts)))
        tol = 1e-10 * max(scale, 1e-30)
        self.knots = make_knots(verts.min(axis=0), verts.max(axis=0), float(max_volume))
        if backend == "gpu":
            self._build_gpu(verts, hs, tol, always_triangulate, device)
            return
        if backend != "host":
            raise ValueError(f"unknown trellis backend {backend!r}")
        kx, ky, kz = self.knots
        nx, ny, nz = len(kx) - 1, len(ky) - 1, len(kz) - 1
        A, b = hs[:, :3], hs[:, 3]
        nrm = np.linalg.norm(A, axis=1)
        An, bn = A / nrm[:, None], b / nrm
        pedges = _poly_edges(verts, hs, tol)

        # signed distances of every knot-grid point to every polyhedron plane
        gx, gy, gz = np.meshgrid(kx, ky, kz, indexing="ij")
        grid = np.stack([gx, gy, gz], axis=-1)           # (nx+1, ny+1, nz+1, 3)
        dist = grid @ An.T + bn                           # (..., nh)
        inside = np.all(dist <= tol, axis=-1)

        node_type = np.zeros(nx * ny * nz, np.int32)
        node_index = np.full(nx * ny * nz, -1, np.int32)

        def corner(arr, c):
            return arr[c[0]:c[0] + nx, c[1]:c[1] + ny, c[2]:c[2] + nz]

        cin = np.stack([corner(inside, c) for c in CUBE_CORNERS], axis=-1)        # (nx, ny, nz, 8)
        out_all = np.ones((nx, ny, nz, len(bn)), bool)
        for c in CUBE_CORNERS:
            out_all &= corner(dist, c) > tol
        null = np.any(out_all, axis=-1)
        cube = cin.all(axis=-1) & ~null & (not always_triangulate)
        # linear node index i + nx (j + ny k): order cells by (k, j, i)
        cube_ijk = np.argwhere(cube.transpose(2, 1, 0))[:, ::-1]                # (i, j, k) in linear order
        cand_ijk = np.argwhere((~cube & ~null).transpose(2, 1, 0))[:, ::-1]
        lin_cube = cube_ijk[:, 0] + nx * (cube_ijk[:, 1] + ny * cube_ijk[:, 2])
        node_type[lin_cube] = NODE_CUBE
        node_index[lin_cube] = np.arange(len(lin_cube), dtype=np.int32)
        cube_pts = [[(i + c[0], j + c[1], k + c[2]) for c in CUBE_CORNERS] for i, j, k in cube_ijk]
        poly_cells = []
        for i, j, k in cand_ijk:
            lo = np.array([kx[i], ky[j], kz[k]])
            hi = np.array([kx[i + 1], ky[j + 1], kz[k + 1]])
            cand = self._cut_cell(lo, hi, verts, pedges, An, bn, tol)
            if cand is not None:
                poly_cells.append((int(i + nx * (j + ny * k)), cand))

        # global vertex list: knot points used by cube nodes first, then the
        # points of the cut cells, merged within tolerance
        grid_flat = grid.reshape(-1, 3)
        used = sorted({(a, b_, c) for cell in cube_pts for (a, b_, c) in cell})
        lin = {g: n for n, g in enumerate(used)}
        all_pts = [grid_flat[(a * (ny + 1) + b_) * (nz + 1) + c] for (a, b_, c) in used]
        offsets = []
        for _, cand in poly_cells:
            offsets.append(len(all_pts))
            all_pts.extend(cand)
        all_pts = np.array(all_pts).reshape(-1, 3)
        uniq_map = self._merge(all_pts, tol)
        keep, inv = np.unique(uniq_map, return_inverse=True)
        self.vertices = all_pts[keep]
        self.cube_vertices = np.array(
            [[inv[lin[p]] for p in cell] for cell in cube_pts], dtype=np.int32).reshape(-1, 8)
        tets, tet_off = [], [0]
        poly_node_ids = []
        for (lin_idx, cand), off in zip(poly_cells, offsets):
            gid = inv[np.arange(off, off + len(cand))]
            local = self._tetrahedralise(self.vertices[gid], tol)
            if len(local) == 0:
                continue
            poly_node_ids.append(lin_idx)
            tets.append(gid[local])
            tet_off.append(tet_off[-1] + len(local))
        tets, spheres, vols = oriented_tets(self.vertices, np.concatenate(tets) if tets else np.zeros((0, 4), int))
        for n, lin_idx in enumerate(poly_node_ids):
            node_type[lin_idx] = NODE_POLY
            node_index[lin_idx] = n
        self.node_type = node_type
        self.node_index = node_index
        self.poly_tet_offset = np.array(tet_off, dtype=np.int32)
        self.tet_vertices = tets
        self.tet_sphere = spheres
        self.tet_volume = vols
        self.shape = (nx, ny, nz)

    def _build_gpu(self, verts, hs, tol, always_triangulate, device):
        import ctypes as C

        from . import _abi
        from ._lib import load

        kx, ky, kz = self.knots
        nx, ny, nz = len(kx) - 1, len(ky) - 1, len(kz) - 1
        A, b = hs[:, :3], hs[:, 3]
        nrm = np.linalg.norm(A, axis=1)
        if not np.all(np.isfinite(hs)) or not np.all(nrm > 0):
            raise ValueError("every half-space needs a finite, non-zero normal")
        planes = np.concatenate([A / nrm[:, None], (b / nrm)[:, None]], axis=1)
        # no two planes alike (the kernel takes each plane as one facet)
        keep = []
        for i, pl in enumerate(planes):
            if not any(np.allclose(pl, planes[k], rtol=0, atol=1e-12) for k in keep):
                keep.append(i)
        planes = np.ascontiguousarray(planes[keep])
        edges = np.ascontiguousarray(_poly_edges(verts, hs, tol), np.int32)
        verts_c = np.ascontiguousarray(verts)
        knots = [np.ascontiguousarray(k, float) for k in self.knots]
        dp = C.POINTER(C.c_double)
        tin = _abi.TrellisIn()
        tin.n_vertices = len(verts_c)
        tin.vertices = verts_c.ctypes.data_as(dp)
        tin.n_planes = len(planes)
        tin.planes = planes.ctypes.data_as(dp)
        tin.n_edges = len(edges)
        tin.edges = edges.ctypes.data_as(C.POINTER(C.c_int32))
        for d in range(3):
            tin.n_knots[d] = len(knots[d])
            tin.knots[d] = knots[d].ctypes.data_as(dp)
        tin.tol = tol
        tin.always_triangulate = 1 if always_triangulate else 0
        cells = _abi.TrellisCells()
        lib = load()
        st = lib.brx_trellis_cells_build(C.byref(tin), int(device), C.byref(cells))
        if st != 0:
            raise RuntimeError(f"brx_trellis_cells_build failed: {_abi.STATUS_NAMES.get(st, st)}")
        try:
            n_nodes, n_poly = int(cells.n_nodes), int(cells.n_poly)
            node_type = np.ctypeslib.as_array(cells.node_type, (n_nodes,)).copy()
            poly_node = np.ctypeslib.as_array(cells.poly_node, (max(n_poly, 1),))[:n_poly].copy()
            poff = np.ctypeslib.as_array(cells.point_offset, (n_poly + 1,)).copy()
            toff = np.ctypeslib.as_array(cells.tet_offset, (n_poly + 1,)).copy()
            cut_pts = np.ctypeslib.as_array(cells.points, (max(int(poff[-1]), 1) * 3,))[:3 * poff[-1]].copy()
            local = np.ctypeslib.as_array(cells.tets, (max(int(toff[-1]), 1) * 4,))[:4 * toff[-1]].copy()
        finally:
            lib.brx_trellis_cells_free(C.byref(cells))
        self._assemble(node_type, poly_node, poff, toff, cut_pts.reshape(-1, 3), local.reshape(-1, 4), tol)

    def _assemble(self, node_type, poly_node, poff, toff, cut_pts, local, tol):
        """Trellis tables from per-cell results (brx_trellis_cells layout):
        node types, the poly nodes' linear indices, and per poly node its
        corner points (poff offsets into cut_pts) and tetrahedra as local
        corner indices (toff offsets into local).  Cube nodes take the knot
        points of their corners; all points are merged within tol."""
        kx, ky, kz = self.knots
        nx, ny, nz = len(kx) - 1, len(ky) - 1, len(kz) - 1
        node_type = np.array(node_type, np.int32)
        poly_node = np.asarray(poly_node, np.int64)
        poff, toff = np.asarray(poff, np.int64), np.asarray(toff, np.int64)
        n_nodes, n_poly = len(node_type), len(poly_node)
        cut_pts = np.asarray(cut_pts, float).reshape(-1, 3)
        local = np.asarray(local).reshape(-1, 4).astype(np.int64)
        # cube nodes: knot points of their corners, first in the vertex list
        lin_cube = np.nonzero(node_type == NODE_CUBE)[0]
        ci, cj, ck = lin_cube % nx, (lin_cube // nx) % ny, lin_cube // (nx * ny)
        g = ((ci[:, None] + CUBE_CORNERS[None, :, 0]) * (ny + 1) + (cj[:, None] + CUBE_CORNERS[None, :, 1])) * (nz + 1) \
            + (ck[:, None] + CUBE_CORNERS[None, :, 2])
        used = np.unique(g)
        ga, gb, gc = used // ((ny + 1) * (nz + 1)), (used // (nz + 1)) % (ny + 1), used % (nz + 1)
        grid_pts = np.stack([kx[ga], ky[gb], kz[gc]], axis=1)
        all_pts = np.concatenate([grid_pts, cut_pts]).reshape(-1, 3)
        uniq_map = self._merge(all_pts, tol)
        keepv, inv = np.unique(uniq_map, return_inverse=True)
        self.vertices = all_pts[keepv]
        self.cube_vertices = inv[np.searchsorted(used, g)].astype(np.int32).reshape(-1, 8)
        tet_cell = np.repeat(np.arange(n_poly), np.diff(toff))
        gtets = inv[len(used) + poff[tet_cell][:, None] + local]
        # corners of one cell merged into one vertex by the global merge
        # (closer than tol to the same point of a neighbour) leave a flat
        # tetrahedron: drop it, and a cell left without any
        ok = np.ones(len(gtets), bool)
        for a_, b_ in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)):
            ok &= gtets[:, a_] != gtets[:, b_]
        if not ok.all():
            gtets, tet_cell = gtets[ok], tet_cell[ok]
            cnt = np.bincount(tet_cell, minlength=n_poly)
            node_type[poly_node[cnt == 0]] = NODE_NULL
            live = cnt > 0
            renum = np.cumsum(live) - 1
            tet_cell = renum[tet_cell]
            poly_node = poly_node[live]
            n_poly = len(poly_node)
            toff = np.concatenate([[0], np.cumsum(cnt[live])])
        tets, spheres, vols = oriented_tets(self.vertices, gtets)
        node_index = np.full(n_nodes, -1, np.int32)
        node_index[lin_cube] = np.arange(len(lin_cube), dtype=np.int32)
        node_index[poly_node] = np.arange(n_poly, dtype=np.int32)
        self.node_type = node_type.astype(np.int32)
        self.node_index = node_index
        self.poly_tet_offset = toff.astype(np.int32)
        self.tet_vertices = tets
        self.tet_sphere = spheres
        self.tet_volume = vols
        self.shape = (nx, ny, nz)

    @staticmethod
    def _merge(points, tol):
        """Index of each point's representative: the lowest index among the
        points joined to it by chains of pairs closer than tol."""
        from scipy.sparse import coo_matrix
        from scipy.sparse.csgraph import connected_components

        n = len(points)
        pairs = cKDTree(points).query_pairs(r=tol, output_type="ndarray")
        if len(pairs) == 0:
            return np.arange(n)
        graph = coo_matrix((np.ones(len(pairs), np.int8), (pairs[:, 0], pairs[:, 1])), shape=(n, n))
        _, label = connected_components(graph, directed=False)
        rep = np.full(label.max() + 1, n, np.int64)
        np.minimum.at(rep, label, np.arange(n))
        return rep[label]

    @staticmethod
    def _cut_cell(lo, hi, verts, pedges, An, bn, tol):
        corners = lo + CUBE_CORNERS * (hi - lo)
        pts = []
        # box corners inside the polyhedron
        d = corners @ An.T + bn
        pts.extend(corners[np.all(d <= tol, axis=1)])
        # polyhedron vertices inside the box
        inbox = np.all((verts >= lo - tol) & (verts <= hi + tol), axis=1)
        pts.extend(verts[inbox])
        # box edges crossing polyhedron planes
        for a, b in _BOX_EDGES:
            pa, pb = corners[a], corners[b]
            da, db = d[a], d[b]
            for h in range(len(bn)):
                if (da[h] < -tol and db[h] > tol) or (da[h] > tol and db[h] < -tol):
                    t = da[h] / (da[h] - db[h])
                    x = pa + t * (pb - pa)
                    if np.all(x @ An.T + bn <= tol):
                        pts.append(x)
        # polyhedron edges crossing box faces
        for a, b in pedges:
            pa, pb = verts[a], verts[b]
            for ax in range(3):
                for plane in (lo[ax], hi[ax]):
                    ua, ub = pa[ax] - plane, pb[ax] - plane
                    if (ua < -tol and ub > tol) or (ua > tol and ub < -tol):
                        t = ua / (ua - ub)
                        x = pa + t * (pb - pa)
                        x[ax] = plane
                        if np.all((x >= lo - tol) & (x <= hi + tol)):
                            pts.append(x)
        if len(pts) < 4:
            return None
        pts = np.array(pts)
        keep = []
        for p in pts:
            if not any(np.linalg.norm(p - q) < tol for q in keep):
                keep.append(p)
        pts = np.clip(np.array(keep), lo, hi)
        if len(pts) < 4:
            return None
        c = pts - pts.mean(axis=0)
        if np.linalg.matrix_rank(c, tol=1e-9 * np.max(hi - lo)) < 3:
            return None
        return pts

    @staticmethod
    def _tetrahedralise(p, tol):
        """Delaunay simplices (m, 4) of the points p that are not flat."""
        try:
            tri = Delaunay(p, qhull_options="Qbb Qc Qz Q12 Qt")
        except Exception:
            return np.zeros((0, 4), np.int64)
        span = np.max(np.ptp(p, axis=0))
        s = tri.simplices
        return s[np.abs(orient_many(p[s])) > 1e-12 * span ** 3]

    @property
    def n_nodes(self):
        return self.node_type.size

    # ---------------------------------------------------------- persistence
    # The reference persists a trellis through HDF5 (bz_trellis.hpp:198-224);
    # here the flat tables go to one .npz file, with a fingerprint of the
    # construction inputs so that a cache can tell a stale file.
    _TABLES = ("vertices", "cube_vertices", "node_type", "node_index", "poly_tet_offset", "tet_vertices",
               "tet_sphere", "tet_volume")

    @staticmethod
    def fingerprint(ir_vertices, ir_halfspaces, max_volume, always_triangulate=False):
        """SHA-256 of the construction inputs (exact bytes)."""
        import hashlib
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(ir_vertices, float).tobytes())
        h.update(np.ascontiguousarray(ir_halfspaces, float).tobytes())
        h.update(np.float64(max_volume).tobytes())
        h.update(b"t" if always_triangulate else b"f")
        return h.hexdigest()

    def save(self, path, fingerprint=""):
        """Write the tables to path (.npz)."""
        arrays = {k: getattr(self, k) for k in self._TABLES}
        for d in range(3):
            arrays[f"knots{d}"] = np.asarray(self.knots[d], float)
        arrays["shape"] = np.asarray(self.shape, np.int64)
        arrays["fingerprint"] = np.array(fingerprint)
        np.savez(path, **arrays)

    @classmethod
    def load(cls, path, fingerprint=None):
        """Tables saved by save(); with fingerprint given, a file made from
        other inputs raises ValueError."""
        z = np.load(path, allow_pickle=False)
        if fingerprint is not None and str(z["fingerprint"]) != fingerprint:
            raise ValueError(f"{path}: trellis tables were built from other inputs")
        t = cls.__new__(cls)
        for k in cls._TABLES:
            setattr(t, k, z[k])
        t.knots = [z[f"knots{d}"] for d in range(3)]
        t.shape = tuple(int(x) for x in z["shape"])
        nx, ny, nz = t.shape
        if (t.node_type.size != nx * ny * nz or any(len(t.knots[d]) != t.shape[d] + 1 for d in range(3))
                or t.poly_tet_offset.size < 1 or t.poly_tet_offset[-1] != len(t.tet_vertices)):
            raise ValueError(f"{path}: inconsistent trellis tables")
        return t

    @classmethod
    def cached(cls, ir_vertices, ir_halfspaces, max_volume, path, always_triangulate=False):
        """Load the trellis for these inputs from path if it holds them, else
        build it and write it there."""
        import os
        fp = cls.fingerprint(ir_vertices, ir_halfspaces, max_volume, always_triangulate)
        if os.path.exists(path):
            try:
                return cls.load(path, fingerprint=fp)
            except ValueError:
                pass
        t = cls(ir_vertices, ir_halfspaces, max_volume, always_triangulate)
        t.save(path, fingerprint=fp)
        return t

    def permutation_keys(self):
        """Keys i*n_vertices+j of every ordered pair of distinct vertices that
        share a cube node or one tetrahedron of a poly node, sorted: the pairs
        whose mode permutations sort() determines (PolyTrellis::collect_keys
        and collect_keys_node, src/trellis_poly_parallel.tpp:485-526;
        permutation_table_keys_from_indicies, src/permutation_table.hpp:284-292)."""
        n = np.int64(len(self.vertices))
        keys = []
        for groups in (self.cube_vertices, self.tet_vertices):
            g = np.asarray(groups, np.int64)
            if g.size == 0:
                continue
            m = g.shape[1]
            a, b = np.nonzero(~np.eye(m, dtype=bool))
            i, j = g[:, a].ravel(), g[:, b].ravel()
            keep = i != j
            keys.append(i[keep] * n + j[keep])
        if not keys:
            return np.zeros(0, np.int64)
        return np.unique(np.concatenate(keys))

    def summary(self):
        return dict(vertices=len(self.vertices), cube=int(np.sum(self.node_type == NODE_CUBE)),
                    poly=int(np.sum(self.node_type == NODE_POLY)), tets=len(self.tet_vertices),
                    nodes=self.n_nodes, shape=self.shape)


class PointTrellis(TrellisBuild):
    """A one-node trellis whose vertices are exactly the given points.

    The single poly node holds the Delaunay tetrahedralisation of the points'
    convex hull.  It is used to re-create a grid from vertex positions alone,
    for example the reference's stored grid in its Γ-rotation fixture.
    """

    def __init__(self, points_xyz):  # noqa: D401 - deliberately skips TrellisBuild.__init__
        p = np.asarray(points_xyz, float)
        lo, hi = p.min(axis=0), p.max(axis=0)
        pad = 1e-9 * max(float(np.max(hi - lo)), 1.0)
        self.knots = [np.array([lo[d] - pad, hi[d] + pad]) for d in range(3)]
        self.vertices = p.copy()
        self.cube_vertices = np.zeros((0, 8), np.int32)
        tets, spheres, vols = oriented_tets(p, self._tetrahedralise(p, 1e-12))
        self.node_type = np.array([NODE_POLY], np.int32)
        self.node_index = np.array([0], np.int32)
        self.poly_tet_offset = np.array([0, len(tets)], np.int32)
        self.tet_vertices = tets
        self.tet_sphere = spheres
        self.tet_volume = vols
        self.shape = (1, 1, 1)
