"""First Brillouin zone, irreducible wedge and irreducible polyhedron.

Set-up code (host, numpy/scipy).  The reference constructs the same objects in
``src/bz.cpp`` (Voronoi cutting) and ``src/bz_wedge.cpp`` (wedge search); both
are one-time set-up and outside the GPU query path.  What the query path
consumes from here is flat:

* per first-zone face: three points on the face, its unit outward normal, the
  primitive reciprocal-lattice vector τ whose bisector it is, and |τ|
  (reference ``BrillouinZone::moveinto``, ``src/bz_move.cpp:123-141``);
* the irreducible-wedge normals (``BrillouinZone::_inside_wedge_outer``,
  ``src/bz.hpp:757-763``);
* the point-group matrices with their inverse and identity indices.

Construction here is this package's own: the zone is the Voronoi cell of the
primitive reciprocal lattice (scipy's Qhull half-space intersection), and the
wedge is the Dirichlet domain of one generic point under the reciprocal-space
point group, a fundamental domain for any finite orthogonal group.  It is a
different construction from the reference's, so the wedge it chooses may
differ; the query path only requires that it be a fundamental domain.
"""
from __future__ import annotations

import itertools

import numpy as np
from scipy.spatial import HalfspaceIntersection

from .crystal import Lattice, PointSymmetry


def _unique_rows(x, tol):
    out = []
    for p in x:
        if not any(np.linalg.norm(p - q) < tol for q in out):
            out.append(p)
    return np.array(out)


def _polytope(halfspaces, interior):
    """Vertices and per-halfspace vertex lists of {x : A x + b <= 0}."""
    hs = HalfspaceIntersection(halfspaces, interior)
    scale = np.max(np.abs(hs.intersections)) if len(hs.intersections) else 1.0
    verts = _unique_rows(hs.intersections, 1e-9 * max(scale, 1.0))
    faces = []
    A, b = halfspaces[:, :3], halfspaces[:, 3]
    nrm = np.linalg.norm(A, axis=1)
    for i in range(len(halfspaces)):
        d = (verts @ A[i] + b[i]) / nrm[i]
        on = np.nonzero(np.abs(d) < 1e-9 * max(scale, 1.0))[0]
        faces.append(on)
    return verts, faces


def _ccw(verts, idx, normal):
    """Order face vertex indices counter-clockwise seen from outside."""
    p = verts[idx]
    c = p.mean(axis=0)
    u = p[0] - c
    u /= np.linalg.norm(u)
    v = np.cross(normal, u)
    ang = np.arctan2((p - c) @ v, (p - c) @ u)
    return np.asarray(idx)[np.argsort(ang)]


def orient3d(a, b, c, d):
    """(a-d)·((b-d)×(c-d)) — the reference's pseudo_orient3d
    (``src/geometry.hpp:118-139``)."""
    return np.dot(a - d, np.cross(b - d, c - d))


def _plane_triple(verts, ring):
    """Three vertices of a face ring spanning the largest triangle."""
    best, trip = -1.0, None
    n = len(ring)
    for j in range(1, n - 1):
        for k in range(j + 1, n):
            area = np.linalg.norm(np.cross(verts[ring[j]] - verts[ring[0]], verts[ring[k]] - verts[ring[0]]))
            if area > best:
                best, trip = area, (ring[0], ring[j], ring[k])
    return trip


class BrillouinZone:
    """First Brillouin zone and irreducible polyhedron of a lattice.

    Mirrors the reference's ``BrillouinZone(lattice, use_primitive=True,
    search_length=1, time_reversal_symmetry=False, wedge_search=True,
    divide_primitive=True)`` surface (``wrap/_bz.cpp:156-203``).  The zone is
    always the Voronoi cell of the primitive reciprocal lattice (the
    reference's ``use_primitive=True``, which the query path needs);
    ``search_length`` sets the shell of lattice points searched, at least 2;
    ``divide_primitive`` and ``approx_config`` are accepted and do not change
    the construction.  ``time_reversal`` is a short name for
    ``time_reversal_symmetry``.
    """

    _ARGS = ("use_primitive", "search_length", "time_reversal_symmetry", "wedge_search", "divide_primitive")
    _DEFAULTS = (True, 1, False, True, True)

    def __init__(self, lattice: Lattice, *args, time_reversal=None, extent=None, **kwargs):
        from .approx import ApproxConfig

        # the reference's two constructors: (lattice, use_primitive, ...) and
        # (lattice, approx_config, use_primitive, ...)
        approx_config = kwargs.pop("approx_config", None)
        if args and isinstance(args[0], ApproxConfig):
            approx_config, args = args[0], args[1:]
        if len(args) > len(self._ARGS):
            raise TypeError("too many arguments for BrillouinZone")
        opt = dict(zip(self._ARGS, self._DEFAULTS))
        opt.update(zip(self._ARGS, args))
        for k, v in kwargs.items():
            if k not in opt:
                raise TypeError(f"BrillouinZone() got an unexpected keyword argument '{k}'")
            opt[k] = v
        if not opt["use_primitive"]:
            raise ValueError("only the primitive Brillouin zone (use_primitive=True) is supported")
        if time_reversal is None:
            time_reversal = opt["time_reversal_symmetry"]
        if extent is None:
            extent = max(2, int(opt["search_length"]))
        wedge_search = opt["wedge_search"]
        self.approx_config = approx_config
        self.lattice = lattice
        self.time_reversal = bool(time_reversal)
        self.wedge_search = bool(wedge_search)
        self.Bp = lattice.primitive_B()
        self._first_zone(extent)
        pg = lattice.pointgroup
        if self.time_reversal:
            pg = pg.add_space_inversion()
        self.pointgroup: PointSymmetry = pg
        self._wedge()

    # ---------------------------------------------------------------- zone
    def _first_zone(self, extent):
        ns = np.array([n for n in itertools.product(range(-extent, extent + 1), repeat=3) if any(n)])
        G = ns @ self.Bp
        hs = np.hstack([G, -0.5 * np.sum(G * G, axis=1)[:, None]])
        verts, faces = _polytope(hs, np.zeros(3))
        keep = [i for i, f in enumerate(faces) if len(f) >= 3]
        self.vertices_invA = verts
        self.face_tau = ns[keep].astype(np.int32)
        Gk = G[keep]
        self.face_tau_len = np.linalg.norm(Gk, axis=1)
        self.face_normal = Gk / self.face_tau_len[:, None]
        rings, abc = [], []
        for i, fi in zip(keep, range(len(keep))):
            ring = _ccw(verts, faces[i], self.face_normal[fi])
            rings.append(ring)
            a, b, c = _plane_triple(verts, ring)
            pa, pb, pc = verts[a], verts[b], verts[c]
            if orient3d(pa, pb, pc, np.zeros(3)) < 0:
                pb, pc = pc, pb
            abc.append(np.concatenate([pa, pb, pc]))
        self.face_rings = rings
        self.face_abc = np.array(abc)
        self.halfspaces = hs[keep]
        self.volume = abs(np.linalg.det(self.Bp))

    # --------------------------------------------------------------- wedge
    def _cartesian_ops(self):
        """Reciprocal-space Cartesian action of each point operation:
        q_xyz -> S q_xyz with S = Bᵀ Wᵀ B⁻ᵀ (q_hkl -> Wᵀ q_hkl)."""
        B = self.lattice.B
        Binv_T = np.linalg.inv(B.T)
        return np.array([B.T @ W.T @ Binv_T for W in self.pointgroup.W])

    def _wedge(self):
        S = self._cartesian_ops()
        inr = np.min(self.face_tau_len) / 2
        normals = []
        if self.wedge_search and self.pointgroup.size > 1:
            p0 = np.array([0.9, 0.2, 0.1]) + np.array([1.3e-3, 2.9e-3, 0.7e-3])
            p0 = 0.25 * inr * p0 / np.linalg.norm(p0)
            cand = []
            for s in S:
                n = p0 - s @ p0
                if np.linalg.norm(n) > 1e-9 * inr:
                    cand.append(n / np.linalg.norm(n))
            cand = _unique_rows(np.array(cand), 1e-9)
            hs = np.vstack([self.halfspaces, np.hstack([-cand, np.zeros((len(cand), 1))])])
            verts, faces = _polytope(hs, p0)
            nz = len(self.halfspaces)
            for k in range(len(cand)):
                if len(faces[nz + k]) >= 3:
                    normals.append(cand[k])
        self.wedge_normal = np.array(normals).reshape(-1, 3)
        # the irreducible polyhedron: zone ∩ wedge
        hs = np.vstack([self.halfspaces, np.hstack([-self.wedge_normal, np.zeros((len(self.wedge_normal), 1))])])
        if len(self.wedge_normal):
            interior = p0
        else:
            interior = np.zeros(3)
        verts, faces = _polytope(hs, interior)
        self.ir_vertices_invA = verts
        self.ir_halfspaces = hs
        self.ir_faces = [f for f in faces if len(f) >= 3]

    # ------------------------------------------------------------- helpers
    def isinside(self, q_hkl):
        """Inside the first zone (tolerant orient3d test, outer lattice)."""
        x = np.atleast_2d(q_hkl) @ self.lattice.B
        a, b, c = self.face_abc[:, 0:3], self.face_abc[:, 3:6], self.face_abc[:, 6:9]
        out = []
        for p in x:
            o = np.einsum("ij,ij->i", a - p, np.cross(b - p, c - p))
            out.append(o.min() > -1e-12)
        return np.array(out)

    # ------------------------------------------------- reference accessors
    def _rlu(self, xyz):
        return np.asarray(xyz) @ np.linalg.inv(self.lattice.B)

    @property
    def vertices(self):
        """First-zone vertices in r.l.u. (wrap/_bz.cpp:267-271); Å⁻¹ in
        ``vertices_invA``."""
        return self._rlu(self.vertices_invA)

    @property
    def ir_vertices(self):
        """Irreducible-polyhedron vertices in r.l.u. (wrap/_bz.cpp:334-338);
        Å⁻¹ in ``ir_vertices_invA``."""
        return self._rlu(self.ir_vertices_invA)

    @property
    def wedge_normals(self):
        """Wedge plane normals in r.l.u. components (wrap/_bz.cpp:361-365);
        Cartesian in ``wedge_normals_invA``."""
        return self._rlu(self.wedge_normal)

    @property
    def wedge_normals_invA(self):
        return self.wedge_normal.copy()

    @property
    def normals_invA(self):
        """Outward unit normals of the first zone's faces (Å⁻¹)."""
        return self.face_normal.copy()

    @property
    def normals(self):
        return self._rlu(self.face_normal)

    @property
    def points_invA(self):
        """Centre of each face: half its reciprocal lattice vector (Å⁻¹)."""
        return 0.5 * self.face_normal * self.face_tau_len[:, None]

    @property
    def points(self):
        return self._rlu(self.points_invA)

    # ------------------------------------------------- moves, on the GPU
    def _mover(self):
        """A query handle whose trellis is the irreducible polyhedron alone:
        its locate kernel runs the move and wedge stages of the query path."""
        if getattr(self, "_move_grid", None) is None:
            from .grid import BZTrellisQdd
            from .trellis import PointTrellis

            self._move_grid = BZTrellisQdd(self, trellis=PointTrellis(self.ir_vertices_invA))
        return self._move_grid

    def _move(self, Q, ir, message):
        Q = np.asarray(Q, dtype=np.float64)
        if Q.shape[-1] != 3:
            raise RuntimeError("The last dimension must have size 3")
        rec = self._mover().locate(Q.reshape(-1, 3), ir=ir)
        # 4: move failed, 5: outside the irreducible zone; locate statuses
        # of the stand-in trellis do not concern the move
        if np.isin(rec["status"], (4, 5)).any():
            raise RuntimeError(message)
        return rec

    def moveinto(self, Q, threads=0):
        """(q, tau) with Q = q + tau, q inside the first zone and tau integer,
        all in r.l.u. (BrillouinZone::moveinto, src/bz_move.cpp:103-163;
        wrap/_bz.cpp:401-432), computed by the query path's FP64 G-shift
        kernel; ``threads`` is accepted for compatibility."""
        Q = np.asarray(Q, dtype=np.float64)
        rec = self._move(Q, False, "failed to move all Q into the first Brillouin Zone")
        return rec["q_ir"].reshape(Q.shape), rec["tau"].reshape(Q.shape)

    def ir_moveinto(self, Q, threads=0):
        """(q_ir, tau, R, R⁻¹): the irreducible q_ir, the lattice vector tau
        and the point operations (direct-lattice integer matrices, one 3×3
        per Q) with Q = Rᵀ q_ir + tau (BrillouinZone::ir_moveinto,
        src/bz_move.cpp:257-295; wrap/_bz.cpp:434-496), computed by the query
        path's G-shift and wedge-search kernel; ``threads`` is accepted for
        compatibility."""
        Q = np.asarray(Q, dtype=np.float64)
        rec = self._move(Q, True, "Moving points into irreducible zone failed.")
        W = np.asarray(self.pointgroup.W, dtype=np.int32)
        shape = Q.shape[:-1] + (3, 3)
        return (rec["q_ir"].reshape(Q.shape), rec["tau"].reshape(Q.shape), W[rec["rot"][:, 0]].reshape(shape),
                W[rec["rot"][:, 1]].reshape(shape))

    @property
    def ir_volume(self):
        from scipy.spatial import ConvexHull
        return ConvexHull(self.ir_vertices_invA).volume
