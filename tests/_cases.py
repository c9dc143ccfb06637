"""Shared test cases: tables, vertex data and queries."""
import functools
import os

import numpy as np

from brille_gb300 import workloads as W
from brille_gb300.bz import BrillouinZone
from brille_gb300.crystal import Basis, Lattice, Symmetry
from brille_gb300.tables import geometry_tables
from brille_gb300.trellis import PointTrellis, TrellisBuild

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@functools.lru_cache(None)
def nacl():
    """The reference's Γ-rotation fixture as tables + data.

    The stored grid points are the reference's trellis vertices for NaCl;
    the wedge chosen by this package for m-3m (x ≥ y ≥ z ≥ 0 in r.l.u.) is
    the reference's, and a one-node trellis over the stored points keeps the
    vertex data usable as given."""
    d = dict(np.load(os.path.join(GOLDEN, "nacl_gamma.npz")))
    lat = Lattice(d["basis_vectors"], symmetry=Symmetry(d["spacegroup_mat"], d["spacegroup_vec"]),
                  basis=Basis(d["atom_positions"], d["atom_index"]))
    bz = BrillouinZone(lat)
    tr = PointTrellis(d["grid_rlu"] @ lat.B)
    return d, lat, bz, tr, geometry_tables(bz, tr)


CRYSTALS = {
    "diamond2": W.diamond_primitive,
    "diamond8": W.diamond_conventional,
    "hex16": W.hexagonal16,
}


@functools.lru_cache(None)
def crystal_case(name, fraction=1 / 2000, always_triangulate=False):
    lat, masses = CRYSTALS[name]() if name in CRYSTALS else W.random_crystal(name, 2, seed=3)
    bz = BrillouinZone(lat)
    tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * fraction, always_triangulate)
    t = geometry_tables(bz, tr)
    model = W.bvk_for(lat, masses)
    qv = tr.vertices @ np.linalg.inv(lat.B)
    # large trellises: eigensolves over spawn-started worker processes
    procs = min(16, os.cpu_count() or 1) if len(qv) > 20000 else 0
    w, v = model.modes(qv, processes=procs)
    return dict(lat=lat, bz=bz, tr=tr, tables=t, model=model, w=w, v=v)


def values_vectors(case):
    w, v = case["w"], case["v"]
    nv, B = w.shape
    vals = (np.ascontiguousarray(w[:, :, None]), [1, 0, 0], 0, 3)
    vecs = (np.ascontiguousarray(v.reshape(nv, B, -1)), [0, v.shape[2] * 3, 0], 2, 1)
    return vals, vecs


def boundary_q(case, n, seed=0, delta=1e-6):
    """Points on or within delta r.l.u. of trellis knots, tetrahedron faces,
    wedge planes and zone faces."""
    rng = np.random.default_rng(seed)
    lat, tr, bz = case["lat"], case["tr"], case["bz"]
    Binv = np.linalg.inv(lat.B)
    out = []
    # tetrahedron face points
    if len(tr.tet_vertices):
        t = tr.tet_vertices[rng.integers(0, len(tr.tet_vertices), n // 3)]
        bc = rng.dirichlet([1, 1, 1], size=len(t))
        p = np.einsum("nk,nkd->nd", bc, tr.vertices[t[:, :3]])
        out.append(p @ Binv)
    # trellis vertices and knot planes
    vx = tr.vertices[rng.integers(0, len(tr.vertices), n // 3)]
    out.append(vx @ Binv)
    # zone face points (moved by reciprocal lattice vectors)
    f = rng.integers(0, len(bz.face_abc), n - 2 * (n // 3))
    abc = bz.face_abc[f].reshape(-1, 3, 3)
    bc = rng.dirichlet([1, 1, 1], size=len(f))
    out.append(np.einsum("nk,nkd->nd", bc, abc) @ Binv)
    q = np.concatenate(out)
    q += rng.uniform(-delta, delta, size=q.shape) * (rng.uniform(size=(len(q), 1)) < 0.5)
    return q


def conditioned_modes(case, Q, ir=True, thresh=0.2):
    """(N, B) mask of (q, mode) whose interpolated eigenvector is well
    defined: for every vertex the Hermitian product with the pivot vertex's
    row is at least `thresh` of the product of norms.  Where it is not, the
    reference's antiphase picks a phase from rounding noise and two correct
    implementations can disagree by O(1)."""
    from oracle.oracle import Oracle

    rec = Oracle(case["tables"]).move_locate(Q, ir=ir)
    v = case["v"].reshape(len(case["v"]), case["v"].shape[1], -1)
    N, B = len(Q), v.shape[1]
    ok = np.ones((N, B), bool)
    piv = v[rec["vertex"][:, 0]]
    pn = np.linalg.norm(piv, axis=-1)
    for x in range(1, 8):
        has = rec["n_weights"] > x
        if not has.any():
            continue
        vx = v[rec["vertex"][:, x]]
        z = np.abs(np.einsum("nbe,nbe->nb", np.conj(piv), vx))
        c = z / np.maximum(pn * np.linalg.norm(vx, axis=-1), 1e-300)
        ok &= ~has[:, None] | (c >= thresh)
    return ok & (rec["status"] == 0)[:, None]
