"""Flatten a Brillouin zone, its trellis and the Γ table into query tables.

The dict returned by `geometry_tables` holds exactly the arrays of
`brx_geometry` (include/brx.h).  A caller that keeps the reference's own C++
objects would fill the same struct from them; this module fills it from the
package's host-side builders.
"""
from __future__ import annotations

import numpy as np

from .bz import BrillouinZone
from .crystal import Lattice, PointSymmetry, Symmetry
from .trellis import TrellisBuild


def _approx_equal_zero(d, e_tol, n_tol):
    """approx_float::equal(d, 0, e_tol, e_tol, n_tol) for a 3-vector
    (src/approx_float.hpp:79-100,171-177)."""
    rel = np.finfo(float).eps * n_tol * 10000
    abs_ = 5.0 / 1e15
    if e_tol > rel:
        rel = e_tol
    if e_tol > abs_:
        abs_ = e_tol
    x = np.abs(d)
    return bool(np.all((x <= abs_ + rel * np.abs(d)) | (x < np.finfo(float).tiny)))


def gamma_table(lattice: Lattice, pointgroup: PointSymmetry, time_reversal=False,
                e_tol=1e-12, n_tol=1000):
    """Restates GammaTable::construct (src/phonon.hpp:114-167).

    Returns (F0, vidx, vectors): F0[k, r] = l, the atom that atom k is sent to
    by the first space-group operation whose rotation is point operation r;
    vidx[k, r] indexes `vectors`, whose entries are R⁻¹ r_l − r_k (fractional,
    the inverse motion's translation reduced into [0, 1)), (0,0,0) first.
    """
    sym: Symmetry = lattice.symmetry
    if time_reversal:
        sym = sym.add_space_inversion()
    basis = lattice.basis
    n_atoms, n_ops = basis.size, pointgroup.size
    p2s = []
    for r in range(n_ops):
        hit = [j for j in range(sym.size) if np.array_equal(sym.W[j], pointgroup.W[r])]
        if not hit:
            raise RuntimeError("Something has gone wrong with the correspondence of spacegroup to pointgroup")
        p2s.append(hit[0])
    vectors = [np.zeros(3)]
    F0 = np.zeros((n_atoms, n_ops), np.int32)
    vidx = np.zeros((n_atoms, n_ops), np.int32)
    for k in range(n_atoms):
        rk = basis.positions[k]
        for r in range(n_ops):
            W = sym.W[p2s[r]].astype(float)
            w = sym.w[p2s[r]]
            K = W @ rk + w
            l = -1
            for i in range(n_atoms):
                if basis.types[i] != basis.types[k]:
                    continue
                d = K - basis.positions[i] + 0.5
                d = np.abs(d - np.floor(d)) - 0.5
                if _approx_equal_zero(d, e_tol, n_tol):
                    l = i
                    break
            if l < 0:
                raise RuntimeError("All atoms in the basis *must* be mapped to an equivalent atom for *all* symmetry operations")
            Wi = np.rint(np.linalg.inv(W))
            wi = -(Wi @ w)
            wi = wi - np.floor(wi)
            vec = (Wi @ basis.positions[l] + wi) - rk
            v = len(vectors)
            for i, u in enumerate(vectors):
                if _approx_equal_zero(np.array([np.linalg.norm(u - vec)]), e_tol, n_tol):
                    v = i
                    break
            if v == len(vectors):
                vectors.append(vec)
            F0[k, r] = l
            vidx[k, r] = v
    return F0, vidx, np.array(vectors)


def geometry_tables(bz: BrillouinZone, trellis: TrellisBuild, gamma=True,
                    float_tolerance=1e-12, digit=1000):
    lat = bz.lattice
    pg = bz.pointgroup
    t = {}
    t["outer_B"] = lat.B
    t["prim_B"] = lat.primitive_B()
    t["to_prim_6Pt"] = lat.six_P().T
    t["from_prim_invPt"] = lat.inv_P().T
    t["is_primitive"] = 1 if lat.centring == "P" else 0
    t["face_abc"] = bz.face_abc
    t["face_normal"] = bz.face_normal
    t["face_tau"] = bz.face_tau
    t["face_tau_len"] = bz.face_tau_len
    t["wedge_normal"] = bz.wedge_normal
    t["wedge_le_ge"] = 0
    t["ops"] = pg.W.reshape(-1, 9)
    t["op_inverse"] = pg.inverse_indices()
    t["identity"] = pg.find_identity_index()
    t["lattice_to_xyz"] = lat.A.T
    t["lattice_from_xyz"] = np.linalg.inv(lat.A.T)
    t["knots"] = [np.asarray(k) for k in trellis.knots]
    t["node_type"] = trellis.node_type
    t["node_index"] = trellis.node_index
    t["cube_vertices"] = trellis.cube_vertices
    t["poly_tet_offset"] = trellis.poly_tet_offset
    t["tet_vertices"] = trellis.tet_vertices
    t["tet_sphere"] = trellis.tet_sphere
    t["tet_volume"] = trellis.tet_volume
    t["vertex_xyz"] = trellis.vertices
    if gamma:
        F0, vidx, vec = gamma_table(lat, pg, bz.time_reversal, float_tolerance, digit)
    else:
        F0 = np.zeros((0, pg.size), np.int32)
        vidx = F0
        vec = np.zeros((1, 3))
    t["n_atoms"] = F0.shape[0]
    t["gamma_F0"] = F0
    t["gamma_vidx"] = vidx
    t["gamma_vectors"] = vec
    t["float_tolerance"] = float_tolerance
    t["digit"] = digit
    return t


def save_tables(path, t):
    flat = {k: np.asarray(v) for k, v in t.items() if k != "knots"}
    for d in range(3):
        flat["knots%d" % d] = np.asarray(t["knots"][d])
    np.savez_compressed(path, **flat)


def load_tables(path):
    z = np.load(path)
    t = {k: z[k] for k in z.files if not k.startswith("knots")}
    t["knots"] = [z["knots%d" % d] for d in range(3)]
    for k in ("is_primitive", "wedge_le_ge", "identity", "n_atoms", "digit"):
        t[k] = int(t[k])
    t["float_tolerance"] = float(t["float_tolerance"])
    return t
