"""Seeded synthetic crystals and queries for the benchmark workloads.

No public dataset exists for this path; these stand in for it with the
shapes and value distributions the workloads specify.

* ``diamond_primitive``: Fd-3m, a = 4.96 Å, the two-atom basis (0,0,0),
  (¼,¼,¼) described in its primitive cell (6 modes).
* ``diamond_conventional``: the same crystal in its conventional cell with the
  eight-atom basis (24 modes).
* ``hexagonal16``: P6₃/mmc, a = 3.2 Å, c = 5.2 Å, sixteen atoms as Wyckoff
  orbits 2a + 2b + 12k with seeded free parameters (x, z), separations
  ≥ 1.2 Å, one seeded mass in [10, 100] amu per orbit (48 modes).
* ``random_crystal``: one of P-1, P2/m, Pmmm, P4/mmm, R-3m, P6/mmm, Fm-3m,
  Im-3m with seeded lattice parameters and symmetric atom orbits.
"""
from __future__ import annotations

import numpy as np

from .bvk import BvKModel
from .bz import BrillouinZone
from .crystal import Basis, Lattice, Symmetry, LATTICE_SYSTEM, min_separation, orbit, spacegroup


def diamond_conventional(a=4.96, mass=28.0):
    sym = spacegroup("Fd-3m")
    pos = orbit(sym, [0, 0, 0])
    lat = Lattice(((a, a, a), (90, 90, 90)), symmetry=sym, basis=Basis(pos, np.zeros(len(pos), int)))
    return lat, np.full(len(pos), mass)


def diamond_primitive(a=4.96, mass=28.0):
    """Fd-3m with the two-atom basis in the primitive cell.  The conventional
    operations are carried into the primitive basis (W_p = P⁻¹ W P,
    w_p = P⁻¹ w) and reduced modulo primitive translations."""
    conv = spacegroup("Fd-3m")
    P = np.array([[0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
    Pi = np.linalg.inv(P)
    A = a * P.T  # rows: primitive vectors a(0,½,½), a(½,0,½), a(½,½,0)
    Ws, ws, seen = [], [], set()
    for W, w in zip(conv.W, conv.w):
        Wp = np.rint(Pi @ W @ P).astype(int)
        wp = (Pi @ w) % 1.0
        wp[np.isclose(wp, 1.0)] = 0.0
        key = (tuple(Wp.ravel()), tuple(np.round(wp * 48).astype(int) % 48))
        if key in seen:
            continue
        seen.add(key)
        Ws.append(Wp)
        ws.append(wp)
    sym = Symmetry(np.array(Ws), np.array(ws))
    pos = np.array([[0, 0, 0], [0.25, 0.25, 0.25]])
    lat = Lattice(A, symmetry=sym, basis=Basis(pos, [0, 0]))
    return lat, np.full(2, mass)


def hexagonal16(seed=0, a=3.2, c=5.2, min_sep=1.2):
    rng = np.random.default_rng(seed)
    sym = spacegroup("P6_3/mmc")
    A = Lattice(((a, a, c), (90, 90, 120))).A
    for _ in range(10000):
        x, z = rng.uniform(0.18, 0.215), rng.uniform(0.10, 0.15)
        orbits = [orbit(sym, [0, 0, 0]), orbit(sym, [0, 0, 0.25]), orbit(sym, [x, 2 * x, z])]
        if [len(o) for o in orbits] != [2, 2, 12]:
            continue
        pos = np.concatenate(orbits)
        if min_separation(A, pos) >= min_sep:
            break
    else:
        raise RuntimeError("no admissible 16-atom arrangement found")
    types = np.concatenate([np.full(len(o), i) for i, o in enumerate(orbits)])
    masses_per = rng.uniform(10, 100, size=len(orbits))
    lat = Lattice(((a, a, c), (90, 90, 120)), symmetry=sym, basis=Basis(pos, types))
    return lat, masses_per[types]


def random_crystal(name, n_orbits, seed=0, min_sep=1.0, max_atoms=32):
    """A crystal of space group `name` with seeded lattice parameters
    (3–8 Å, free angles 60–120°) and up to `n_orbits` symmetric atom orbits
    (at least one), at most `max_atoms` atoms in all."""
    rng = np.random.default_rng(seed)
    sym = spacegroup(name)
    system = LATTICE_SYSTEM[name]
    special = np.array([0.0, 0.5, 0.25, 0.75, 1 / 3, 2 / 3])
    for _ in range(500):
        a, b, c = rng.uniform(3, 8, 3)
        al = be = ga = 90.0
        if system == "triclinic":
            al, be, ga = rng.uniform(60, 120, 3)
        elif system == "monoclinic":
            be = rng.uniform(60, 120)
        elif system == "tetragonal":
            b = a
        elif system == "hexagonal":
            b, ga = a, 120.0
        elif system == "cubic":
            b = c = a
        try:
            lat0 = Lattice(((a, b, c), (al, be, ga)), symmetry=sym)
        except ValueError:
            continue
        orbits = [orbit(sym, [0, 0, 0])]
        for _t in range(20 * n_orbits):
            if len(orbits) >= n_orbits:
                break
            p = np.where(rng.uniform(size=3) < 0.6, special[rng.integers(0, len(special), 3)], rng.uniform(0, 1, 3))
            o = orbit(sym, p)
            if sum(len(x) for x in orbits) + len(o) > max_atoms:
                continue
            if min_separation(lat0.A, np.concatenate(orbits + [o])) < min_sep:
                continue
            orbits.append(o)
        pos = np.concatenate(orbits)
        if min_separation(lat0.A, pos) < min_sep:
            continue
        types = np.concatenate([np.full(len(o), t) for t, o in enumerate(orbits)])
        masses = rng.uniform(10, 100, len(orbits))[types]
        return Lattice(lat0.A, symmetry=sym, basis=Basis(pos, types)), masses
    raise RuntimeError("no admissible crystal found")


def uniform_q(n, lo=-1.0, hi=1.0, seed=0):
    return np.random.default_rng(seed).uniform(lo, hi, size=(n, 3))


def grid_for(lat, max_volume_fraction, masses=None, time_reversal=False):
    """BrillouinZone plus trellis with max node volume = |BZ| · fraction."""
    from .trellis import TrellisBuild

    bz = BrillouinZone(lat, time_reversal=time_reversal)
    tr = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, bz.volume * max_volume_fraction)
    return bz, tr


def bvk_for(lat, masses):
    return BvKModel(lat, masses, cutoff=6.0, decay=1.5)


def near_boundary_q(bz, tr, n, delta=1e-6, seed=0):
    """q within `delta` r.l.u. of trellis faces (tetrahedron faces and knot
    planes) and of high-symmetry lines (edges of the irreducible polyhedron),
    carried to random symmetry images and zones so that every stage meets
    them."""
    from .trellis import _poly_edges

    rng = np.random.default_rng(seed)
    lat = bz.lattice
    Binv = np.linalg.inv(lat.B)
    parts = []
    k = n // 3
    # tetrahedron faces
    t = tr.tet_vertices[rng.integers(0, len(tr.tet_vertices), k)]
    bc = rng.dirichlet([1, 1, 1], size=k)
    parts.append(np.einsum("nk,nkd->nd", bc, tr.vertices[t[:, :3]]))
    # knot planes inside cube nodes
    cv = tr.cube_vertices[rng.integers(0, max(len(tr.cube_vertices), 1), k)] if len(tr.cube_vertices) else None
    if cv is not None:
        lo, hi = tr.vertices[cv[:, 0]], tr.vertices[cv[:, 7]]
        x = lo + rng.uniform(size=(k, 3)) * (hi - lo)
        axis = rng.integers(0, 3, k)
        x[np.arange(k), axis] = np.where(rng.uniform(size=(k, 1)) < 0.5, lo, hi)[np.arange(k), axis]
        parts.append(x)
    # edges of the irreducible polyhedron (high-symmetry lines)
    edges = _poly_edges(bz.ir_vertices_invA, bz.ir_halfspaces, 1e-9 * np.abs(bz.ir_vertices_invA).max())
    m = n - sum(len(p) for p in parts)
    e = edges[rng.integers(0, len(edges), m)]
    s = rng.uniform(size=(m, 1))
    parts.append(bz.ir_vertices_invA[e[:, 0]] * (1 - s) + bz.ir_vertices_invA[e[:, 1]] * s)
    q = np.concatenate(parts) @ Binv
    q += rng.uniform(-delta, delta, size=q.shape)
    W = bz.pointgroup.W[rng.integers(0, bz.pointgroup.size, len(q))]
    q = np.einsum("nji,nj->ni", W, q)
    P = lat.inv_P().T  # conventional components of primitive translations
    G = rng.integers(-2, 3, size=(len(q), 3)) @ P.T
    return q + G
