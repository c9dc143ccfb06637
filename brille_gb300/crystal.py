"""Host-side crystal description: lattice, space-group operations, basis.

This is set-up code for the GPU query path, not part of it.  It produces the
integer rotation matrices, primitive transforms and Gamma-table inputs that
`brille_gb300.trellis` flattens into the tables the CUDA kernels read.

Conventions follow the reference's public Python surface:

* a direct lattice is given by its basis vectors (rows, Cartesian Å) or by
  ``((a, b, c), (alpha, beta, gamma))`` with ``a`` along x and ``b`` in the
  xy-plane;
* reciprocal basis vectors are the rows of ``B = 2π (A⁻¹)ᵀ`` so that
  ``Q_xyz = Q_hkl @ B`` (reference ``src/lattice_dual.hpp``);
* space-group operations ``(W, w)`` act on fractional direct coordinates,
  ``x' = W x + w`` (reference ``src/symmetry.hpp``);
* the point group is the list of distinct ``W`` in order of first appearance;
  its matrices act on reciprocal vectors through their transposes,
  ``q' = Wᵀ q`` (reference ``src/bz_move.cpp:257-285``).
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np

TWO_PI = 2.0 * np.pi

# Primitive transforms (a_p, b_p, c_p) = (a, b, c) P for each lattice centring,
# stored as 6P so that every entry is an integer.  These are the standard
# crystallographic choices; the reference holds the same table in
# ``src/primitive.hpp:103-115``.
_SIX_P = {
    "P": np.diag([6, 6, 6]),
    "I": np.array([[-3, 3, 3], [3, -3, 3], [3, 3, -3]]),
    "F": np.array([[0, 3, 3], [3, 0, 3], [3, 3, 0]]),
    "A": np.array([[6, 0, 0], [0, 3, -3], [0, 3, 3]]),
    "B": np.array([[3, 0, -3], [0, 6, 0], [3, 0, 3]]),
    "C": np.array([[3, 3, 0], [-3, 3, 0], [0, 0, 6]]),
    "R": np.array([[4, -2, -2], [2, 2, -4], [2, 2, 2]]),
}


def _lattice_matrix(lengths, angles_deg):
    a, b, c = lengths
    al, be, ga = np.radians(angles_deg)
    ax = np.array([a, 0.0, 0.0])
    bx = np.array([b * np.cos(ga), b * np.sin(ga), 0.0])
    cx = c * np.cos(be)
    cy = c * (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    cz = np.sqrt(max(c * c - cx * cx - cy * cy, 0.0))
    return np.array([ax, bx, [cx, cy, cz]])


def _wrap(t):
    """Reduce fractional translations into [0, 1) with a stable tie at 1."""
    t = np.asarray(t, dtype=float) % 1.0
    t[np.isclose(t, 1.0, atol=1e-9)] = 0.0
    t[np.isclose(t, 0.0, atol=1e-9)] = 0.0
    return t


@dataclass
class Symmetry:
    """Space-group operations ``x' = W x + w`` in the conventional cell."""

    W: np.ndarray  # (n, 3, 3) int
    w: np.ndarray  # (n, 3) float

    def __post_init__(self):
        self.W = np.asarray(self.W, dtype=np.int32).reshape(-1, 3, 3)
        self.w = np.asarray(self.w, dtype=float).reshape(-1, 3)
        if self.W.shape[0] != self.w.shape[0]:
            raise ValueError("W and w must hold the same number of operations")

    @classmethod
    def from_generators(cls, generators, centring="P"):
        """Close a generator set under composition (translations mod 1)."""
        ops = [(np.eye(3, dtype=np.int64), np.zeros(3))]
        cent = centring_vectors(centring)
        for t in cent[1:]:
            ops.append((np.eye(3, dtype=np.int64), np.array(t, dtype=float)))
        gens = [(np.asarray(W, dtype=np.int64), _wrap(w)) for W, w in generators]
        ops += gens

        def key(W, w):
            return (tuple(W.ravel()), tuple(np.round(_wrap(w) * 48).astype(int)))

        seen = {}
        for W, w in ops:
            seen.setdefault(key(W, w), (W, _wrap(w)))
        frontier = list(seen.values())
        while frontier:
            new = []
            for W1, w1 in frontier:
                for W2, w2 in list(seen.values()):
                    for Wa, wa, Wb, wb in ((W1, w1, W2, w2), (W2, w2, W1, w1)):
                        W3 = Wa @ Wb
                        w3 = _wrap(Wa @ wb + wa)
                        k = key(W3, w3)
                        if k not in seen:
                            seen[k] = (W3, w3)
                            new.append((W3, w3))
            frontier = new
            if len(seen) > 1000:
                raise RuntimeError("generator closure exceeded 1000 operations")
        items = list(seen.values())
        # identity first, then the centring translations, then the rest in
        # a deterministic order (rotation part, then translation)
        def order(op):
            W, w = op
            return (not np.array_equal(W, np.eye(3)), tuple(W.ravel()), tuple(w))
        items.sort(key=order)
        return cls(np.array([W for W, _ in items]), np.array([w for _, w in items]))

    @property
    def size(self):
        return self.W.shape[0]

    def pointgroup(self) -> "PointSymmetry":
        mats = []
        for W in self.W:
            if not any(np.array_equal(W, m) for m in mats):
                mats.append(W.copy())
        return PointSymmetry(np.array(mats))

    def has_space_inversion(self):
        return any(np.array_equal(W, -np.eye(3)) for W in self.W)

    def add_space_inversion(self) -> "Symmetry":
        if self.has_space_inversion():
            return self
        W = np.concatenate([self.W, -self.W])
        w = np.concatenate([self.w, self.w])
        return Symmetry(W, w)

    def centring(self):
        pure = [tuple(np.round(t, 6)) for W, t in zip(self.W, self.w)
                if np.array_equal(W, np.eye(3)) and np.any(np.abs(t) > 1e-9)]
        for name in ("I", "F", "A", "B", "C", "R"):
            want = [tuple(np.round(v, 6)) for v in centring_vectors(name)[1:]]
            if all(any(np.allclose(v, p, atol=1e-6) for p in pure) for v in want) and len(pure) == len(want):
                return name
        return "P"


def centring_vectors(name):
    h = 0.5
    table = {
        "P": [(0, 0, 0)],
        "I": [(0, 0, 0), (h, h, h)],
        "F": [(0, 0, 0), (0, h, h), (h, 0, h), (h, h, 0)],
        "A": [(0, 0, 0), (0, h, h)],
        "B": [(0, 0, 0), (h, 0, h)],
        "C": [(0, 0, 0), (h, h, 0)],
        "R": [(0, 0, 0), (2 / 3, 1 / 3, 1 / 3), (1 / 3, 2 / 3, 2 / 3)],
    }
    return [np.array(v, dtype=float) for v in table[name]]


@dataclass
class PointSymmetry:
    """Distinct rotation parts of a space group (direct-lattice integers)."""

    W: np.ndarray

    def __post_init__(self):
        self.W = np.asarray(self.W, dtype=np.int32).reshape(-1, 3, 3)

    @property
    def size(self):
        return self.W.shape[0]

    def find_identity_index(self):
        for i, W in enumerate(self.W):
            if np.array_equal(W, np.eye(3)):
                return i
        raise RuntimeError("point group has no identity")

    def inverse_indices(self):
        inv = np.full(self.size, -1, dtype=np.int32)
        for i, W in enumerate(self.W):
            Wi = np.rint(np.linalg.inv(W)).astype(np.int32)
            for j, V in enumerate(self.W):
                if np.array_equal(V, Wi):
                    inv[i] = j
                    break
            if inv[i] < 0:
                raise RuntimeError("point group is not closed under inversion")
        return inv

    def add_space_inversion(self):
        if any(np.array_equal(W, -np.eye(3)) for W in self.W):
            return self
        return PointSymmetry(np.concatenate([self.W, -self.W]))


@dataclass
class Basis:
    """Atom positions (fractional, conventional cell) and integer types."""

    positions: np.ndarray
    types: np.ndarray = None

    def __post_init__(self):
        self.positions = np.asarray(self.positions, dtype=float).reshape(-1, 3)
        if self.types is None:
            self.types = np.arange(self.positions.shape[0])
        self.types = np.asarray(self.types, dtype=np.int64).ravel()

    @property
    def size(self):
        return self.positions.shape[0]

    def equivalent_to(self, t, pos, tol=1e-6):
        """Index of the atom of type t at pos modulo lattice translations."""
        for l in range(self.size):
            if self.types[l] != t:
                continue
            d = self.positions[l] - pos
            d -= np.rint(d)
            if np.all(np.abs(d) < tol):
                return l
        return -1


class Lattice:
    """A direct lattice with optional symmetry and basis.

    ``Lattice(A)`` with A a 3×3 matrix of basis vectors as rows, or
    ``Lattice(((a, b, c), (alpha, beta, gamma)))``.
    """

    def __init__(self, vectors, symmetry: Symmetry | None = None, basis: Basis | None = None, *,
                 spacegroup=None, real_space=True, row_vectors=True):
        """Also the reference's Python forms (brille/lattice.py:10-120):
        ``values`` as (lengths, angles) — angles in radians when none
        exceeds π, else degrees — or basis vectors (``row_vectors``);
        ``spacegroup`` by name (str) as the second positional argument or
        by keyword; ``symmetry`` as (rotations, translations) and ``basis``
        as (positions, types) tuples; ``real_space=False`` for reciprocal
        lattice parameters (Å⁻¹)."""
        if isinstance(symmetry, str):
            spacegroup, symmetry = symmetry, None
        if spacegroup is not None:
            if symmetry is not None:
                raise ValueError("give either a spacegroup or a symmetry, not both")
            symmetry = spacegroup_by_name(spacegroup)
        if symmetry is not None and not isinstance(symmetry, Symmetry):
            W, w = symmetry
            symmetry = Symmetry(np.asarray(W, dtype=np.int32).reshape(-1, 3, 3), np.asarray(w, float).reshape(-1, 3))
        if basis is not None and not isinstance(basis, Basis):
            basis = Basis(*basis) if isinstance(basis, (tuple, list)) and len(basis) == 2 else Basis(basis)
        arr = vectors
        if isinstance(arr, (tuple, list)) and len(arr) == 1:
            arr = arr[0]
        if isinstance(arr, (tuple, list)) and len(arr) == 2 and np.size(arr[0]) == 3 and np.size(arr[1]) == 3:
            angles = np.asarray(arr[1], dtype=float)
            if not (angles > np.pi).any():
                angles = np.degrees(angles)
            A = _lattice_matrix(arr[0], angles)
        else:
            A = np.asarray(arr, dtype=float).reshape(3, 3)
            if not row_vectors:
                A = A.T
        if not real_space:
            A = TWO_PI * np.linalg.inv(A).T  # the given rows are the reciprocal basis
        self.A = A
        self.B = TWO_PI * np.linalg.inv(A).T
        if symmetry is None:
            symmetry = Symmetry(np.eye(3, dtype=np.int32)[None], np.zeros((1, 3)))
        self.symmetry = symmetry
        if basis is None:
            basis = Basis(np.zeros((1, 3)), np.zeros(1))
        self.basis = basis
        self._check_symmetry()

    def _check_symmetry(self):
        G = self.A @ self.A.T
        for W in self.symmetry.W:
            if not np.allclose(W.T @ G @ W, G, rtol=1e-8, atol=1e-8):
                raise ValueError("a symmetry operation does not preserve the lattice metric")

    @property
    def pointgroup(self) -> PointSymmetry:
        return self.symmetry.pointgroup()

    @property
    def centring(self):
        return self.symmetry.centring()

    def six_P(self):
        return _SIX_P[self.centring].astype(np.int32)

    def inv_P(self):
        P = self.six_P() / 6.0
        return np.rint(np.linalg.inv(P)).astype(np.int32)

    def primitive_B(self):
        """Rows of the primitive reciprocal basis: B_p = P⁻¹ B, so that a
        conventional (h,k,l) and its primitive components q_p = Pᵀ q give the
        same Cartesian vector."""
        return self.inv_P() @ self.B

    def has_space_inversion(self):
        return self.symmetry.has_space_inversion()


# --------------------------------------------------------------------------
# Named space groups used by the synthetic workloads.  Generators are given in
# the standard (International Tables) settings as (W, w) pairs acting on
# fractional coordinates; closure is done by Symmetry.from_generators.
# --------------------------------------------------------------------------
_I3 = np.eye(3, dtype=int)
_INV = -_I3
_2X = np.diag([1, -1, -1])
_2Y = np.diag([-1, 1, -1])
_2Z = np.diag([-1, -1, 1])
_4Z = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]])
_3D = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]])          # (z, x, y)
_3Z = np.array([[0, -1, 0], [1, -1, 0], [0, 0, 1]])        # hexagonal (-y, x-y, z)
_6Z = np.array([[1, -1, 0], [1, 0, 0], [0, 0, 1]])         # hexagonal (x-y, x, z)
_2XY = np.array([[0, 1, 0], [1, 0, 0], [0, 0, -1]])        # (y, x, -z)
_Z = np.zeros(3)
_Q = 0.25

SPACEGROUPS = {
    "P-1": ([(_INV, _Z)], "P"),
    "P2/m": ([(_2Y, _Z), (_INV, _Z)], "P"),
    "Pmmm": ([(_2Z, _Z), (_2Y, _Z), (_INV, _Z)], "P"),
    "P4/mmm": ([(_4Z, _Z), (_2Y, _Z), (_INV, _Z)], "P"),
    "R-3m": ([(_3Z, _Z), (_2XY, _Z), (_INV, _Z)], "R"),
    "P6/mmm": ([(_6Z, _Z), (_2XY, _Z), (_INV, _Z)], "P"),
    "P6_3/mmc": ([(_6Z, np.array([0, 0, 0.5])), (_2XY, _Z), (_INV, _Z)], "P"),
    "Fm-3m": ([(_4Z, _Z), (_3D, _Z), (_INV, _Z)], "F"),
    "Im-3m": ([(_4Z, _Z), (_3D, _Z), (_INV, _Z)], "I"),
    # origin choice 1: 4-fold screw and inversion carry a (1/4,1/4,1/4) shift
    "Fd-3m": ([(_4Z, np.array([_Q, _Q, _Q])), (_2X, _Z), (_3D, _Z),
               (_INV, np.array([_Q, _Q, _Q]))], "F"),
}

# crystal-system constraints on the free lattice parameters of each group
LATTICE_SYSTEM = {
    "P-1": "triclinic", "P2/m": "monoclinic", "Pmmm": "orthorhombic",
    "P4/mmm": "tetragonal", "R-3m": "hexagonal", "P6/mmm": "hexagonal",
    "P6_3/mmc": "hexagonal", "Fm-3m": "cubic", "Im-3m": "cubic", "Fd-3m": "cubic",
}


def spacegroup_by_name(name) -> Symmetry:
    """A space group of the table below by its International Tables name
    (spaces and underscores ignored); "P1" is the identity alone."""
    key = str(name).replace(" ", "")
    if key in ("P1", "1"):
        return Symmetry(np.eye(3, dtype=np.int32)[None], np.zeros((1, 3)))
    for k in SPACEGROUPS:
        if k.replace("_", "") == key.replace("_", ""):
            return spacegroup(k)
    raise ValueError(f"space group {name!r} is not in this package's table ({', '.join(sorted(SPACEGROUPS))}, P1); "
                     "give the symmetry operations instead")


def spacegroup(name) -> Symmetry:
    gens, cent = SPACEGROUPS[name]
    return Symmetry.from_generators(gens, cent)


def orbit(sym: Symmetry, x, tol=1e-6):
    """Distinct images of fractional point x under the space group, in [0,1)."""
    pts = []
    for W, w in zip(sym.W, sym.w):
        p = _wrap(W @ np.asarray(x, float) + w)
        if not any(np.all(np.abs(((p - q) + 0.5) % 1.0 - 0.5) < tol) for q in pts):
            pts.append(p)
    return np.array(pts)


def min_separation(A, positions):
    """Smallest interatomic distance (Å) including periodic images."""
    pos = np.asarray(positions, float)
    best = np.inf
    shifts = np.array(list(itertools.product((-1, 0, 1), repeat=3)), float)
    for i in range(len(pos)):
        d = pos[None, :, :] - pos[i][None, None, :] + shifts[:, None, :]
        r = np.linalg.norm(d @ A, axis=-1)
        r[13, i] = np.inf
        best = min(best, r.min())
    return best
