"""BZTrellisQdd / BZTrellisQdc / BZTrellisQcc on one GB300.

Mirrors the reference's pybind11 grid surface (wrap/_trellis.hpp:27-101,
wrap/_common_grid.hpp:21-440): construction from a BrillouinZone and a
maximum node volume, ``fill``, ``ir_interpolate_at`` and ``interpolate_at``
with the same argument meaning, output shapes and error messages
(raised as RuntimeError).  Queries run through libbrx.so (the C ABI in
include/brx.h); ``useparallel``/``threads`` are accepted for compatibility
and have no effect on the GPU.

Additions, all keyword-only: ``storage`` on fill ("f64" as given, "f32",
"bf16" for the vertex data kept on the device) and ``out_f32`` on the queries
(float32 / complex64 results).
"""
from __future__ import annotations

import ctypes as C
from enum import IntEnum

import numpy as np

from . import _abi
from ._lib import BrxError, check, load
from .bz import BrillouinZone
from .tables import geometry_tables
from .trellis import TrellisBuild

_STORAGE = {"f64": _abi.BRX_STORE_F64, "f32": _abi.BRX_STORE_F32, "bf16": _abi.BRX_STORE_BF16}


def _elements(arr, el):
    """Decode an elements vector and the data shape as the reference's
    fill_check / Interpolator::check_elements do (wrap/_interpolator.hpp:13-110,
    src/interpolator.hpp:547-586).  Returns (B, [scalars, vector elems,
    matrix elems], rotates_like, length_unit)."""
    el = np.asarray(el).astype(np.int64).ravel()
    e = [int(el[i]) if i < el.size else 0 for i in range(3)]
    rot = int(el[3]) if el.size > 3 else 0
    lu = int(el[4]) if el.size > 4 else 3
    if rot not in (0, 1, 2):
        raise RuntimeError(f"Unknown RotatesLike value {rot}")
    if lu not in (0, 1, 2, 3, 4):
        raise RuntimeError(f"Unknown LengthUnit value {lu}")
    shape = arr.shape
    x = sum(e)
    if arr.ndim == 1:
        if x == 0:
            e[0] = x = 1
        if x > 1:
            raise RuntimeError("1-D data must represent one scalar per point!")
        B = 1
    elif arr.ndim == 2:
        if x == 0:
            e[0] = x = shape[1]
        if shape[1] % x:
            raise RuntimeError("2-D data requires an integer number of branches!")
        B = shape[1] // x
    elif arr.ndim == 3:
        if x == 0:
            e[0] = x = shape[2]
        if shape[2] != x:
            raise RuntimeError("3-D data requires that the last dimension matches the specified number of elements!")
        B = shape[1]
    elif arr.ndim == 4:
        if shape[3] != 3:
            raise RuntimeError("4-D data can only be 3-vectors")
        if x == 0:
            e[1] = x = shape[2] * 3
        if shape[2] * 3 != x:
            raise RuntimeError("4-D data requires that the last two dimensions match the specified number of vector elements!")
        B = shape[1]
    elif arr.ndim == 5:
        if shape[3] != 3 or shape[4] != 3:
            raise RuntimeError("5-D data can only be matrices")
        if x == 0:
            e[2] = x = shape[2] * 9
        if shape[2] * 9 != x:
            raise RuntimeError("5-D data requires the last three dimensions match the specified number of matrix elements!")
        B = shape[1]
    else:
        raise RuntimeError("Interpolator data is expected to be 1- to 5-D")
    return B, e, rot, lu


_FILL_NAMES = ("values_data", "values_elements", "values_weights", "vectors_data", "vectors_elements",
               "vectors_weights", "sort")


def _fill_arguments(args, kwargs):
    """The arguments of fill() by name.  Positional forms, as the reference
    binds them: (values, elements), (values, elements, vectors, elements
    [, sort]) and (values, elements, weights, vectors, elements, weights
    [, sort]); keywords fill in or replace nothing twice."""
    n = len(args)
    if n in (0, 1, 2):
        names = _FILL_NAMES[:n]
    elif n in (3, 4, 5):
        names = ("values_data", "values_elements", "vectors_data", "vectors_elements", "sort")[:n]
    elif n in (6, 7):
        names = _FILL_NAMES[:n]
    else:
        raise TypeError("fill() takes at most 7 positional arguments")
    if n == 3:
        raise TypeError("fill() needs the vectors' elements with the vectors")
    out = dict(zip(names, args))
    for k, v in kwargs.items():
        if k not in _FILL_NAMES:
            raise TypeError(f"fill() got an unexpected keyword argument '{k}'")
        if k in out:
            raise TypeError(f"fill() got multiple values for argument '{k}'")
        out[k] = v
    if "values_data" not in out or "values_elements" not in out:
        raise TypeError("fill() needs values_data and values_elements")
    if ("vectors_data" in out) != ("vectors_elements" in out):
        raise TypeError("fill() needs vectors_data and vectors_elements together")
    out.setdefault("values_weights", (1.0, 1.0, 1.0))
    out.setdefault("vectors_weights", (1.0, 1.0, 1.0))
    out.setdefault("vectors_data", None)
    out.setdefault("vectors_elements", None)
    out["sort"] = bool(out.get("sort", False))
    return out


def _cost_fns(el):
    """(scalar, vector) cost-function codes of an elements vector: entries 5
    and 6, default 0 (wrap/_interpolator.hpp:95-98)."""
    el = np.asarray(el).astype(np.int64).ravel()
    return (int(el[5]) if el.size > 5 else 0, int(el[6]) if el.size > 6 else 0)


class NodeType(IntEnum):
    """Trellis node types with the reference's names and values
    (src/enums.hpp:43, wrap/_enums.cpp:41-48); the tables store them as
    BRX_NODE_NULL / CUBE / POLY (include/brx.h), see ``node_type``."""
    assumed_null = 0
    found_null = 1
    null = 2
    cube = 3
    polygon = 4
    poly = 4


class RotatesLike(IntEnum):
    """How vector data transform (src/rotates.hpp:27); the codes of fill's
    elements[3]."""
    vector = 0
    pseudovector = 1
    Gamma = 2


class LengthUnit(IntEnum):
    """Units of vector data (src/enums.hpp:37); the codes of fill's
    elements[4]."""
    none = 0
    angstrom = 1
    inverse_angstrom = 2
    real_lattice = 3
    reciprocal_lattice = 4


def node_type(table_code):
    """NodeType of a node-table code (BRX_NODE_NULL, _CUBE, _POLY)."""
    return (NodeType.null, NodeType.cube, NodeType.polygon)[int(table_code)]


def table_from_moved(keys, moved, perms, n_branches):
    """(keys, perm_ids, perms) for brx_set_permutations from sorted keys, a
    mask of the keys whose permutation is not the identity and those
    permutations in key order: id 0 is the identity, the moved keys take
    ids 1, 2, … in order."""
    keys = np.ascontiguousarray(keys, np.int64)
    moved = np.asarray(moved, bool)
    perms = np.asarray(perms, np.int32).reshape(-1, n_branches)
    if moved.shape != keys.shape or int(moved.sum()) != len(perms):
        raise ValueError("the mask and the permutations do not match the keys")
    ids = np.zeros(len(keys), np.int32)
    ids[moved] = np.arange(1, len(perms) + 1, dtype=np.int32)
    table = np.concatenate([np.arange(n_branches, dtype=np.int32)[None, :], perms])
    return keys, ids, table


def _is_device(x):
    return hasattr(x, "data_ptr") and bool(getattr(x, "is_cuda", False))


def _as_data(x, dt):
    """numpy arrays are converted to the grid's dtype on the host; CUDA
    tensors stay on the device (float32/complex64 or float64/complex128) and
    are converted by brx_fill."""
    if _is_device(x):
        import torch

        want_cplx = np.dtype(dt).kind == "c"
        if x.is_complex() != want_cplx:
            x = x.to(torch.complex128 if want_cplx else torch.float64)
        if x.dtype not in (torch.float64, torch.complex128, torch.float32, torch.complex64):
            x = x.to(torch.float64)
        return x.contiguous()
    return np.ascontiguousarray(np.asarray(x), dtype=dt)


def _make_data(arr, nv, B, e, rot, lu):
    if not _is_device(arr):
        return _abi.make_data(arr.reshape(nv, -1), B, e, rot, lu)
    import torch

    codes = {torch.float64: _abi.BRX_F64, torch.complex128: _abi.BRX_C128, torch.float32: _abi.BRX_F32,
             torch.complex64: _abi.BRX_C64}
    d = _abi.Data()
    d.data = arr.data_ptr()
    d.dtype = codes[arr.dtype]
    d.n_branches = int(B)
    d.elements[:] = [int(x) for x in e]
    d.rotates_like = int(rot)
    d.length_unit = int(lu)
    return d, arr


def _ptr(obj):
    """Address of a numpy array or of an object with data_ptr() (torch)."""
    if obj is None:
        return None
    if hasattr(obj, "data_ptr"):
        return obj.data_ptr()
    return obj.ctypes.data


class _Grid:
    VALUE_COMPLEX = False
    VECTOR_COMPLEX = True

    def __init__(self, bz: BrillouinZone, node_volume_fraction=0.1, always_triangulate=False, approx_config=None, *,
                 max_volume=None, trellis=None, device=0, float_tolerance=None, digit=None,
                 trellis_backend="host"):
        """(wrap/_trellis.hpp:36-38) The reference's ``node_volume_fraction``
        is handed to its PolyTrellis as the maximum node volume in Å⁻³
        (src/trellis_poly.hpp:148-160), and so it is here; ``max_volume`` is
        the same number under its own name and wins when given.  Tolerances:
        ``approx_config`` (an ApproxConfig), else the zone's, else the global
        configuration (brille_gb300.approx); ``float_tolerance`` / ``digit``
        override them.  ``trellis_backend="gpu"`` builds the trellis on the
        grid's device (brx_trellis_cells_build: cells classified and cut
        polytopes split into tetrahedra by kernels), "host" on the host."""
        from . import approx

        cfg = approx_config or getattr(bz, "approx_config", None) or approx.config
        float_tolerance = cfg.reciprocal_space_tolerance if float_tolerance is None else float_tolerance
        digit = cfg.digits if digit is None else digit
        if trellis is None:
            vol = float(node_volume_fraction if max_volume is None else max_volume)
            if not vol > 0:
                raise ValueError("the maximum node volume must be positive")
            trellis = TrellisBuild(bz.ir_vertices_invA, bz.ir_halfspaces, vol, always_triangulate,
                                   backend=trellis_backend, device=device)
        self.bz = bz
        self.trellis = trellis
        self.tables = geometry_tables(bz, trellis, gamma=True, float_tolerance=float_tolerance, digit=digit)
        self._geom = _abi.GeometryHolder(self.tables)
        self.device = device
        self._h = None
        self._fill = None

    # ------------------------------------------------------------ accessors
    @property
    def invA(self):
        return self.trellis.vertices.copy()

    @property
    def rlu(self):
        return self.trellis.vertices @ np.linalg.inv(self.bz.lattice.B)

    @property
    def vertices(self):
        return self.rlu

    @property
    def tetrahedra(self):
        return self.trellis.tet_vertices.copy()

    @property
    def BrillouinZone(self):
        return self.bz

    def _rlu(self, xyz):
        return xyz @ np.linalg.inv(self.bz.lattice.B)

    @property
    def inner_invA(self):
        """Vertices of the cube nodes (wrap/_trellis.hpp:45-47)."""
        idx = np.unique(self.trellis.cube_vertices)
        return self.trellis.vertices[idx]

    @property
    def outer_invA(self):
        """Vertices of the poly nodes' tetrahedra (wrap/_trellis.hpp:48-50)."""
        idx = np.unique(self.trellis.tet_vertices)
        return self.trellis.vertices[idx]

    @property
    def inner_rlu(self):
        return self._rlu(self.inner_invA)

    @property
    def outer_rlu(self):
        return self._rlu(self.outer_invA)

    def all_node_types(self):
        """Type of every node in linear order i + nx(j + ny k)
        (wrap/_trellis.hpp:96-98)."""
        return [node_type(t) for t in self.trellis.node_type]

    def node_at_type(self, subscript):
        """Type of the node at subscript (i, j, k) (wrap/_trellis.hpp:84-86)."""
        nx, ny, nz = self.trellis.shape
        i, j, k = (int(x) for x in subscript)
        if not (0 <= i < nx and 0 <= j < ny and 0 <= k < nz):
            raise IndexError(f"node subscript {subscript} outside {self.trellis.shape}")
        return node_type(self.trellis.node_type[i + nx * (j + ny * k)])

    def node_containing_type(self, Q):
        """Type of the node whose cell holds each Q (r.l.u., not moved), as
        the query's locate finds it (wrap/_trellis.hpp:88-94); NodeType.null
        where no node holds Q."""
        rec = self.locate(np.asarray(Q, dtype=np.float64).reshape(-1, 3), ir=False, do_not_move_points=True)
        node = rec["node"][:, 0]
        out = []
        for n in node:
            out.append(node_type(self.trellis.node_type[n]) if n >= 0 else NodeType.null)
        return out

    @property
    def values(self):
        return None if self._fill is None else self._fill["values"]

    @property
    def vectors(self):
        return None if self._fill is None else self._fill["vectors"]

    # --------------------------------------------------------------- handle
    def _handle(self):
        if self._h is None:
            lib = load()
            h = C.c_void_p()
            st = lib.brx_create(C.byref(self._geom.struct), self.device, C.byref(h))
            if st != 0:
                raise BrxError(st, f"brx_create failed with status {st}")
            self._h = h
        return self._h

    def __del__(self):
        try:
            if self._h is not None:
                load().brx_destroy(self._h)
        except Exception:
            pass

    # ----------------------------------------------------------------- fill
    def fill(self, *args, storage="f64", **kwargs):
        """fill(values_data, values_elements[, values_weights], vectors_data,
        vectors_elements[, vectors_weights][, sort]), positionally or by the
        reference's keyword names (wrap/_common_grid.hpp:26-47, 127-147); the
        vectors may be left out for values-only data."""
        a = _fill_arguments(args, kwargs)
        values, values_elements, values_weights = a["values_data"], a["values_elements"], a["values_weights"]
        vectors, vectors_elements, vectors_weights = a["vectors_data"], a["vectors_elements"], a["vectors_weights"]
        sort = a["sort"]
        vdt = np.complex128 if self.VALUE_COMPLEX else np.float64
        cdt = np.complex128 if self.VECTOR_COMPLEX else np.float64
        vals = _as_data(values, vdt)
        nv = self.trellis.vertices.shape[0]
        if vals.shape[0] != nv:
            raise RuntimeError(f"Provided {vals.shape[0]} arrays but {nv} were expected!")
        Bv, ev, rv, lv = _elements(vals, values_elements)
        vd, vkeep = _make_data(vals, nv, Bv, ev, rv, lv)
        cd = ckeep = None
        Bc = ev_c = None
        vecs = None
        if vectors is not None:
            vecs = _as_data(vectors, cdt)
            if vecs.shape[0] != nv:
                raise RuntimeError(f"Provided {vecs.shape[0]} arrays but {nv} were expected!")
            Bc, ev_c, rc, lc = _elements(vecs, vectors_elements)
            if Bc != Bv:
                raise RuntimeError("The values and vectors must have matching number of points and branches")
            cd, ckeep = _make_data(vecs, nv, Bc, ev_c, rc, lc)
        h = self._handle()
        st = load().brx_fill(h, C.byref(vd), C.byref(cd) if cd is not None else None, _STORAGE[storage])
        check(st, h)
        self._fill = dict(values=vals, vectors=vecs,
                          vshape=tuple(vals.shape[1:]), cshape=None if vecs is None else tuple(vecs.shape[1:]),
                          vdtype=vdt, cdtype=cdt, values_weights=values_weights, vectors_weights=vectors_weights,
                          storage=storage, B=Bv, values_fns=_cost_fns(values_elements),
                          vectors_fns=None if vecs is None else _cost_fns(vectors_elements))
        if sort:
            self.sort()
        return True

    def set_flags_weights(self, values_flags, values_weights, vectors_flags, vectors_weights, sort=False):
        """Cost functions and relative cost weights of the values and vectors
        (wrap/_common_grid.hpp:481-560; flags [RotatesLike, LengthUnit,
        scalar cost function, vector cost function], decoded as set_check,
        wrap/_interpolator.cpp:43-81), then sort() when asked."""
        if self._fill is None:
            raise RuntimeError("The interpolation data must be filled before setting cost information.")
        f = self._fill
        for name, flags, weights in (("values", values_flags, values_weights), ("vectors", vectors_flags,
                                                                                 vectors_weights)):
            fl = np.asarray(flags).astype(np.int64).ravel()
            if fl.size > 0 and int(fl[0]) not in (0, 1, 2):
                raise RuntimeError(f"Unknown RotatesLike value {int(fl[0])}")
            if fl.size > 1 and int(fl[1]) not in (0, 1, 2, 3, 4):
                raise RuntimeError(f"Unknown LengthUnit value {int(fl[1])}")
            fns = (int(fl[2]) if fl.size > 2 else 0, int(fl[3]) if fl.size > 3 else 0)
            w = [1.0, 1.0, 1.0]
            for i, x in enumerate(np.asarray(weights, dtype=np.float64).ravel()[:3]):
                w[i] = float(x)
            if name == "values" or f["vectors"] is not None:
                f[name + "_fns"] = fns
                f[name + "_weights"] = tuple(w)
        if sort:
            self.sort()

    def permutation_keys(self):
        """The vertex pairs sort() visits (keys i*n_vertices+j, sorted)."""
        if getattr(self, "_perm_keys", None) is None:
            self._perm_keys = self.trellis.permutation_keys()
        return self._perm_keys

    def sort(self, *, stream=None):
        """Find the mode permutation between every pair of vertices that share
        a node, on the GPU (DualInterpolator::sort,
        src/interpolatordual.hpp:398-434), and use it in every later query."""
        if self._fill is None:
            raise RuntimeError("The interpolation data must be filled before sorting.")
        f = self._fill
        keys = self.permutation_keys()

        def cost(fns, weights):
            c = _abi.SortCost()
            c.scalar_fn, c.vector_fn = int(fns[0]), int(fns[1])
            w = [1.0, 1.0, 1.0]
            for i, x in enumerate(np.asarray(weights, dtype=np.float64).ravel()[:3]):
                w[i] = float(x)
            c.weight[:] = w
            return c

        vc = cost(f["values_fns"], f["values_weights"])
        cc = cost(f["vectors_fns"], f["vectors_weights"]) if f["vectors"] is not None else None
        h = self._handle()
        check(load().brx_sort(h, keys.size, keys.ctypes.data, C.byref(vc), C.byref(cc) if cc is not None else None,
                              stream), h)

    def save_permutations(self, path):
        """Write the permutation table to an .npz file: the keys, and the
        permutations of the keys that are not the identity (the reference
        keeps its table in the grid's HDF5 file, src/permutation_table.hpp)."""
        keys, perms = self.permutation_table()
        moved = (perms != np.arange(perms.shape[1], dtype=perms.dtype)).any(axis=1) if len(keys) else np.zeros(0, bool)
        np.savez(path, keys=keys, moved=moved, perms=perms[moved], n_vertices=len(self.trellis.vertices),
                 n_branches=int(self._fill["B"]))

    def load_permutations(self, path):
        """Read a table written by save_permutations into this grid (filled
        with data of the same vertex and mode counts)."""
        if self._fill is None:
            raise RuntimeError("The interpolation data must be filled before setting permutations.")
        d = np.load(path)
        if int(d["n_vertices"]) != len(self.trellis.vertices) or int(d["n_branches"]) != int(self._fill["B"]):
            raise ValueError(f"{path}: the table belongs to a grid of {int(d['n_vertices'])} vertices and "
                             f"{int(d['n_branches'])} modes")
        keys, ids, table = table_from_moved(d["keys"], d["moved"], d["perms"], int(d["n_branches"]))
        self.set_permutations(keys, ids, table)

    def permutation_table(self):
        """(keys, perms): every key i*n_vertices+j the handle holds and its
        permutation of the modes (perms[k][b] is the mode of vertex j that
        mode b of vertex i pairs with; identity where none is set)."""
        h = self._handle()
        n = int(load().brx_permutation_count(h))
        B = int(self._fill["B"]) if self._fill is not None else 0
        keys = np.zeros(n, np.int64)
        perms = np.zeros((n, B), np.int32)
        check(load().brx_get_permutations(h, n, keys.ctypes.data, perms.ctypes.data), h)
        return keys, perms

    def set_permutations(self, keys, perm_ids, perms):
        """Mode permutations per vertex pair (keys i*n_vertices+j, sorted)."""
        keys = np.ascontiguousarray(keys, np.int64)
        ids = np.ascontiguousarray(perm_ids, np.int32)
        perms = np.ascontiguousarray(perms, np.int32)
        h = self._handle()
        check(load().brx_set_permutations(h, keys.size, keys.ctypes.data, ids.ctypes.data,
                                          perms.shape[0] if perms.ndim == 2 else 0, perms.ctypes.data), h)

    # -------------------------------------------------------------- queries
    def _query(self, ir, Q, do_not_move_points=False, out_f32=False):
        if self._fill is None:
            raise RuntimeError("The interpolation data must be filled before interpolating.")
        Q = np.ascontiguousarray(np.asarray(Q, dtype=np.float64))
        if Q.ndim != 2 or Q.shape[1] != 3:
            raise RuntimeError("Only (n,3) two-dimensional Q vectors supported in interpolating.")
        n = Q.shape[0]
        f = self._fill
        vdt = np.complex64 if (out_f32 and f["vdtype"] == np.complex128) else (np.float32 if out_f32 else f["vdtype"])
        cdt = np.complex64 if (out_f32 and f["cdtype"] == np.complex128) else (np.float32 if out_f32 else f["cdtype"])
        vals = np.empty((n,) + tuple(f["vshape"]), dtype=vdt)
        vecs = np.empty((n,) + tuple(f["cshape"]), dtype=cdt) if f["cshape"] is not None else None
        flags = (_abi.BRX_FLAG_NO_MOVE if do_not_move_points else 0) | (_abi.BRX_FLAG_OUT_F32 if out_f32 else 0)
        fn = load().brx_ir_interpolate_at if ir else load().brx_interpolate_at
        h = self._handle()
        st = fn(h, Q.ctypes.data, n, vals.ctypes.data, vecs.ctypes.data if vecs is not None else None, flags, None)
        check(st, h)
        return vals, vecs

    def ir_interpolate_at(self, Q, useparallel=False, threads=-1, do_not_move_points=False, *, out_f32=False):
        """(wrap/_common_grid.hpp:276-300; src/bz_trellis.hpp:155-196)"""
        return self._query(True, Q, do_not_move_points, out_f32)

    def interpolate_at(self, Q, useparallel=False, threads=-1, do_not_move_points=False, *, out_f32=False):
        """(wrap/_common_grid.hpp:412-440; src/bz_trellis.hpp:113-129)"""
        return self._query(False, Q, do_not_move_points, out_f32)

    def set_atoms(self, weights, positions):
        """Atoms of the structure factor: weights c_k = b_k/sqrt(m_k) and
        fractional positions x_k (n × 3) in the lattice of the query's r.l.u."""
        w = np.ascontiguousarray(weights, dtype=np.float64).reshape(-1)
        x = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        if len(w) != len(x):
            raise ValueError("one weight per atom position is needed")
        self._atoms = (w, x)  # keeps the arrays alive for the call
        a = _abi.Atoms(len(w), w.ctypes.data_as(C.POINTER(C.c_double)), x.ctypes.data_as(C.POINTER(C.c_double)))
        h = self._handle()
        check(load().brx_set_atoms(h, C.byref(a)), h)

    def ir_structure_factor(self, Q, *, out_f32=True):
        """(values, S) at Q: the interpolated values and, per q and mode, the
        coherent one-phonon structure factor |Σ_k c_k e^{2πi Q·x_k} (Q_c·e_k)|²
        of the interpolated eigenvectors (float32, n × B), without writing the
        eigenvectors out.  set_atoms first."""
        if self._fill is None:
            raise RuntimeError("The interpolation data must be filled before interpolating.")
        Q = np.ascontiguousarray(np.asarray(Q, dtype=np.float64))
        if Q.ndim != 2 or Q.shape[1] != 3:
            raise RuntimeError("Only (n,3) two-dimensional Q vectors supported in interpolating.")
        n = Q.shape[0]
        f = self._fill
        vdt = np.complex64 if (out_f32 and f["vdtype"] == np.complex128) else (np.float32 if out_f32 else f["vdtype"])
        vals = np.empty((n,) + tuple(f["vshape"]), dtype=vdt)
        sf = np.empty((n, f["cshape"][0]), dtype=np.float32)
        flags = _abi.BRX_FLAG_OUT_F32 if out_f32 else 0
        h = self._handle()
        check(load().brx_ir_structure_factor(h, Q.ctypes.data, n, vals.ctypes.data, sf.ctypes.data, flags, None), h)
        return vals, sf

    def structure_factor_into(self, Q, n, values_out, sf_out, *, out_f32=True, async_=False, stream=None):
        """ir_structure_factor on caller-owned buffers (host or device)."""
        flags = (_abi.BRX_FLAG_OUT_F32 if out_f32 else 0) | (_abi.BRX_FLAG_ASYNC if async_ else 0)
        addr = lambda o: o if isinstance(o, int) else _ptr(o)  # noqa: E731
        h = self._handle()
        check(load().brx_ir_structure_factor(h, addr(Q), int(n), addr(values_out), addr(sf_out), flags, stream), h)

    def query_into(self, Q, n, values_out, vectors_out, *, ir=True, out_f32=False, no_move=False,
                   async_=False, stream=None):
        """Raw query on caller-owned buffers (numpy arrays, torch tensors or
        integer addresses; host or device).  Returns nothing; raises on error.
        async_=True returns at once for device buffers and for page-locked
        host buffers (outputs complete after sync() or an event recorded on
        `stream` behind the call); pageable host buffers make it synchronous."""
        flags = ((_abi.BRX_FLAG_NO_MOVE if no_move else 0) | (_abi.BRX_FLAG_OUT_F32 if out_f32 else 0) |
                 (_abi.BRX_FLAG_ASYNC if async_ else 0))
        fn = load().brx_ir_interpolate_at if ir else load().brx_interpolate_at
        h = self._handle()
        addr = lambda o: o if isinstance(o, int) else _ptr(o)  # noqa: E731
        st = fn(h, addr(Q), int(n), addr(values_out), addr(vectors_out) if vectors_out is not None else None, flags,
                stream)
        check(st, h)

    def sync(self, stream=None):
        h = self._handle()
        check(load().brx_sync(h, stream), h)

    def locate(self, Q, ir=True, do_not_move_points=False):
        """Every intermediate index of the locate stages (for parity checks)."""
        Q = np.ascontiguousarray(np.asarray(Q, dtype=np.float64).reshape(-1, 3))
        n = Q.shape[0]
        out = dict(q_ir=np.zeros((n, 3)), tau=np.zeros((n, 3), np.int32), rot=np.zeros((n, 2), np.int32),
                   node=np.zeros((n, 2), np.int32), n_weights=np.zeros(n, np.int32),
                   vertex=np.zeros((n, 8), np.int32), weight=np.zeros((n, 8)), status=np.zeros(n, np.int32))
        lo = _abi.LocateOut()
        for k, v in out.items():
            setattr(lo, k, v.ctypes.data_as(type(getattr(lo, k))))
        h = self._handle()
        flags = _abi.BRX_FLAG_NO_MOVE if do_not_move_points else 0
        check(load().brx_locate(h, Q.ctypes.data, n, 1 if ir else 0, flags, C.byref(lo), None), h)
        return out

    def profile(self, enable=True):
        h = self._handle()
        check(load().brx_profile(h, 1 if enable else 0), h)

    def stage_times(self):
        """(ms per stage: locate, grouping, values gather, vectors gather;
        q count; number of gather groups)."""
        ms = (C.c_double * 4)()
        q = C.c_int64()
        ng = C.c_int64()
        h = self._handle()
        check(load().brx_stage_times(h, ms, 4, C.byref(q), C.byref(ng)), h)
        return list(ms), int(q.value), int(ng.value)

    def tune(self, Q, *, out_f32=False, reps=2, stream=None, values_out=None, vectors_out=None):
        """Pick the gathers' shared-memory budgets by timing a sample query
        (brx_tune), into the given output buffers or temporary ones; returns
        the chosen shapes (see tuning())."""
        h = self._handle()
        flags = _abi.BRX_FLAG_OUT_F32 if out_f32 else 0
        n = int(Q.shape[0])
        check(load().brx_tune(h, _ptr(Q), n, _ptr(values_out), _ptr(vectors_out), flags, stream, int(reps)), h)
        return self.tuning()

    def tuning(self):
        """(values smem KB, vectors smem KB, q per work descriptor, work
        units per thread, FP32 gather kernel: 0 warp-independent, 1
        CTA-synchronous)."""
        v = (C.c_int32 * 5)()
        h = self._handle()
        check(load().brx_tuning(h, v, 5), h)
        return tuple(int(x) for x in v)

    def set_tuning(self, values):
        """Apply a tuning() tuple (e.g. saved from an earlier tune())."""
        v = (C.c_int32 * 5)(*(int(x) for x in values))
        h = self._handle()
        check(load().brx_set_tuning(h, v, 5), h)

    def launch_count(self):
        return int(load().brx_launch_count(self._handle()))


class BZTrellisQdd(_Grid):
    VALUE_COMPLEX = False
    VECTOR_COMPLEX = False


class BZTrellisQdc(_Grid):
    VALUE_COMPLEX = False
    VECTOR_COMPLEX = True


class BZTrellisQcc(_Grid):
    VALUE_COMPLEX = True
    VECTOR_COMPLEX = True


class _MeshGrid(_Grid):
    """BZMeshQ*: a tetrahedral mesh of the irreducible polyhedron
    (wrap/_mesh.hpp:29-53, src/bz_mesh.hpp:45-140).  ``max_size`` bounds the
    tetrahedron volume in Å⁻³ (−1: the polyhedron's vertices alone),
    ``max_points`` the vertex count; ``num_levels`` is accepted for
    compatibility: the reference's coarser layers only speed its search, which
    the knot grid of the mesh tables does here.  Queries run on the same GPU
    path as the trellis."""

    def __init__(self, bz: BrillouinZone, max_size=-1.0, num_levels=3, max_points=-1, *, mesh=None, device=0,
                 float_tolerance=None, digit=None):
        from .mesh import MeshTrellis

        if mesh is None:
            mesh = MeshTrellis(bz.ir_vertices_invA, float(max_size), int(max_points))
        self.num_levels = int(num_levels)
        super().__init__(bz, trellis=mesh, device=device, float_tolerance=float_tolerance, digit=digit)

    @property
    def tetrahedra(self):
        return self.trellis.mesh_tetrahedra.copy()


class _NestGrid(_Grid):
    """BZNestQ*: the leaves of a nested tetrahedral refinement of the
    irreducible polyhedron (wrap/_nest.hpp:29-72, src/bz_nest.hpp,
    src/nest.hpp:302-320).  The second argument is the maximum leaf volume in
    Å⁻³ (a float) or a number density (an int: the polyhedron's volume over
    it); ``max_branchings`` is accepted for compatibility: the reference's
    tree only speeds its search, which the knot grid of the mesh tables does
    here.  Queries run on the same GPU path as the trellis."""

    def __init__(self, bz: BrillouinZone, max_volume, max_branchings=5, *, mesh=None, device=0,
                 float_tolerance=None, digit=None):
        from .mesh import MeshTrellis

        if isinstance(max_volume, (int, np.integer)) and not isinstance(max_volume, bool):
            if max_volume < 1:
                raise ValueError("the number density must be positive")
            vol = bz.ir_volume / float(max_volume)
        else:
            vol = float(max_volume)
        if mesh is None:
            mesh = MeshTrellis(bz.ir_vertices_invA, vol)
        self.max_branchings = int(max_branchings)
        super().__init__(bz, trellis=mesh, device=device, float_tolerance=float_tolerance, digit=digit)

    @property
    def all_invA(self):
        return self.invA

    @property
    def all_rlu(self):
        return self.rlu

    @property
    def tetrahedra(self):
        return self.trellis.mesh_tetrahedra.copy()

    @property
    def bytes_per_point(self):
        """Bytes of the device tables per vertex (vertex data not counted)."""
        t = self.trellis
        total = (t.vertices.nbytes + t.tet_vertices.nbytes + t.tet_sphere.nbytes + t.tet_volume.nbytes +
                 t.node_type.nbytes + t.node_index.nbytes + t.poly_tet_offset.nbytes)
        return total / max(1, len(t.vertices))


class BZMeshQdd(_MeshGrid):
    VALUE_COMPLEX = False
    VECTOR_COMPLEX = False


class BZMeshQdc(_MeshGrid):
    VALUE_COMPLEX = False
    VECTOR_COMPLEX = True


class BZMeshQcc(_MeshGrid):
    VALUE_COMPLEX = True
    VECTOR_COMPLEX = True


class BZNestQdd(_NestGrid):
    VALUE_COMPLEX = False
    VECTOR_COMPLEX = False


class BZNestQdc(_NestGrid):
    VALUE_COMPLEX = False
    VECTOR_COMPLEX = True


class BZNestQcc(_NestGrid):
    VALUE_COMPLEX = True
    VECTOR_COMPLEX = True
