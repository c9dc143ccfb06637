"""ctypes mirror of include/brx.h and helpers to fill it from numpy arrays."""
from __future__ import annotations

import ctypes as C

import numpy as np

BRX_OK = 0
STATUS_NAMES = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "not filled", 4: "move failed",
    5: "outside irreducible zone", 6: "not found", 7: "null node", 8: "unsupported",
    9: "impossible", 10: "out of memory", 11: "timeout",
}
BRX_F64, BRX_C128, BRX_F32, BRX_C64, BRX_BF16 = 0, 1, 2, 3, 4
BRX_STORE_F64, BRX_STORE_F32, BRX_STORE_BF16 = 0, 1, 2
BRX_FLAG_NO_MOVE, BRX_FLAG_OUT_F32, BRX_FLAG_ASYNC = 0x1, 0x2, 0x4

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)


class Geometry(C.Structure):
    _fields_ = [
        ("outer_B", C.c_double * 9), ("prim_B", C.c_double * 9),
        ("to_prim_6Pt", C.c_int32 * 9), ("from_prim_invPt", C.c_int32 * 9),
        ("is_primitive", C.c_int32),
        ("n_faces", C.c_int32), ("face_abc", _dp), ("face_normal", _dp),
        ("face_tau", _ip), ("face_tau_len", _dp),
        ("n_wedge", C.c_int32), ("wedge_normal", _dp), ("wedge_le_ge", C.c_int32),
        ("n_ops", C.c_int32), ("ops", _ip), ("op_inverse", _ip), ("identity", C.c_int32),
        ("lattice_to_xyz", C.c_double * 9), ("lattice_from_xyz", C.c_double * 9),
        ("n_knots", C.c_int32 * 3), ("knots", _dp * 3),
        ("n_nodes", C.c_int64), ("node_type", _ip), ("node_index", _ip),
        ("n_cube", C.c_int32), ("cube_vertices", _ip),
        ("n_poly", C.c_int32), ("poly_tet_offset", _ip),
        ("n_tets", C.c_int64), ("tet_vertices", _ip), ("tet_sphere", _dp), ("tet_volume", _dp),
        ("n_vertices", C.c_int64), ("vertex_xyz", _dp),
        ("n_atoms", C.c_int32), ("gamma_F0", _ip), ("gamma_vidx", _ip),
        ("n_gamma_vectors", C.c_int32), ("gamma_vectors", _dp),
        ("float_tolerance", C.c_double), ("digit", C.c_int32),
    ]


class Data(C.Structure):
    _fields_ = [
        ("data", C.c_void_p), ("dtype", C.c_int32), ("n_branches", C.c_int32),
        ("elements", C.c_int32 * 3), ("rotates_like", C.c_int32), ("length_unit", C.c_int32),
    ]


class LocateOut(C.Structure):
    _fields_ = [
        ("q_ir", _dp), ("tau", _ip), ("rot", _ip), ("node", _ip), ("n_weights", _ip),
        ("vertex", _ip), ("weight", _dp), ("status", _ip),
    ]


class MlpDims(C.Structure):
    _fields_ = [("d_in", C.c_int32), ("n_out", C.c_int32), ("n_modes", C.c_int32), ("flags", C.c_int32)]


BRX_MLP_FP32 = 0x1


class SortCost(C.Structure):
    _fields_ = [("scalar_fn", C.c_int32), ("vector_fn", C.c_int32), ("weight", C.c_double * 3)]


class TrellisIn(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("vertices", _dp), ("n_planes", C.c_int32), ("planes", _dp),
                ("n_edges", C.c_int32), ("edges", _ip), ("n_knots", C.c_int32 * 3), ("knots", _dp * 3),
                ("tol", C.c_double), ("always_triangulate", C.c_int32)]


class TrellisCells(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("node_type", _ip), ("n_poly", C.c_int64), ("poly_node", _ip),
                ("point_offset", _lp), ("points", _dp), ("tet_offset", _lp), ("tets", _ip)]


class Atoms(C.Structure):
    _fields_ = [("n_atoms", C.c_int32), ("weight", C.POINTER(C.c_double)), ("position", C.POINTER(C.c_double))]


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None and a.size else C.POINTER(ctype)()


class GeometryHolder:
    """Owns contiguous copies of the table arrays and the ctypes struct
    pointing at them.  `tables` is the dict produced by
    brille_gb300.grid.geometry_tables()."""

    def __init__(self, t: dict):
        keep = {}

        def arr(name, dtype):
            a = np.ascontiguousarray(np.asarray(t[name], dtype=dtype))
            keep[name] = a
            return a

        g = Geometry()
        for name in ("outer_B", "prim_B", "lattice_to_xyz", "lattice_from_xyz"):
            getattr(g, name)[:] = np.asarray(t[name], float).ravel().tolist()
        for name in ("to_prim_6Pt", "from_prim_invPt"):
            getattr(g, name)[:] = np.asarray(t[name], np.int32).ravel().tolist()
        g.is_primitive = int(t["is_primitive"])
        fa = arr("face_abc", np.float64)
        g.n_faces = fa.shape[0]
        g.face_abc = _ptr(fa, C.c_double)
        g.face_normal = _ptr(arr("face_normal", np.float64), C.c_double)
        g.face_tau = _ptr(arr("face_tau", np.int32), C.c_int32)
        g.face_tau_len = _ptr(arr("face_tau_len", np.float64), C.c_double)
        wn = arr("wedge_normal", np.float64).reshape(-1, 3)
        keep["wedge_normal"] = wn
        g.n_wedge = wn.shape[0]
        g.wedge_normal = _ptr(wn, C.c_double)
        g.wedge_le_ge = int(t.get("wedge_le_ge", 0))
        ops = arr("ops", np.int32).reshape(-1, 9)
        keep["ops"] = ops
        g.n_ops = ops.shape[0]
        g.ops = _ptr(ops, C.c_int32)
        g.op_inverse = _ptr(arr("op_inverse", np.int32), C.c_int32)
        g.identity = int(t["identity"])
        for d in range(3):
            k = np.ascontiguousarray(np.asarray(t["knots"][d], np.float64))
            keep["knots%d" % d] = k
            g.n_knots[d] = k.size
            g.knots[d] = _ptr(k, C.c_double)
        nt = arr("node_type", np.int32)
        g.n_nodes = nt.size
        g.node_type = _ptr(nt, C.c_int32)
        g.node_index = _ptr(arr("node_index", np.int32), C.c_int32)
        cv = arr("cube_vertices", np.int32).reshape(-1, 8)
        keep["cube_vertices"] = cv
        g.n_cube = cv.shape[0]
        g.cube_vertices = _ptr(cv, C.c_int32)
        po = arr("poly_tet_offset", np.int32)
        g.n_poly = po.size - 1
        g.poly_tet_offset = _ptr(po, C.c_int32)
        tv = arr("tet_vertices", np.int32).reshape(-1, 4)
        keep["tet_vertices"] = tv
        g.n_tets = tv.shape[0]
        g.tet_vertices = _ptr(tv, C.c_int32)
        g.tet_sphere = _ptr(arr("tet_sphere", np.float64), C.c_double)
        g.tet_volume = _ptr(arr("tet_volume", np.float64), C.c_double)
        vx = arr("vertex_xyz", np.float64).reshape(-1, 3)
        keep["vertex_xyz"] = vx
        g.n_vertices = vx.shape[0]
        g.vertex_xyz = _ptr(vx, C.c_double)
        f0 = arr("gamma_F0", np.int32)
        g.n_atoms = int(t["n_atoms"])
        g.gamma_F0 = _ptr(f0, C.c_int32)
        g.gamma_vidx = _ptr(arr("gamma_vidx", np.int32), C.c_int32)
        gv = arr("gamma_vectors", np.float64).reshape(-1, 3)
        keep["gamma_vectors"] = gv
        g.n_gamma_vectors = gv.shape[0]
        g.gamma_vectors = _ptr(gv, C.c_double)
        g.float_tolerance = float(t.get("float_tolerance", 1e-12))
        g.digit = int(t.get("digit", 1000))
        self.struct = g
        self._keep = keep
        self.tables = t


def make_data(array, n_branches, elements, rotates_like, length_unit):
    """A Data struct for a (V, B, span) float64 or complex128 array."""
    a = np.ascontiguousarray(array)
    d = Data()
    if np.iscomplexobj(a):
        a = np.ascontiguousarray(a, dtype=np.complex128)
        d.dtype = BRX_C128
    else:
        a = np.ascontiguousarray(a, dtype=np.float64)
        d.dtype = BRX_F64
    d.data = a.ctypes.data
    d.n_branches = int(n_branches)
    d.elements[:] = [int(x) for x in elements]
    d.rotates_like = int(rotates_like)
    d.length_unit = int(length_unit)
    return d, a
