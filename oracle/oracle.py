"""ctypes wrapper of the CPU oracle (brx_oracle.c).  TEST INFRASTRUCTURE.

Only the tests, the smoke check and the CPU-baseline leg of bench.py use this
module; the product (brille_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from brille_gb300._abi import GeometryHolder, make_data

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build(force=False):
    """Compile the oracle with gcc (-ffp-contract=off keeps FP64 operation
    order identical on x86-64 and aarch64)."""
    src = os.path.join(HERE, "brx_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB + ".tmp", src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class OrcPerm(C.Structure):
    _fields_ = [("n_keys", C.c_int64), ("keys", C.POINTER(C.c_int64)), ("ids", C.POINTER(C.c_int32)),
                ("n_perms", C.c_int32), ("n_branches", C.c_int32), ("perms", C.POINTER(C.c_int32))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.orc_move.restype = C.c_int
        _lib.orc_move_locate.restype = C.c_int
        _lib.orc_locate.restype = C.c_int
        _lib.orc_interpolate_at.restype = C.c_int
        _lib.orc_rotate.restype = C.c_int
        _lib.orc_max_threads.restype = C.c_int
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p()


class Oracle:
    """The oracle bound to one geometry (dict of tables)."""

    def __init__(self, tables):
        self.holder = GeometryHolder(tables)
        self.g = C.byref(self.holder.struct)
        self.t = tables

    def move(self, Q, ir=True):
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, 3)
        n = Q.shape[0]
        q = np.zeros((n, 3))
        tau = np.zeros((n, 3), np.int32)
        rot = np.zeros((n, 2), np.int32)
        st = np.zeros(n, np.int32)
        lib().orc_move(self.g, _p(Q), C.c_int64(n), C.c_int(int(ir)), _p(q), _p(tau), _p(rot), _p(st))
        return q, tau, rot, st

    def move_locate(self, Q, ir=True, no_move=False):
        """Every intermediate index of move + locate, as brx_locate returns them."""
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, 3)
        n = Q.shape[0]
        out = dict(q_ir=np.zeros((n, 3)), tau=np.zeros((n, 3), np.int32), rot=np.zeros((n, 2), np.int32),
                   node=np.zeros((n, 2), np.int32), n_weights=np.zeros(n, np.int32),
                   vertex=np.zeros((n, 8), np.int32), weight=np.zeros((n, 8)), status=np.zeros(n, np.int32))
        lib().orc_move_locate(self.g, _p(Q), C.c_int64(n), C.c_int(int(ir)), C.c_int(int(no_move)),
                              _p(out["q_ir"]), _p(out["tau"]), _p(out["rot"]), _p(out["node"]),
                              _p(out["n_weights"]), _p(out["vertex"]), _p(out["weight"]), _p(out["status"]))
        return out

    def locate(self, xyz, threads=0):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = xyz.shape[0]
        node = np.zeros((n, 2), np.int32)
        nw = np.zeros(n, np.int32)
        vi = np.full((n, 8), -1, np.int32)
        w = np.zeros((n, 8))
        st = np.zeros(n, np.int32)
        lib().orc_locate(self.g, _p(xyz), C.c_int64(n), _p(node), _p(nw), _p(vi), _p(w), _p(st), C.c_int(threads))
        return node, nw, vi, w, st

    def interpolate_at(self, Q, values, vectors=None, ir=True, no_move=False, threads=0,
                       perm=None):
        """values/vectors: (array (V,B,span), elements[3], rotates_like, length_unit)."""
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, 3)
        n = Q.shape[0]
        vd, va = make_data(values[0], values[0].shape[1], values[1], values[2], values[3])
        outs = []
        vo = np.zeros((n,) + va.shape[1:], dtype=va.dtype)
        if vectors is not None:
            cd, ca = make_data(vectors[0], vectors[0].shape[1], vectors[1], vectors[2], vectors[3])
            co = np.zeros((n,) + ca.shape[1:], dtype=ca.dtype)
            cptr = C.byref(cd)
        else:
            cd, ca, co, cptr = None, None, None, None
        st = np.zeros(n, np.int32)
        pp = None
        if perm is not None:
            keys, ids, perms = perm
            keys = np.ascontiguousarray(keys, np.int64)
            ids = np.ascontiguousarray(ids, np.int32)
            perms = np.ascontiguousarray(perms, np.int32)
            pstruct = OrcPerm(keys.size, keys.ctypes.data_as(C.POINTER(C.c_int64)),
                              ids.ctypes.data_as(C.POINTER(C.c_int32)), perms.shape[0], perms.shape[1],
                              perms.ctypes.data_as(C.POINTER(C.c_int32)))
            pp = C.byref(pstruct)
        rc = lib().orc_interpolate_at(self.g, C.byref(vd), cptr, pp, _p(Q), C.c_int64(n), C.c_int(int(ir)),
                                      C.c_int(int(no_move)), _p(vo), _p(co) if co is not None else C.c_void_p(),
                                      _p(st), C.c_int(threads))
        return vo, co, rc, st

    @staticmethod
    def max_threads():
        return lib().orc_max_threads()


class OrcSortSide(C.Structure):
    _fields_ = [("data", C.c_void_p), ("cplx", C.c_int32), ("s", C.c_int32), ("e0", C.c_int32), ("e1", C.c_int32),
                ("e2", C.c_int32), ("vf", C.c_int32), ("phase", C.c_int32), ("w", C.c_double * 3)]


def sort_permutations(values, vectors, keys, threads=0, return_costs=False):
    """sort() on the CPU: per key the permutation of the modes (row → column
    for i < j, column → row for the reverse key), as brx_sort computes it.

    values / vectors: (array (V, B, span) float64 or complex128, elements[3],
    vector cost function, weights[3]); vectors may be None.  Returns perm
    (n_keys × B int32) and, with return_costs, the cost matrices of the keys
    with i < j (n_keys × B × B, zero elsewhere)."""
    keys = np.ascontiguousarray(keys, np.int64)
    sides, keep = [], []
    for k, spec in enumerate((values, vectors)):
        if spec is None:
            continue
        arr, el, vf, w = spec
        arr = np.ascontiguousarray(arr)
        cplx = np.iscomplexobj(arr)
        arr = np.ascontiguousarray(arr, np.complex128 if cplx else np.float64)
        keep.append(arr)
        s = OrcSortSide()
        s.data = arr.ctypes.data
        s.cplx = int(cplx)
        s.e0, s.e1, s.e2 = (int(x) for x in el)
        s.s = s.e0 + s.e1 + s.e2
        s.vf = int(vf)
        s.phase = int(k == 1)
        s.w[:] = [float(x) for x in w]
        sides.append(s)
    V, B = keep[0].shape[0], keep[0].shape[1]
    arr_t = OrcSortSide * len(sides)
    sa = arr_t(*sides)
    perm = np.zeros((keys.size, B), np.int32)
    costs = np.zeros((keys.size, B, B)) if return_costs else None
    rc = lib().orc_sort(sa, C.c_int(len(sides)), C.c_int(B), C.c_int64(V), C.c_int64(keys.size),
                        C.c_void_p(keys.ctypes.data), C.c_void_p(perm.ctypes.data),
                        C.c_void_p(costs.ctypes.data) if costs is not None else C.c_void_p(), C.c_int(threads))
    if rc:
        raise RuntimeError(f"orc_sort failed with status {rc}")
    return (perm, costs) if return_costs else perm


def assign(cost):
    """Exact assignment of a square cost matrix: col_of_row[r] for each row."""
    cost = np.ascontiguousarray(cost, np.float64)
    n = cost.shape[0]
    p = np.zeros(n, np.int32)
    rc = lib().orc_assign(C.c_void_p(cost.ctypes.data), C.c_int(n), C.c_void_p(p.ctypes.data))
    if rc:
        raise RuntimeError("no finite assignment")
    out = np.empty(n, np.int64)
    out[p - 1] = np.arange(n)
    return out
