"""The C-ABI library builds, loads and exports what include/brx.h declares;
host-side validation rejects malformed geometry without touching a GPU."""
import ctypes as C
import os
import re
import subprocess

import numpy as np

from brille_gb300 import _abi
from brille_gb300._lib import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "brx.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(brx_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_declared_symbol():
    lib = load()
    names = declared_functions()
    assert "brx_ir_interpolate_at" in names and "brx_create" in names
    for n in names:
        assert hasattr(lib, n), n
    assert lib.brx_abi_version() == 1


def test_struct_layout_matches_header(tmp_path):
    """ctypes mirrors of brx_geometry / brx_data / brx_locate_out have the C
    sizes and field offsets."""
    fields = {"brx_geometry": _abi.Geometry, "brx_data": _abi.Data, "brx_locate_out": _abi.LocateOut,
              "brx_mlp_dims": _abi.MlpDims, "brx_sort_cost": _abi.SortCost, "brx_trellis_in": _abi.TrellisIn,
              "brx_trellis_cells": _abi.TrellisCells}
    src = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, py in fields.items():
        src.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            src.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    src.append("return 0;}")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(c), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.split() for line in out if line)
    for cname, py in fields.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(py, f).offset, f


def test_create_rejects_bad_geometry():
    """brx_create validates indices on the host before any CUDA call."""
    from _cases import crystal_case
    c = crystal_case("diamond2")
    t = dict(c["tables"])
    tv = np.array(t["tet_vertices"], copy=True)
    tv[0, 0] = 10 ** 6  # out of range
    t["tet_vertices"] = tv
    holder = _abi.GeometryHolder(t)
    h = C.c_void_p()
    st = load().brx_create(C.byref(holder.struct), 0, C.byref(h))
    assert st == 1 and not h.value
    st = load().brx_create(None, 0, C.byref(h))
    assert st == 1


def test_header_is_strict_c(tmp_path):
    """include/brx.h compiles as strict C99 and C++17 with every warning an
    error, and a C program links against libbrx.so and calls it (no GPU
    work: the ABI version and a rejected geometry)."""
    from brille_gb300._lib import LIB_PATH

    load()
    src = tmp_path / "consumer.c"
    src.write_text(f"""#include "{HEADER}"
#include <stdio.h>
int main(void) {{
  brx_handle* h = 0;
  brx_status st = brx_create(0, 0, &h);
  printf("%d %d\\n", (int)brx_abi_version(), (int)st);
  return st == BRX_ERR_INVALID_ARGUMENT && h == 0 ? 0 : 1;
}}
""")
    exe = tmp_path / "consumer"
    lib_dir = os.path.dirname(LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", str(src), "-o", str(exe),
                    "-L" + lib_dir, "-lbrx", "-Wl,-rpath," + lib_dir], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert out == ["1", "1"]
    cpp = tmp_path / "consumer.cpp"
    cpp.write_text(f'#include "{HEADER}"\nint main() {{ return brx_abi_version() == BRX_ABI_VERSION ? 0 : 1; }}\n')
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only", str(cpp)],
                   check=True)


def _cube_polyhedron(n_planes=6):
    """The unit cube [0,1]^3 as brx_trellis_in arrays (vertices, unit
    outward planes n.x + d <= 0 inside, edges); extra planes repeat the
    first face."""
    v = np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], float)
    planes = [[-1, 0, 0, 0], [1, 0, 0, -1], [0, -1, 0, 0], [0, 1, 0, -1], [0, 0, -1, 0], [0, 0, 1, -1]]
    planes = np.array((planes * (n_planes // 6 + 1))[:n_planes], float)
    edges = np.array([[i, j] for i in range(8) for j in range(i + 1, 8)
                      if np.abs(v[i] - v[j]).sum() == 1], np.int32)
    return v, planes, edges


def _trellis_in(v, planes, edges, knots, tol=1e-12):
    dp = C.POINTER(C.c_double)
    t = _abi.TrellisIn()
    t.n_vertices, t.vertices = len(v), v.ctypes.data_as(dp)
    t.n_planes, t.planes = len(planes), planes.ctypes.data_as(dp)
    t.n_edges, t.edges = len(edges), edges.ctypes.data_as(C.POINTER(C.c_int32))
    for d in range(3):
        t.n_knots[d], t.knots[d] = len(knots[d]), knots[d].ctypes.data_as(dp)
    t.tol = tol
    return t


def test_trellis_build_rejects_bad_input_on_the_host():
    """brx_trellis_cells_build checks its input before any CUDA call:
    missing arrays, out-of-range edges, unsorted knots and a negative
    tolerance are invalid arguments; more planes than the kernels hold is
    unsupported; the output struct is cleared either way."""
    lib = load()
    v, planes, edges = _cube_polyhedron()
    k = np.linspace(0, 1, 5)
    knots = [k, k.copy(), k.copy()]
    out = _abi.TrellisCells()
    bad_edges = edges.copy()
    bad_edges[0, 1] = 8
    unsorted = [k, k[::-1].copy(), k.copy()]
    cases = [
        (_trellis_in(v, planes, bad_edges, knots), 1),
        (_trellis_in(v, planes, edges, unsorted), 1),
        (_trellis_in(v, planes, edges, knots, tol=-1.0), 1),
        (_trellis_in(v, planes[:3], edges, knots), 1),
    ]
    many_v, many_p, many_e = _cube_polyhedron(65)
    cases.append((_trellis_in(many_v, many_p, many_e, knots), 8))  # BRX_ERR_UNSUPPORTED
    for tin, want in cases:
        out.n_nodes = 7
        assert lib.brx_trellis_cells_build(C.byref(tin), 0, C.byref(out)) == want
        assert out.n_nodes == 0 and not out.node_type
    assert lib.brx_trellis_cells_build(None, 0, C.byref(out)) == 1
    lib.brx_trellis_cells_free(C.byref(out))
    lib.brx_trellis_cells_free(None)

