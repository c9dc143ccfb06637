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
              "brx_mlp_dims": _abi.MlpDims, "brx_sort_cost": _abi.SortCost}
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
