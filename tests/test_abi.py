"""The C ABI: the library builds for sm_103a, loads, and exports every entry
point include/*.h declares; the ctypes mirror matches the C struct layout.
No GPU needed (nothing here launches a kernel)."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", text, flags=re.M):
            if m.group(1) not in ("if", "while", "sizeof"):
                names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from landslidehysea_gb300 import build as B
    from landslidehysea_gb300 import solver
    B.build()
    return solver.load()


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("lsh_create", "lsh_step", "lsh_set_state", "lsh_get_state", "shallowWater", "comprobarSoporteCUDA",
              "lsh_load_datadat", "lsh_nc_create", "lsh_step_noalloc"):
        assert n in names, n


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_mirror_covers_header():
    from landslidehysea_gb300 import io, solver
    missing = [n for n in declared_functions() if n not in solver.SIGNATURES and n not in io.SIGNATURES]
    assert not missing, missing


def test_params_layout_matches_c(tmp_path):
    from landslidehysea_gb300._abi import LshParams
    fields = [f for f, _ in LshParams._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lsh.h"\nint main(void){\n'
                   'printf("%zu\\n", sizeof(lsh_params));\n' +
                   "".join(f'printf("%zu\\n", offsetof(lsh_params, {f}));\n' for f in fields) + "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(LshParams)
    for f, off in zip(fields, out[1:]):
        assert getattr(LshParams, f).offset == off, f


def test_defaults_match_c(lib):
    from landslidehysea_gb300._abi import LshParams, default_params
    p = LshParams()
    assert lib.lsh_params_default(ctypes.byref(p)) == 0
    q = default_params()
    for f, _ in LshParams._fields_:
        assert getattr(p, f) == getattr(q, f), f


def test_status_strings(lib):
    for s in range(10):
        assert lib.lsh_status_string(s)
