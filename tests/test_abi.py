"""The C ABI library: it loads, exports every function include/isosim.h
declares, and fails cleanly (status code, message) without a GPU."""
import ctypes as C
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "isosim.h")
PKG = os.path.join(ROOT, "isosurface-analysis_gb300")
LIB = os.path.join(PKG, "lib", "libisosim.so")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"ISO_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        subprocess.run([sys.executable, os.path.join(PKG, "build.py")], check=True)
    return C.CDLL(LIB)


def test_header_declares_entry_points():
    names = declared_functions()
    for want in ("iso_ctx_create", "iso_ism", "calculate_histogram_h", "approximate_isosurfaces_h",
                 "iso_marching_cube_h", "iso_generate_hierarchy_h", "iso_select_representatives"):
        assert want in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "isosim.h"\nint main(void){iso_opts o={0,0,0,1,128};(void)o;return 0;}\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-c", str(src),
                        "-o", str(tmp_path / "t.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_host_only_entry_points(lib):
    """Representative selection runs on the host: check it against the oracle."""
    import numpy as np
    import oracle
    sys.path.insert(0, PKG)
    import isosim
    rng = np.random.default_rng(7)
    m = 40
    a = rng.uniform(0, 1, (m, m)).astype(np.float32)
    ism = ((a + a.T) / 2).astype(np.float32)
    np.fill_diagonal(ism, 1.0)
    ids = np.arange(3, 3 + m, dtype=np.int32)
    isos = np.linspace(-1, 1, m + 3).astype(np.float32)
    for cnt in (1, 16, 60):
        assert isosim.select_representatives(ism, ids, isos, cnt) == oracle.select_representatives(ism, ids, isos, cnt)


def test_no_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib.iso_ctx_create.restype = C.c_int
    lib.iso_ctx_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    lib.iso_last_error.restype = C.c_char_p
    h = C.c_void_p()
    rc = lib.iso_ctx_create(0, C.byref(h))
    assert rc < 0
    assert lib.iso_last_error().decode()
