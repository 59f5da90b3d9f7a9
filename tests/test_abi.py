"""The C-ABI library builds, loads without a GPU and exports every entry point that
include/rbffd.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(rbf_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    pkg = g.load_package()
    path = pkg.build_library()
    return ctypes.CDLL(path), pkg


def test_every_declared_symbol_is_exported(lib):
    L, pkg = lib
    names = _declared()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/ but not exported"


def test_python_binding_covers_header(lib):
    L, pkg = lib
    assert set(_declared()) <= set(pkg._native.SIGNATURES)


def test_struct_layouts_match_header(lib):
    """ctypes mirrors of the C structs have the C sizes (checked with the host compiler)."""
    import subprocess
    import tempfile
    _, pkg = lib
    src = r'''
#include <stdio.h>
#include "rbffd.h"
int main(void){printf("%zu %zu %zu %zu\n", sizeof(rbf_build_cfg), sizeof(rbf_hermite), sizeof(rbf_build_stats),
                      sizeof(rbf_csr));return 0;}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        sizes = list(map(int, subprocess.run([exe], capture_output=True, text=True).stdout.split()))
    n = pkg._native
    assert sizes == [ctypes.sizeof(n.BuildCfg), ctypes.sizeof(n.Hermite), ctypes.sizeof(n.BuildStats),
                     ctypes.sizeof(n.Csr)]


def test_version_without_gpu(lib):
    L, pkg = lib
    L.rbf_version.restype = ctypes.c_char_p
    assert b"sm_103a" in L.rbf_version()


def test_package_front_end_without_gpu(lib):
    _, pkg = lib
    import numpy as np
    assert pkg.autoselect_k(np.zeros((50, 2)), pkg.PHS(3, poly_deg=2)) == 12
    assert pkg.autoselect_k(np.zeros((50, 2)), pkg.PHS(3, poly_deg=1)) == 6
    assert pkg.autoselect_k(np.zeros((50, 2)), pkg.PHS(3, poly_deg=0)) == 5
    assert pkg.autoselect_k(np.zeros((5, 2)), pkg.PHS(3, poly_deg=2)) == 5
    assert repr(pkg.PHS(5, poly_deg=0)) == "Polyharmonic spline (r⁵)\n└─Polynomial augmentation: degree 0"
    with pytest.raises(ValueError):
        pkg.PHS(2, poly_deg=-1)
    with pytest.raises(ValueError):
        pkg.Partial(3, 1)
    assert pkg.Dirichlet().is_dirichlet() and pkg.Neumann().is_neumann() and pkg.Robin(0.5, 0.5).is_robin()
