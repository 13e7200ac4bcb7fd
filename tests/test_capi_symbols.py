"""The C-ABI library builds, loads and exports every entry point include/gbmv.h declares
(CPU: no compute calls)."""
import ctypes
import os
import re

import pytest

from conftest import PKG, ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "gbmv.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbmv_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_path():
    syms = declared_symbols()
    for s in ("gbmv_feuler", "gbmv_feuler_async", "gbmv_chem_rhs", "gbmv_chem_jac",
              "gbmv_block_lu_factor", "gbmv_block_lu_solve", "gbmv_fexpl"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    import build_lib
    lib = build_lib.build()
    L = ctypes.CDLL(lib)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_python_mirror_binds_every_symbol():
    import gbmv
    bound = {n for n, _, _ in gbmv.SIGNATURES}
    assert set(declared_symbols()) <= bound, set(declared_symbols()) - bound


def test_no_cpu_fallback_without_library(tmp_path):
    import gbmv
    with pytest.raises(gbmv.GbmvError):
        gbmv._lib = None
        gbmv.load(str(tmp_path / "missing.so"))
