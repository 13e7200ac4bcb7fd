"""Shared test configuration.

Markers: `gpu` tests need a CUDA device and the built libgbmv.so; everything else runs on CPU.
The oracle (oracle/oracle.c, built on first use) is the checker; golden fixtures under
tests/golden were produced by the reference's own code (tests/golden/make_golden.py).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sundials-manyvector-demo_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
TABLES = os.path.join(GOLDEN, "primordial_tables.h5")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libgbmv.so")


def maxnorm_err(a, b):
    """max |a-b| / max |b| over one field (the per-field max-normalised error), NaN-aware:
    NaN positions must coincide."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return np.inf
    m = ~nb
    if not m.any():
        return 0.0
    scale = np.max(np.abs(b[m]))
    d = np.max(np.abs(a[m] - b[m]))
    if scale == 0.0:
        return float(d)
    return float(d / scale)


@pytest.fixture(scope="session")
def tables():
    import h5tables
    return h5tables.load_table_block(TABLES)


@pytest.fixture(scope="session")
def golden_feuler():
    return np.load(os.path.join(GOLDEN, "feuler_cases.npz"))


@pytest.fixture(scope="session")
def golden_chem():
    return np.load(os.path.join(GOLDEN, "chem_cases.npz"))


def feuler_case_names(g):
    return sorted({k.split("/")[0] for k in g.files})


def case_fields(g, name):
    nchem = int(g[f"{name}/nchem"])
    nf = 5 + (1 if nchem else 0)
    w = [g[f"{name}/w{i}"] for i in range(nf)]
    return w, nchem, tuple(int(x) for x in g[f"{name}/bc"]), float(g[f"{name}/gamma"]), \
        g[f"{name}/force"]


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gbmv
    lib = os.path.join(PKG, "_build", "libgbmv.so")
    if not os.path.exists(lib):
        import build_lib
        build_lib.build()
    gbmv.load()
    return torch
