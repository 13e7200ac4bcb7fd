"""gbmv_feuler_noalloc: the flux divergence for callers that cannot allocate device memory
(an integrator or application that owns all of HBM through its own pool, or code that must
not trigger the synchronisation an allocation can cause).  It runs the same FP64 kernels as
gbmv_feuler with its scratch in a fixed 64 MiB array inside the library.

Called straight through the C ABI with ctypes; its output must match the handle-based entry
point within the FP64 parity tolerance on two calls in a row (the shared array keeps the
previous call's contents), the shared status word must be cleared between calls, and grids
beyond the array's capacity must be refused.  Kept in a file of its own, collected last.
"""
import ctypes as C

import numpy as np
import pytest

import workloads as W
from conftest import maxnorm_err

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _ptrs(torch_list):
    arr = (C.c_void_p * 6)()
    for i, t in enumerate(torch_list):
        arr[i] = t.data_ptr()
    return arr


def _call_noalloc(lib, wl, w, wdot, stream):
    import gbmv
    nz, ny, nx = wl["fields"][0].shape
    g = gbmv.grid_struct((nx, ny, nz), wl["nchem"], wl["bc"], wl["gamma"])
    force = None
    if wl["force"] is not None:
        fa = np.ascontiguousarray(wl["force"], dtype=np.float64)
        force = fa.ctypes.data_as(C.POINTER(C.c_double))
    return lib.gbmv_feuler_noalloc(C.byref(g), force, C.c_double(0.0), _ptrs(w), _ptrs(wdot),
                                   C.c_void_p(stream))


def _reference_entry(torch, wl):
    import gbmv
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), wl["nchem"], wl["bc"], wl["gamma"], wl["force"])
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    wdot = [torch.empty_like(f) for f in w]
    assert h.fEuler(0.0, w, wdot) == 0
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in wdot]


def test_noalloc_matches_allocating_entry_twice(cuda):
    torch = cuda
    import gbmv
    lib = gbmv.load()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [W.rayleigh_taylor(shape=(40, 36, 32), nchem=10, seed=W.SEED_BASE + 200),
             W.rayleigh_taylor(shape=(24, 30, 20), nchem=4, seed=W.SEED_BASE + 201)]
    cases[1]["bc"] = (3, 3, 0, 0, 1, 1)
    for wl in cases:  # two calls in a row through the shared array
        w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
        wdot = [torch.full_like(f, np.nan) for f in w]
        rc = _call_noalloc(lib, wl, w, wdot, stream)
        assert rc == 0, lib.gbmv_last_error()
        torch.cuda.synchronize()
        ref = _reference_entry(torch, wl)
        for a, b in zip(wdot, ref):
            assert maxnorm_err(a.cpu().numpy(), b) <= TOL


def test_noalloc_status_is_cleared_between_calls(cuda):
    torch = cuda
    import gbmv
    lib = gbmv.load()
    stream = torch.cuda.current_stream().cuda_stream
    bad = W.rayleigh_taylor(shape=(8, 7, 6), nchem=0, seed=W.SEED_BASE + 202)
    bad["fields"][0][2, 2, 2] = -1.0
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in bad["fields"]]
    wdot = [torch.empty_like(f) for f in w]
    assert _call_noalloc(lib, bad, w, wdot, stream) == -1
    good = W.rayleigh_taylor(shape=(8, 7, 6), nchem=0, seed=W.SEED_BASE + 203)
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in good["fields"]]
    wdot = [torch.empty_like(f) for f in w]
    assert _call_noalloc(lib, good, w, wdot, stream) == 0
    torch.cuda.synchronize()
    ref = _reference_entry(torch, good)
    for a, b in zip(wdot, ref):
        assert maxnorm_err(a.cpu().numpy(), b) <= TOL


def test_noalloc_rejects_grids_beyond_capacity(cuda):
    torch = cuda
    import gbmv
    lib = gbmv.load()
    g = gbmv.grid_struct((128, 128, 128), 10, (0,) * 6, 1.4)
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    arr = _ptrs([dummy] * 6)
    rc = lib.gbmv_feuler_noalloc(C.byref(g), None, C.c_double(0.0), arr, arr,
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -101
    assert b"scratch" in lib.gbmv_last_error()
