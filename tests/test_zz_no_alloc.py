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
from conftest import case_fields, feuler_case_names, maxnorm_err

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
    g = gbmv.grid_struct((nx, ny, nz), wl["nchem"], wl["bc"], wl["gamma"],
                         wl.get("domain", (0.0, 1.0, 0.0, 1.0, 0.0, 1.0)))
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


def test_noalloc_matches_reference_fixtures(cuda, golden_feuler):
    """Against the outputs of the reference's own fEuler (tests/golden), every fixture case,
    two calls in a row per case through the shared array."""
    torch = cuda
    import gbmv
    lib = gbmv.load()
    stream = torch.cuda.current_stream().cuda_stream
    g = golden_feuler
    for name in feuler_case_names(g):
        fields, nchem, bc, gamma, force = case_fields(g, name)
        wl = dict(fields=fields, nchem=nchem, bc=bc, gamma=gamma,
                  force=None if force is None or np.ndim(force) == 0 else force)
        w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in fields]
        for _ in range(2):
            wdot = [torch.full_like(f, np.nan) for f in w]
            rc = _call_noalloc(lib, wl, w, wdot, stream)
            assert rc == int(g[f"{name}/status"]), (name, rc, lib.gbmv_last_error())
            if rc:
                continue
            torch.cuda.synchronize()
            for i, o in enumerate(wdot):
                e = maxnorm_err(o.cpu().numpy(), g[f"{name}/wdot{i}"])
                assert e <= TOL, (name, i, e)


def test_noalloc_second_call_commits_no_memory(cuda):
    """The first call on a device may commit the fixed array (lazy module loading); after it,
    calls take no device memory: the device's free memory is the same before and after."""
    torch = cuda
    import gbmv
    lib = gbmv.load()
    stream = torch.cuda.current_stream().cuda_stream
    wl = W.rayleigh_taylor(shape=(20, 18, 16), nchem=10, seed=W.SEED_BASE + 204)
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    wdot = [torch.empty_like(f) for f in w]
    assert _call_noalloc(lib, wl, w, wdot, stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call_noalloc(lib, wl, w, wdot, stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_reports_refusals(cuda):
    """Every refusal sets the message: bad grids as gbmv_hydro_create, null fields."""
    torch = cuda
    import gbmv
    lib = gbmv.load()
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    arr = _ptrs([dummy] * 6)
    g = gbmv.grid_struct((8, 8, 8), 3, (0,) * 6, 1.4)
    assert lib.gbmv_feuler_noalloc(C.byref(g), None, C.c_double(0.0), arr, arr, s) == -104
    assert b"nchem" in lib.gbmv_last_error()
    g = gbmv.grid_struct((8, 8, 8), 0, (0,) * 6, 1.4)
    empty = (C.c_void_p * 6)()
    assert lib.gbmv_feuler_noalloc(C.byref(g), None, C.c_double(0.0), empty, arr, s) == -101
    assert b"null field" in lib.gbmv_last_error()
