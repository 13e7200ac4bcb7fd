"""The ARKODE-signature adapter (sundials-manyvector-demo_gb300/adapter/gbmv_arkode.cpp):
compiled with g++ against test-only SUNDIALS 6 stand-in headers (tests/arkode_shim: a
ManyVector of device arrays, the block-matrix data accessor, the generic SUNLinearSolver and
the MRI inner-stepper forcing interface) and linked against libgbmv.so; every callback is
called as ARKStep / MRIStep would call it and must reproduce the direct drop-in entry points
bit for bit (the same kernels on the same inputs).  CPU: it compiles, links and loads."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import workloads as W
from conftest import PKG, ROOT

SHIM = os.path.join(ROOT, "tests", "arkode_shim")
ADAPTER = os.path.join(PKG, "adapter")
_VP, _P = C.c_void_p, C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def drv(tmp_path_factory):
    import build_lib
    lib = build_lib.build()
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("arkdrv") / "libarkdrv.so")
    subprocess.check_call([cxx, "-std=c++17", "-O1", "-fPIC", "-shared", "-Wall", "-Werror",
                           "-I" + os.path.join(ROOT, "include"), "-I" + SHIM, "-I" + ADAPTER,
                           os.path.join(ADAPTER, "gbmv_arkode.cpp"),
                           os.path.join(SHIM, "shim_driver.cpp"),
                           "-L" + os.path.dirname(lib), "-lgbmv",
                           "-Wl,-rpath," + os.path.dirname(lib), "-o", out])
    L = C.CDLL(out)
    for name in ("drv_setup", "drv_rhs", "drv_ffast", "drv_jac", "drv_linsol", "drv_inner",
                 "drv_post", "drv_stability"):
        getattr(L, name).restype = C.c_int
    return L


def test_adapter_compiles_links_and_loads(drv):
    for name in ("gbmv_ark_feuler", "gbmv_ark_fexpl", "gbmv_ark_fimpl", "gbmv_ark_ffast",
                 "gbmv_ark_jac", "gbmv_ark_postprocess", "gbmv_ark_stability",
                 "gbmv_SUNLinSol_Block", "gbmv_inner_evolve", "gbmv_inner_fullrhs",
                 "gbmv_inner_reset"):
        assert hasattr(drv, name), name


def _ptrs(ts):
    a = (_VP * 6)()
    for i, t in enumerate(ts):
        a[i] = t.data_ptr()
    return a


def _lens(ts):
    a = (C.c_long * 6)()
    for i, t in enumerate(ts):
        a[i] = t.numel()
    return a


def _state(torch, wl):
    return [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]


def _same(a, b):
    return all(np.array_equal(x.cpu().numpy(), y.cpu().numpy(), equal_nan=True)
               for x, y in zip(a, b))


@pytest.mark.gpu
def test_adapter_rhs_callbacks_match_the_entries(cuda, tables, drv):
    torch = cuda
    import gbmv
    s = torch.cuda.current_stream().cuda_stream
    # fEuler on a pure-hydrodynamics ManyVector (5 components) and with tracers
    for nchem in (0, 10):
        wl = W.rayleigh_taylor(shape=(12, 10, 8), nchem=nchem, seed=W.SEED_BASE + 700 + nchem)
        nz, ny, nx = wl["fields"][0].shape
        h = gbmv.Hydro((nx, ny, nz), nchem, wl["bc"], wl["gamma"], wl["force"])
        w = _state(torch, wl)
        ref = [torch.empty_like(x) for x in w]
        got = [torch.empty_like(x) for x in w]
        assert h.fEuler(0.0, w, ref) == 0
        assert drv.drv_setup(h.h, None, C.c_double(1.0), C.c_double(1.0), C.c_double(0.5), 0,
                             C.c_void_p(s), None) == 0
        assert drv.drv_rhs(0, C.c_double(0.0), _ptrs(w), _ptrs(got), _lens(w), len(w)) == 0
        torch.cuda.synchronize()
        assert _same(got, ref)
        dt = C.c_double()
        assert drv.drv_stability(_ptrs(w), _lens(w), len(w), C.byref(dt)) == 0
        assert dt.value == h.stability(w, 0.5)
    # the chemistry-hydrodynamics callbacks
    wl = W.chem_hydro(shape=(10, 8, 6))
    nz, ny, nx = wl["fields"][0].shape
    n = nx * ny * nz
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    h = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])

    def chem():
        c = gbmv.Chem(n, tables)
        c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
        return c
    ca, cb = chem(), chem()
    drv.drv_setup(h.h, cb.c, C.c_double(eu), C.c_double(tu), C.c_double(0.0), 0, C.c_void_p(s),
                  None)
    wa, wb = _state(torch, wl), _state(torch, wl)
    ra, rb = [torch.empty_like(x) for x in wa], [torch.empty_like(x) for x in wa]
    assert gbmv.fexpl(h, ca, 0.0, wa, ra, eu) == 0
    assert drv.drv_rhs(1, C.c_double(0.0), _ptrs(wb), _ptrs(rb), _lens(wb), 6) == 0
    torch.cuda.synchronize()
    assert _same(ra, rb) and _same(wa, wb)   # fexpl rewrites et (and the chemistry round trip)
    gbmv.ffast(h, ca, 0.0, wa, ra, tu)
    assert drv.drv_rhs(2, C.c_double(0.0), _ptrs(wb), _ptrs(rb), _lens(wb), 6) == 0
    torch.cuda.synchronize()
    assert _same(ra, rb)
    # ffast with two forcing vectors
    rng = np.random.default_rng(3)
    fh = [[torch.from_numpy(1e-3 * rng.standard_normal(f.shape)).cuda() for f in wl["fields"]]
          for _ in range(2)]
    fptr = (_VP * 12)(*[t.data_ptr() for fv in fh for t in fv])
    gbmv.ffast(h, ca, 0.3, wa, ra, tu, fh, 0.1, 2.0)
    assert drv.drv_ffast(C.c_double(0.3), _ptrs(wb), _ptrs(rb), _lens(wb), 2, fptr,
                         C.c_double(0.1), C.c_double(2.0)) == 0
    torch.cuda.synchronize()
    assert _same(ra, rb)
    # PostprocessStep
    assert gbmv.PostprocessStep(h, ca, wa, eu) == 0
    assert drv.drv_post(C.c_double(0.0), _ptrs(wb), _lens(wb)) == 0
    torch.cuda.synchronize()
    assert _same(wa, wb)


@pytest.mark.gpu
def test_adapter_jacobian_and_linear_solver_match_the_entries(cuda, tables, drv):
    torch = cuda
    import gbmv
    s = torch.cuda.current_stream().cuda_stream
    wl = W.chem_hydro(shape=(8, 6, 5))
    nz, ny, nx = wl["fields"][0].shape
    n = nx * ny * nz
    tu = wl["units"]["TimeUnits"]
    h = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(n, tables)
    c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
    drv.drv_setup(h.h, c.c, C.c_double(1.0), C.c_double(tu), C.c_double(0.0), 0, C.c_void_p(s),
                  None)
    w = _state(torch, wl)
    f = torch.empty_like(w[5])
    c.calculate_rhs_cvklu(0.0, w[5].view(-1), f.view(-1), tu)  # the rates the Jacobian uses
    Ja = torch.empty(100 * n, dtype=torch.float64, device="cuda")
    Jb = torch.empty_like(Ja)
    c.calculate_jacobian_cvklu(0.0, w[5].view(-1), Ja, tu)
    assert drv.drv_jac(C.c_double(0.0), _ptrs(w), _lens(w), C.c_void_p(Jb.data_ptr()), n) == 0
    torch.cuda.synchronize()
    assert torch.equal(Ja, Jb)
    # ARKLS forms A = I - gamma J, then the solver's setup and solve on subvector 5
    gbmv.form_newton_matrix(Ja, 1e-4)
    gbmv.form_newton_matrix(Jb, 1e-4)
    b = [torch.from_numpy(np.random.default_rng(4).standard_normal(tuple(x.shape))).cuda()
         for x in w]
    xa = torch.empty_like(w[5])
    ls = gbmv.BlockLinearSolver(n)
    assert ls.setup(Ja) == 0
    ls.solve(Ja, xa.view(-1), b[5].view(-1))
    x = [torch.zeros_like(t) for t in w]
    assert drv.drv_linsol(_ptrs(x), _ptrs(b), _lens(w), C.c_void_p(Jb.data_ptr()), n) == 0
    torch.cuda.synchronize()
    assert torch.equal(xa, x[5]) and torch.equal(Ja, Jb)


@pytest.mark.gpu
def test_adapter_inner_stepper_matches_the_entries(cuda, tables, drv):
    """MRIStepInnerStepper evolve (forced), fullrhs (unforced ffast) and reset."""
    torch = cuda
    import gbmv
    s = torch.cuda.current_stream().cuda_stream
    wl = W.chem_hydro(shape=(8, 6, 5))
    nz, ny, nx = wl["fields"][0].shape
    n = nx * ny * nz
    tu = wl["units"]["TimeUnits"]
    h = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])

    def chem():
        c = gbmv.Chem(n, tables)
        c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
        return c
    ca, cb = chem(), chem()
    opts = gbmv.dirk_opts(rtol=1e-6, atol=1e-10, maxcor=10, nlscoef=0.01, block=64)
    drv.drv_setup(h.h, cb.c, C.c_double(1.0), C.c_double(tu), C.c_double(0.0), 0, C.c_void_p(s),
                  C.byref(opts))
    rng = np.random.default_rng(5)
    fh = [[torch.from_numpy(1e-2 * rng.standard_normal(f.shape)).cuda() for f in wl["fields"]]
          for _ in range(2)]
    fptr = (_VP * 12)(*[t.data_ptr() for fv in fh for t in fv])
    wa, wb = _state(torch, wl), _state(torch, wl)
    t0, t1, tshift, tscale = 0.2, 0.2 + 1e-4, 0.2, 1e-4
    nfa = gbmv.mri_fast_evolve(h, ca, t0, t1, wa, tu, fh, tshift, tscale, rtol=1e-6, atol=1e-10,
                               maxcor=10, nlscoef=0.01, block=64)
    rc = drv.drv_inner(0, C.c_double(t0), C.c_double(t1), _ptrs(wb), None, _lens(wb), 2, fptr,
                       C.c_double(tshift), C.c_double(tscale))
    torch.cuda.synchronize()
    assert nfa == 0 and rc == 0
    assert _same(wa, wb)
    fa, fb = [torch.empty_like(x) for x in wa], [torch.empty_like(x) for x in wa]
    gbmv.ffast(h, ca, t1, wa, fa, tu)
    assert drv.drv_inner(1, C.c_double(t1), C.c_double(0.0), _ptrs(wb), _ptrs(fb), _lens(wb),
                         2, fptr, C.c_double(tshift), C.c_double(tscale)) == 0
    torch.cuda.synchronize()
    assert _same(fa, fb)
    assert drv.drv_inner(2, C.c_double(t1), C.c_double(0.0), _ptrs(wb), None, _lens(wb), 0,
                         None, C.c_double(0.0), C.c_double(1.0)) == 0
