"""Python host mirror of the reference's RHS-path interface over the C ABI (include/gbmv.h).

Names and argument meanings follow the reference so that tests read like its drivers:

  EulerData-like ``Hydro``   .fEuler(t, w, wdot)          src/utilities.cpp:17
  cvklu_data-like ``Chem``   .calculate_rhs_cvklu(...)    src/raja_primordial_network.cpp:1015
                             .calculate_jacobian_cvklu(...) :1393
                             .prepare_Dengo_structures(...) src/primordial_static.cpp:227
  ``BlockLinearSolver``      .setup(A) / .solve(A, x, b)   src/multirate_chem_hydro_main.cpp:1360-1395
  ``fexpl`` / ``PostprocessStep``                          src/imex_chem_hydro_main.cpp:910, 1002

A ManyVector is a list of torch CUDA float64 tensors: [rho, mx, my, mz, et] each (nz, ny, nx)
and, when nchem > 0, chem (nz, ny, nx, nchem).  Errors follow ARKODE conventions (int return
codes); any negative code other than -1 (illegal state) raises GbmvError.  There is no CPU
fallback: without the CUDA library and a GPU every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libgbmv.so")

BC_PERIODIC, BC_NEUMANN, BC_DIRICHLET, BC_REFLECTING = 0, 1, 2, 3
FP64, MIXED, MIXED_FAST = 0, 1, 2
SWEEPS_ALONE, SWEEPS_SHARED = 0, 1  # gbmv_hydro_set_sweep_budget
FORCE_IN_WDOT = 1


class GbmvError(RuntimeError):
    pass


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_long), ("ny", C.c_long), ("nz", C.c_long), ("nchem", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("gamma", C.c_double), ("bc", C.c_int * 6)]


class _DirkOpts(C.Structure):
    """gbmv_dirk_opts (include/gbmv.h)."""
    _fields_ = [(k, C.c_double) for k in ("rtol", "atol", "nlscoef", "h0", "safety", "dgmax",
                                          "growth", "etamx1", "hmax")] + \
               [(k, C.c_int) for k in ("maxcor", "max_steps", "msbp", "maxnef", "maxncf",
                                       "precision", "refine", "block", "table",
                                       "setup_batch", "order", "deduce")]


MAX_STAGES = 7


class _Butcher(C.Structure):
    """gbmv_butcher (include/gbmv.h)."""
    _fields_ = [("id", C.c_int), ("stages", C.c_int), ("q", C.c_int), ("p", C.c_int),
                ("c", C.c_double * MAX_STAGES), ("A", (C.c_double * MAX_STAGES) * MAX_STAGES),
                ("b", C.c_double * MAX_STAGES), ("bhat", C.c_double * MAX_STAGES),
                ("name", C.c_char * 32)]


class _StepParams(C.Structure):
    """gbmv_step_params (include/gbmv.h)."""
    _fields_ = [(k, C.c_double) for k in ("hmax", "safety", "bias", "growth", "etamx1",
                                          "etamxf", "k1", "k2", "k3")] + \
               [(k, C.c_int) for k in ("order", "small_nef", "maxnef", "max_attempts", "fixed")]


# indices of the device step state (GBMV_ST_* of include/gbmv.h)
ST = dict(t=0, h=1, h_used=2, accept=3, done=4, e1=5, e2=6, first=7, nef=8, steps=9,
          attempts=10, fails=11, status=12, last=13, h_prop=14, tf=15)
STEP_STATE = 16

_P = C.POINTER(C.c_double)
_VP = C.c_void_p

# (name, restype, argtypes) for every symbol of include/gbmv.h
SIGNATURES = [
    ("gbmv_hydro_create", C.c_int, [C.POINTER(_Grid), C.POINTER(_VP)]),
    ("gbmv_hydro_destroy", C.c_int, [_VP]),
    ("gbmv_hydro_set_force", C.c_int, [_VP, _P]),
    ("gbmv_feuler", C.c_int, [_VP, C.c_double, C.POINTER(_VP), C.POINTER(_VP), C.c_int, _VP]),
    ("gbmv_feuler_async", C.c_int, [_VP, C.c_double, C.POINTER(_VP), C.POINTER(_VP), C.c_int,
                                    C.c_int, _VP, _VP]),
    ("gbmv_feuler_noalloc", C.c_int, [C.POINTER(_Grid), _P, C.c_double, C.POINTER(_VP),
                                      C.POINTER(_VP), _VP]),
    ("gbmv_stability", C.c_int, [_VP, C.POINTER(_VP), C.c_double, _P, _VP]),
    ("gbmv_hydro_autotune", C.c_int, [_VP, C.POINTER(_VP), C.c_int, C.POINTER(C.c_int), _VP]),
    ("gbmv_hydro_set_sweep_budget", C.c_int, [_VP, C.c_int]),
    ("gbmv_hydro_set_sweep_threads", C.c_int, [_VP, C.c_int, C.c_int]),
    ("gbmv_chem_newton_autotune", C.c_int, [_VP, _VP, C.c_double, C.c_double, C.c_int, C.c_int,
                                            C.POINTER(C.c_int), _VP]),
    ("gbmv_pack1d", C.c_int, [_VP, C.POINTER(_VP), C.c_int, _VP, _VP]),
    ("gbmv_conservation", C.c_int, [_VP, C.POINTER(_VP), C.c_double, C.c_double, _P, _VP]),
    ("gbmv_wrms_norm", C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP), C.c_double, C.c_double,
                                 _P, _VP]),
    ("gbmv_print_stats", C.c_int, [_VP, C.POINTER(_VP), C.c_double, C.c_double, C.c_double,
                                   _P, _VP]),
    ("gbmv_feuler_jvp", C.c_int, [_VP, C.c_double, C.POINTER(_VP), C.POINTER(_VP),
                                  C.POINTER(_VP), _VP]),
    ("gbmv_feuler_vjp", C.c_int, [_VP, C.c_double, C.POINTER(_VP), C.POINTER(_VP),
                                  C.POINTER(_VP), _VP]),
    ("gbmv_chem_jvp", C.c_int, [_VP, C.c_double, _VP, _VP, _VP, C.c_double, _VP]),
    ("gbmv_chem_vjp", C.c_int, [_VP, C.c_double, _VP, _VP, _VP, C.c_double, _VP]),
    ("gbmv_chem_create", C.c_int, [C.c_long, _P, C.c_double, C.POINTER(_VP)]),
    ("gbmv_chem_destroy", C.c_int, [_VP]),
    ("gbmv_chem_prepare", C.c_int, [_VP, _VP, _VP]),
    ("gbmv_chem_set_scale", C.c_int, [_VP, _VP, _VP]),
    ("gbmv_chem_apply_scaling", C.c_int, [_VP, _VP, _VP]),
    ("gbmv_chem_unapply_scaling", C.c_int, [_VP, _VP, _VP]),
    ("gbmv_chem_rhs", C.c_int, [_VP, C.c_double, _VP, _VP, C.c_double, _VP]),
    ("gbmv_chem_jac", C.c_int, [_VP, C.c_double, _VP, _VP, C.c_double, _VP]),
    ("gbmv_chem_state", _VP, [_VP, C.c_int]),
    ("gbmv_chem_newton", C.c_int, [_VP, C.c_double, _VP, _VP, _VP, C.c_double, C.c_double,
                                   C.c_int, C.c_int, _VP]),
    ("gbmv_block_lu_factor", C.c_int, [C.c_long, _VP, _VP, _VP]),
    ("gbmv_block_lu_solve", C.c_int, [C.c_long, _VP, _VP, _VP, _VP, _VP]),
    ("gbmv_block_form_newton", C.c_int, [C.c_long, _VP, C.c_double, _VP]),
    ("gbmv_block_ls_create", C.c_int, [C.c_long, C.POINTER(_VP)]),
    ("gbmv_block_ls_destroy", C.c_int, [_VP]),
    ("gbmv_block_ls_setup", C.c_int, [_VP, _VP, _VP]),
    ("gbmv_block_ls_solve", C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    ("gbmv_fexpl", C.c_int, [_VP, _VP, C.c_double, C.POINTER(_VP), C.POINTER(_VP), C.c_double,
                             C.c_int, _VP]),
    ("gbmv_fexpl_async", C.c_int, [_VP, _VP, C.c_double, C.POINTER(_VP), C.POINTER(_VP),
                                   C.c_double, C.c_int, _VP, _VP]),
    ("gbmv_chem_newton_stage", C.c_int, [_VP, C.c_double, _VP, _VP, _VP, _VP, C.c_double,
                                         C.c_double, C.c_int, C.c_int, _VP]),
    ("gbmv_chem_newton_async", C.c_int, [_VP, C.c_double, _VP, _VP, _VP, C.c_double, C.c_double,
                                         C.c_int, C.c_int, _VP, _VP]),
    ("gbmv_chem_newton_queue_async", C.c_int, [_VP, C.c_double, _VP, _VP, _VP, C.c_double,
                                               C.c_double, C.c_int, C.c_int, _VP, C.c_int, _VP,
                                               _VP]),
    ("gbmv_dirk_opts_default", None, [C.POINTER(_DirkOpts)]),
    ("gbmv_chem_dirk_evolve", C.c_int, [_VP, C.c_double, C.c_double, _VP, C.c_double,
                                        C.POINTER(_DirkOpts), _VP, _VP]),
    ("gbmv_chem_dirk_evolve_async", C.c_int, [_VP, C.c_double, C.c_double, _VP, C.c_double,
                                              C.POINTER(_DirkOpts), _VP, _VP, _VP]),
    ("gbmv_chem_dirk_block", C.c_int, [_VP, C.c_int]),
    ("gbmv_chem_dirk_retried", C.c_int, [_VP, C.POINTER(C.c_int), C.c_int, _VP]),
    ("gbmv_chem_set_newton_occupancy", C.c_int, [_VP, C.c_int]),
    ("gbmv_mri_fast_evolve", C.c_int, [_VP, _VP, C.c_double, C.c_double, C.POINTER(_VP),
                                       C.c_double, C.c_int, C.POINTER(_VP), C.c_double,
                                       C.c_double, C.POINTER(_DirkOpts), _VP, _VP]),
    ("gbmv_mri_fast_evolve_async", C.c_int, [_VP, _VP, C.c_double, C.c_double, C.POINTER(_VP),
                                             C.c_double, C.c_int, C.POINTER(_VP), C.c_double,
                                             C.c_double, C.POINTER(_DirkOpts), _VP, _VP, _VP]),
    ("gbmv_ffast", C.c_int, [_VP, _VP, C.c_double, C.POINTER(_VP), C.POINTER(_VP), C.c_double,
                             C.c_int, C.POINTER(_VP), C.c_double, C.c_double, _VP]),
    ("gbmv_postprocess_step", C.c_int, [_VP, _VP, C.POINTER(_VP), C.c_double, _VP]),
    ("gbmv_step_begin", C.c_int, [_VP, C.POINTER(_StepParams), _VP]),
    ("gbmv_step_end", C.c_int, [_VP, _VP, C.POINTER(_StepParams), _VP]),
    ("gbmv_step_select", C.c_int, [C.c_long, _VP, _VP, _VP, _VP]),
    ("gbmv_feuler_kink_mask", C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP), C.c_double, _VP,
                                        _VP]),
    ("gbmv_wrms_norm_async", C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP), C.c_double,
                                       C.c_double, _VP, _VP]),
    ("gbmv_butcher_table", C.c_int, [C.c_int, C.POINTER(_Butcher)]),
    ("gbmv_erk_default_table", C.c_int, [C.c_int]),
    ("gbmv_version", C.c_char_p, []),
    ("gbmv_last_error", C.c_char_p, []),
    ("gbmv_launch_count", C.c_long, []),
    ("gbmv_diag_fma_rate", C.c_int, [C.c_int, _P]),
    ("gbmv_diag_convert_check", C.c_int, [_VP, C.c_long, C.POINTER(C.c_ulonglong), _VP]),
    ("gbmv_profile_enable", C.c_int, [C.c_int]),
    ("gbmv_profile_reset", C.c_int, []),
    ("gbmv_profile_get", C.c_int, [C.c_char_p, _P, C.POINTER(C.c_long)]),
]

_lib = None


def load(path: str = LIB_PATH):
    """Load libgbmv.so (built by build_lib.build()); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise GbmvError(f"{path} not built: run __graft_entry__.build()")
        L = C.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int, what: str, allow=(0,)):
    if rc in allow:
        return rc
    if rc < 0 and rc != -1:
        raise GbmvError(f"{what} failed ({rc}): {load().gbmv_last_error().decode()}")
    return rc


def _dev_ptr(t):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise GbmvError("expected a CUDA tensor")
    if t.dtype != torch.float64 or not t.is_contiguous():
        raise GbmvError("expected a contiguous float64 tensor")
    return t.data_ptr()


def _stream_ptr(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _vec(fields):
    arr = (_VP * 6)()
    for i, f in enumerate(fields):
        arr[i] = _dev_ptr(f)
    return arr


def grid_struct(shape, nchem, bc, gamma, domain=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)):
    nx, ny, nz = shape
    g = _Grid()
    g.nx, g.ny, g.nz, g.nchem = nx, ny, nz, nchem
    g.dx = (domain[1] - domain[0]) / nx  # EulerData::SetupDecomp (src/euler3D.hpp:412-414)
    g.dy = (domain[3] - domain[2]) / ny
    g.dz = (domain[5] - domain[4]) / nz
    g.gamma = gamma
    for i in range(6):
        g.bc[i] = bc[i]
    return g


class Hydro:
    """Device-side EulerData: grid, boundary conditions, gamma, constant forcing."""

    def __init__(self, shape, nchem, bc, gamma=1.4, force=None,
                 domain=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)):
        L = load()
        self.shape, self.nchem = tuple(shape), nchem
        self.grid = grid_struct(shape, nchem, bc, gamma, domain)
        h = _VP()
        _check(L.gbmv_hydro_create(C.byref(self.grid), C.byref(h)), "gbmv_hydro_create")
        self.h = h
        if force is not None:
            fa = np.ascontiguousarray(force, dtype=np.float64)
            _check(L.gbmv_hydro_set_force(h, fa.ctypes.data_as(_P)), "gbmv_hydro_set_force")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.gbmv_hydro_destroy(self.h)
            self.h = None

    def fEuler(self, t, w, wdot, precision=FP64, stream=None) -> int:
        """Returns 0, or -1 on an illegal state (as the reference's fEuler)."""
        return _check(load().gbmv_feuler(self.h, t, _vec(w), _vec(wdot), precision,
                                         _stream_ptr(stream)), "gbmv_feuler", allow=(0, -1))

    def stability(self, w, cfl, stream=None) -> float:
        """CFL-limited step (the reference's ARKStabilityFn `stability`)."""
        dt = C.c_double()
        _check(load().gbmv_stability(self.h, _vec(w[:5]), cfl, C.byref(dt), _stream_ptr(stream)),
               "gbmv_stability")
        return dt.value

    def fEuler_async(self, t, w, wdot, status, precision=FP64, flags=0, stream=None) -> int:
        return _check(load().gbmv_feuler_async(self.h, t, _vec(w), _vec(wdot), precision, flags,
                                               status.data_ptr(), _stream_ptr(stream)),
                      "gbmv_feuler_async")

    def pack1D(self, w, direction, out, stream=None):
        """Stencils of every face normal to `direction` (pack1D_x/y/z(_bdry),
        src/euler3D.hpp:1197): out is a CUDA float64 tensor of 6 * NVAR * nfaces."""
        return _check(load().gbmv_pack1d(self.h, _vec(w), direction, _dev_ptr(out),
                                         _stream_ptr(stream)), "gbmv_pack1d")

    def check_conservation(self, w, mass_factor=1.0, energy_factor=1.0, stream=None):
        """(total mass, total energy) as check_conservation (src/io.cpp:503) sums them."""
        out = (C.c_double * 2)()
        _check(load().gbmv_conservation(self.h, _vec(w), mass_factor, energy_factor, out,
                                        _stream_ptr(stream)), "gbmv_conservation")
        return out[0], out[1]

    def wrms_norm(self, v, y, rtol, atol, stream=None) -> float:
        """ARKODE's WRMS norm of the ManyVector v with weights 1 / (rtol |y| + atol)."""
        out = (C.c_double * 1)()
        _check(load().gbmv_wrms_norm(self.h, _vec(v), _vec(y), rtol, atol, out,
                                     _stream_ptr(stream)), "gbmv_wrms_norm")
        return out[0]

    def autotune(self, w, precision=FP64, stream=None) -> int:
        """gbmv_hydro_autotune: the face sweeps' threads per block for this precision."""
        t = C.c_int()
        _check(load().gbmv_hydro_autotune(self.h, _vec(w), precision, C.byref(t),
                                          _stream_ptr(stream)), "gbmv_hydro_autotune")
        return t.value

    def set_sweep_budget(self, shared: bool) -> None:
        """gbmv_hydro_set_sweep_budget: GBMV_MIXED_FAST face sweeps sized to run alone (False)
        or beside another kernel on the same SMs (True)."""
        _check(load().gbmv_hydro_set_sweep_budget(self.h, SWEEPS_SHARED if shared
                                                  else SWEEPS_ALONE),
               "gbmv_hydro_set_sweep_budget")

    def set_sweep_threads(self, precision, threads) -> None:
        """gbmv_hydro_set_sweep_threads: the face sweeps' threads per block (0 = default)."""
        _check(load().gbmv_hydro_set_sweep_threads(self.h, precision, threads),
               "gbmv_hydro_set_sweep_threads")

    def kink_mask(self, w, dw, eps, mask, stream=None):
        """gbmv_feuler_kink_mask into `mask` (CUDA uint8 tensor of ncells): 1 where a central
        difference of fEuler along dw with step eps crosses a Lax-Friedrichs branch."""
        import torch
        ncell = self.shape[0] * self.shape[1] * self.shape[2]
        if mask.dtype != torch.uint8 or not mask.is_cuda or mask.numel() != ncell:
            raise GbmvError("mask must be a CUDA uint8 tensor of ncells")
        _check(load().gbmv_feuler_kink_mask(self.h, _vec(w), _vec(dw), eps, mask.data_ptr(),
                                            _stream_ptr(stream)), "gbmv_feuler_kink_mask")

    def wrms_norm_async(self, v, y, rtol, atol, out, stream=None):
        """gbmv_wrms_norm_async: the norm into the 1-element CUDA float64 tensor `out`."""
        _check(load().gbmv_wrms_norm_async(self.h, _vec(v), _vec(y), rtol, atol, _dev_ptr(out),
                                           _stream_ptr(stream)), "gbmv_wrms_norm_async")

    def print_stats(self, w, units=(1.0, 1.0, 1.0), stream=None):
        """Per-field RMS over the grid as print_stats (src/io.cpp:552) computes it; units =
        (DensityUnits, MomentumUnits, EnergyUnits) for CGS output."""
        nv = 5 + self.nchem
        out = (C.c_double * nv)()
        _check(load().gbmv_print_stats(self.h, _vec(w), units[0], units[1], units[2], out,
                                       _stream_ptr(stream)), "gbmv_print_stats")
        return list(out)

    def fEuler_jvp(self, t, w, dw, jv, stream=None) -> int:
        """jv = (d fEuler / d w) dw (FP64 form, forward mode)."""
        return _check(load().gbmv_feuler_jvp(self.h, t, _vec(w), _vec(dw), _vec(jv),
                                             _stream_ptr(stream)), "gbmv_feuler_jvp")

    def fEuler_vjp(self, t, w, v, u, stream=None) -> int:
        """u = (d fEuler / d w)^T v (FP64 form, hand-written reverse mode)."""
        return _check(load().gbmv_feuler_vjp(self.h, t, _vec(w), _vec(v), _vec(u),
                                             _stream_ptr(stream)), "gbmv_feuler_vjp")


class Chem:
    """Device-side cvklu_data: rate tables, scale arrays, temperature state."""

    def __init__(self, ncells: int, tables: np.ndarray, current_z: float = -1.0):
        L = load()
        tab = np.ascontiguousarray(tables, dtype=np.float64)
        if tab.shape != (50, 1024):
            raise GbmvError("tables must be the (50, 1024) block of h5tables.load_table_block")
        c = _VP()
        _check(L.gbmv_chem_create(ncells, tab.ctypes.data_as(_P), current_z, C.byref(c)),
               "gbmv_chem_create")
        self.c, self.n = c, ncells

    def __del__(self):
        if getattr(self, "c", None) and _lib is not None:
            _lib.gbmv_chem_destroy(self.c)
            self.c = None

    def state(self, which: str):
        """Torch view of a persistent per-cell array (Ts, dTs_ge, mdensity, inv_mdensity,
        cie_optical_depth_approx, h2_optical_depth_approx, scale, inv_scale)."""
        import torch
        idx = ["Ts", "dTs_ge", "mdensity", "inv_mdensity", "cie_optical_depth_approx",
               "h2_optical_depth_approx", "scale", "inv_scale"].index(which)
        ptr = load().gbmv_chem_state(self.c, idx)
        n = self.n * (10 if idx >= 6 else 1)
        return _wrap_device(ptr, n)

    def prepare_Dengo_structures(self, chem, stream=None):
        _check(load().gbmv_chem_prepare(self.c, _dev_ptr(chem), _stream_ptr(stream)), "prepare")

    def set_scale(self, scale, stream=None):
        _check(load().gbmv_chem_set_scale(self.c, _dev_ptr(scale), _stream_ptr(stream)), "set_scale")

    def apply_Dengo_scaling(self, chem, stream=None):
        _check(load().gbmv_chem_apply_scaling(self.c, _dev_ptr(chem), _stream_ptr(stream)), "apply")

    def unapply_Dengo_scaling(self, chem, stream=None):
        _check(load().gbmv_chem_unapply_scaling(self.c, _dev_ptr(chem), _stream_ptr(stream)),
               "unapply")

    def calculate_rhs_cvklu(self, t, y, ydot, time_units=1.0, stream=None):
        return _check(load().gbmv_chem_rhs(self.c, t, _dev_ptr(y), _dev_ptr(ydot), time_units,
                                           _stream_ptr(stream)), "gbmv_chem_rhs")

    def newton_iteration(self, t, y, f, x, gamma, time_units=1.0, lu_precision=FP64, refine=2,
                         stream=None) -> int:
        """Fused f = TimeUnits*f(y) and x = (I - gamma*J(y))^{-1} f; 0, or 1 if singular."""
        return _check(load().gbmv_chem_newton(self.c, t, _dev_ptr(y), _dev_ptr(f), _dev_ptr(x),
                                              gamma, time_units, lu_precision, refine,
                                              _stream_ptr(stream)),
                      "gbmv_chem_newton", allow=(0, 1))

    def newton_stage(self, t, y, b, f, x, gamma, time_units=1.0, lu_precision=FP64, refine=2,
                     stream=None) -> int:
        """Fused implicit-stage correction: f = TimeUnits*f(y) and
        x = (I - gamma*J(y))^{-1} (b + gamma*f); 0, or 1 if a block is singular."""
        return _check(load().gbmv_chem_newton_stage(self.c, t, _dev_ptr(y), _dev_ptr(b),
                                                    _dev_ptr(f), _dev_ptr(x), gamma, time_units,
                                                    lu_precision, refine, _stream_ptr(stream)),
                      "gbmv_chem_newton_stage", allow=(0, 1))

    def calculate_jacobian_cvklu(self, t, y, J, time_units=1.0, stream=None):
        return _check(load().gbmv_chem_jac(self.c, t, _dev_ptr(y), _dev_ptr(J), time_units,
                                           _stream_ptr(stream)), "gbmv_chem_jac")

    def jvp(self, t, y, dy, out, time_units=1.0, stream=None) -> int:
        """out = J dy with J = time_units * df/dy (entries of calculate_jacobian_cvklu)."""
        return _check(load().gbmv_chem_jvp(self.c, t, _dev_ptr(y), _dev_ptr(dy), _dev_ptr(out),
                                           time_units, _stream_ptr(stream)), "gbmv_chem_jvp")

    def vjp(self, t, y, v, out, time_units=1.0, stream=None) -> int:
        """out = J^T v (the adjoint of the chemistry source)."""
        return _check(load().gbmv_chem_vjp(self.c, t, _dev_ptr(y), _dev_ptr(v), _dev_ptr(out),
                                           time_units, _stream_ptr(stream)), "gbmv_chem_vjp")

    def dirk_evolve(self, t0, tout, y, time_units=1.0, stats=None, stream=None, **opts) -> int:
        """Evolve every cell's chemistry from t0 to tout in place (persistent batched DIRK +
        Newton, gbmv_chem_dirk_evolve): the fast-stage integration of the chemistry drivers.
        opts: fields of gbmv_dirk_opts (rtol, atol, nlscoef, maxcor, precision, refine,
        block, ...).  stats: None or a CUDA int32 tensor of 8 * ncells.  Returns the number of
        failed cells."""
        o = dirk_opts(**opts)
        sp = None
        if stats is not None:
            import torch
            if stats.dtype != torch.int32 or not stats.is_cuda or stats.numel() != 8 * self.n:
                raise GbmvError("stats must be a CUDA int32 tensor of 8 * ncells")
            sp = stats.data_ptr()
        return _check(load().gbmv_chem_dirk_evolve(self.c, t0, tout, _dev_ptr(y), time_units,
                                                   C.byref(o), sp, _stream_ptr(stream)),
                      "gbmv_chem_dirk_evolve", allow=range(0, self.n + 1))

    def dirk_evolve_async(self, t0, tout, y, nfail, time_units=1.0, stats=None, stream=None,
                          **opts):
        """Same, asynchronous and graph-capturable; failures are added to nfail (CUDA int32)."""
        o = dirk_opts(**opts)
        return _check(load().gbmv_chem_dirk_evolve_async(
            self.c, t0, tout, _dev_ptr(y), time_units, C.byref(o),
            stats.data_ptr() if stats is not None else None, nfail.data_ptr(),
            _stream_ptr(stream)), "gbmv_chem_dirk_evolve_async")

    def newton_autotune(self, y, gamma, time_units=1.0, lu_precision=MIXED, refine=2,
                        stream=None) -> int:
        """gbmv_chem_newton_autotune: the fused Newton's resident blocks per SM (0 = deep
        grid), kept as the handle's Newton occupancy."""
        b = C.c_int()
        _check(load().gbmv_chem_newton_autotune(self.c, _dev_ptr(y), gamma, time_units,
                                                lu_precision, refine, C.byref(b),
                                                _stream_ptr(stream)),
               "gbmv_chem_newton_autotune")
        return b.value

    def set_newton_occupancy(self, blocks_per_sm: int):
        """Resident blocks per SM of the fused Newton kernel (0 = default deep grid)."""
        _check(load().gbmv_chem_set_newton_occupancy(self.c, blocks_per_sm), "set_newton_occupancy")

    def dirk_retried(self, max_cells=1 << 20, stream=None):
        """Cells the last GBMV_MIXED DIRK call integrated again in FP64 (gbmv_chem_dirk_retried):
        their indices as a numpy array."""
        buf = (C.c_int * max_cells)()
        n = _check(load().gbmv_chem_dirk_retried(self.c, buf, max_cells, _stream_ptr(stream)),
                   "gbmv_chem_dirk_retried", allow=range(0, 1 << 31))
        return np.array(buf[:min(n, max_cells)], dtype=np.int64)

    def dirk_block(self, precision=FP64) -> int:
        """Block size the autotuner picked for a precision (0 = not tuned yet)."""
        return load().gbmv_chem_dirk_block(self.c, precision)


DIRK_STATS = ("steps", "newton_iters", "error_fails", "newton_fails", "setups", "jacobians",
              "f_evals", "failed")


def dirk_opts(**kw) -> _DirkOpts:
    """gbmv_dirk_opts with the library defaults, overridden by keyword."""
    o = _DirkOpts()
    load().gbmv_dirk_opts_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise GbmvError(f"unknown DIRK option {k}")
        setattr(o, k, v)
    return o


def step_params(order, hmax=0.0, safety=0.96, bias=1.5, growth=20.0, etamx1=1e4,
                etamxf=0.3, k1=0.58, k2=0.21, k3=0.1, small_nef=2, maxnef=7,
                max_attempts=100000, fixed=False) -> _StepParams:
    """gbmv_step_params (ARKODE's defaults: the PID controller)."""
    p = _StepParams()
    p.hmax, p.safety, p.bias, p.growth = hmax, safety, bias, growth
    p.etamx1, p.etamxf, p.k1, p.k2, p.k3 = etamx1, etamxf, k1, k2, k3
    p.order, p.small_nef, p.maxnef, p.max_attempts = order, small_nef, maxnef, max_attempts
    p.fixed = int(bool(fixed))
    return p


def step_begin(state, params, stream=None):
    _check(load().gbmv_step_begin(_dev_ptr(state), C.byref(params), _stream_ptr(stream)),
           "gbmv_step_begin")


def step_end(state, dsm, params, stream=None):
    _check(load().gbmv_step_end(_dev_ptr(state), _dev_ptr(dsm), C.byref(params),
                                _stream_ptr(stream)), "gbmv_step_end")


def step_select(state, y, ynew, stream=None):
    _check(load().gbmv_step_select(y.numel(), _dev_ptr(state), _dev_ptr(y), _dev_ptr(ynew),
                                   _stream_ptr(stream)), "gbmv_step_select")


def butcher_table(table_id: int) -> dict:
    """The Runge-Kutta table of ARKODE number `table_id` (gbmv_butcher_table): dict with name,
    s, q (method order), p (embedding order), c, A (rows, diagonal included), b, bhat.
    Host-only (no GPU needed)."""
    t = _Butcher()
    _check(load().gbmv_butcher_table(int(table_id), C.byref(t)), "gbmv_butcher_table")
    s = t.stages
    return {"id": t.id, "name": t.name.decode(), "s": s, "q": t.q, "p": t.p,
            "c": [t.c[i] for i in range(s)],
            "A": [[t.A[i][j] for j in range(s)] for i in range(s)],
            "b": [t.b[i] for i in range(s)], "bhat": [t.bhat[i] for i in range(s)]}


def erk_default_table(order: int) -> int:
    """ARKODE's default explicit table number for an order (-1 if none)."""
    return load().gbmv_erk_default_table(int(order))


def _wrap_device(ptr: int, n: int):
    """Non-owning float64 CUDA tensor over library-owned device memory."""
    import torch

    class _Holder:
        def __init__(self, p, nbytes):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8",
                                             "data": (p, False), "version": 3,
                                             "strides": None}

    return torch.as_tensor(_Holder(ptr, n * 8), device="cuda")


class BlockLinearSolver:
    """Block-diagonal direct solver on the chemistry subvector (SUNLinSol_RankLocalLS /
    SUNLinSol_BDMPIMV over the batched dense LU, gbmv_block_ls): setup factors A in place;
    the handle owns the pivots and its singular-block word."""

    def __init__(self, nblocks: int):
        self.nb = nblocks
        h = _VP()
        _check(load().gbmv_block_ls_create(nblocks, C.byref(h)), "gbmv_block_ls_create")
        self.ls = h
        self.last_flag = 0

    def __del__(self):
        if getattr(self, "ls", None) and _lib is not None:
            _lib.gbmv_block_ls_destroy(self.ls)
            self.ls = None

    def setup(self, A, stream=None) -> int:
        self.last_flag = _check(load().gbmv_block_ls_setup(self.ls, _dev_ptr(A),
                                                           _stream_ptr(stream)),
                                "gbmv_block_ls_setup", allow=(0, 1))
        return self.last_flag

    def solve(self, A, x, b, tol=0.0, stream=None) -> int:
        self.last_flag = _check(load().gbmv_block_ls_solve(self.ls, _dev_ptr(A), _dev_ptr(b),
                                                           _dev_ptr(x), _stream_ptr(stream)),
                                "gbmv_block_ls_solve")
        return self.last_flag


def form_newton_matrix(J, gamma, stream=None):
    """A = I - gamma*J in place (ARKLS's SUNMatScaleAddI on the block matrix)."""
    nb = J.numel() // 100
    _check(load().gbmv_block_form_newton(nb, _dev_ptr(J), gamma, _stream_ptr(stream)),
           "gbmv_block_form_newton")


def fexpl(hydro: Hydro, chem: Chem, t, w, wdot, energy_units, precision=FP64, stream=None):
    return _check(load().gbmv_fexpl(hydro.h, chem.c, t, _vec(w), _vec(wdot), energy_units,
                                    precision, _stream_ptr(stream)), "gbmv_fexpl", allow=(0, -1))


def fexpl_async(hydro: Hydro, chem: Chem, t, w, wdot, energy_units, status, precision=FP64,
                stream=None):
    """Graph-capturable fexpl: the legal-state mask is OR-ed into `status` (int32 CUDA tensor)."""
    return _check(load().gbmv_fexpl_async(hydro.h, chem.c, t, _vec(w), _vec(wdot), energy_units,
                                          precision, status.data_ptr(), _stream_ptr(stream)),
                  "gbmv_fexpl_async")


def chem_newton_async(chem: Chem, t, y, f, x, gamma, time_units, info, lu_precision=FP64,
                      refine=4, stream=None):
    """Graph-capturable fused Newton iteration; singular blocks set `info` (int32 tensor)."""
    return _check(load().gbmv_chem_newton_async(chem.c, t, _dev_ptr(y), _dev_ptr(f), _dev_ptr(x),
                                                gamma, time_units, lu_precision, refine,
                                                info.data_ptr(), _stream_ptr(stream)),
                  "gbmv_chem_newton_async")


def chem_newton_queue_async(chem: Chem, t, y, f, x, gamma, time_units, info, queue,
                            blocks_per_sm=0, lu_precision=FP64, refine=4, stream=None):
    """gbmv_chem_newton_queue_async: the fused Newton over 32-cell chunks taken from `queue`
    (a zeroed CUDA int64 tensor of one element, shared by the launches that split the cells)."""
    import torch
    if queue.dtype != torch.int64 or not queue.is_cuda or queue.numel() < 1:
        raise GbmvError("queue must be a CUDA int64 tensor")
    return _check(load().gbmv_chem_newton_queue_async(chem.c, t, _dev_ptr(y), _dev_ptr(f),
                                                      _dev_ptr(x), gamma, time_units,
                                                      lu_precision, refine, queue.data_ptr(),
                                                      blocks_per_sm, info.data_ptr(),
                                                      _stream_ptr(stream)),
                  "gbmv_chem_newton_queue_async")


def ffast(hydro: Hydro, chem: Chem, t, w, wdot, time_units, forcing=(), tshift=0.0, tscale=1.0,
          stream=None):
    """ffast (src/multirate_chem_hydro_main.cpp:897): chemistry RHS times TimeUnits on the
    chemistry component, zero fluid tendencies, plus the MRI forcing sum_i tau^i forcing[i]
    (each forcing[i] a ManyVector like w)."""
    nf = len(forcing)
    arr = (_VP * max(1, 6 * nf))()
    for i, fv in enumerate(forcing):
        for k, comp in enumerate(fv):
            arr[6 * i + k] = _dev_ptr(comp)
    return _check(load().gbmv_ffast(hydro.h, chem.c, t, _vec(w), _vec(wdot), time_units, nf,
                                    arr if nf else None, tshift, tscale, _stream_ptr(stream)),
                  "gbmv_ffast")


def mri_fast_evolve(hydro: Hydro, chem: Chem, t0, tout, w, time_units, forcing=(), tshift=0.0,
                    tscale=1.0, stats=None, stream=None, **opts) -> int:
    """RankLocalStepper_Evolve (src/multirate_chem_hydro_main.cpp:1114): advance the fast
    problem w' = ffast(t, w) (chemistry by the persistent DIRK with the forcing's chemistry
    component, fluid by the forcing's exact integral) from t0 to tout in place.  Returns the
    number of failed cells."""
    nf = len(forcing)
    arr = (_VP * max(1, 6 * nf))()
    for i, fv in enumerate(forcing):
        for k, comp in enumerate(fv):
            arr[6 * i + k] = _dev_ptr(comp)
    o = dirk_opts(**opts)
    return _check(load().gbmv_mri_fast_evolve(hydro.h, chem.c, t0, tout, _vec(w), time_units, nf,
                                              arr if nf else None, tshift, tscale, C.byref(o),
                                              stats.data_ptr() if stats is not None else None,
                                              _stream_ptr(stream)),
                  "gbmv_mri_fast_evolve", allow=range(0, chem.n + 1))


def mri_fast_evolve_async(hydro: Hydro, chem: Chem, t0, tout, w, time_units, nfail, forcing=(),
                          tshift=0.0, tscale=1.0, stats=None, stream=None, **opts) -> int:
    """gbmv_mri_fast_evolve_async: graph-capturable; failed cells added to nfail (CUDA int32);
    opts must fix `block` (or an earlier synchronous call must have tuned it)."""
    nf = len(forcing)
    arr = (_VP * max(1, 6 * nf))()
    for i, fv in enumerate(forcing):
        for k, comp in enumerate(fv):
            arr[6 * i + k] = _dev_ptr(comp)
    o = dirk_opts(**opts)
    return _check(load().gbmv_mri_fast_evolve_async(
        hydro.h, chem.c, t0, tout, _vec(w), time_units, nf, arr if nf else None, tshift, tscale,
        C.byref(o), stats.data_ptr() if stats is not None else None, nfail.data_ptr(),
        _stream_ptr(stream)), "gbmv_mri_fast_evolve_async")


def PostprocessStep(hydro: Hydro, chem: Chem, w, energy_units, stream=None):
    return _check(load().gbmv_postprocess_step(hydro.h, chem.c, _vec(w), energy_units,
                                               _stream_ptr(stream)), "gbmv_postprocess_step")


def convert_check(d) -> int:
    """Mismatches of the integer-instruction conversions against the hardware ones over the
    doubles of the CUDA tensor d (0 when they agree bit for bit)."""
    out = C.c_ulonglong(0)
    _check(load().gbmv_diag_convert_check(_dev_ptr(d), d.numel(), C.byref(out), None),
           "gbmv_diag_convert_check")
    return int(out.value)


def fma_rate(fp64: bool = True) -> float:
    """Measured peak FMA throughput (flop/s) of the FP64 or FP32 pipes."""
    v = C.c_double()
    _check(load().gbmv_diag_fma_rate(1 if fp64 else 0, C.byref(v)), "gbmv_diag_fma_rate")
    return v.value


def profile_enable(on: bool = True):
    _check(load().gbmv_profile_enable(1 if on else 0), "gbmv_profile_enable")


def profile_reset():
    _check(load().gbmv_profile_reset(), "gbmv_profile_reset")


def profile_get(family: str):
    """(total milliseconds, launches) recorded for a kernel family since the last reset."""
    ms, n = C.c_double(), C.c_long()
    _check(load().gbmv_profile_get(family.encode(), C.byref(ms), C.byref(n)), "gbmv_profile_get")
    return ms.value, n.value


def launch_count() -> int:
    return int(load().gbmv_launch_count())
