"""ctypes bindings for the CPU oracle (oracle/oracle.c) and, where it has been built, for the
reference's own code compiled against the one-rank shims (oracle/_ref, see build_ref.sh).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline legs, never by the product path.
"""
from __future__ import annotations

import ctypes as C
import concurrent.futures as cf
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")

_P = C.POINTER(C.c_double)


def build(force: bool = False) -> str:
    """Compile oracle.c into oracle/_build/liboracle.so (plain gcc, no FMA contraction)."""
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        os.makedirs(BUILD, exist_ok=True)
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-shared", src,
                               "-o", tmp, "-lm"])
        os.replace(tmp, LIB)
    return LIB


class OrcGrid(C.Structure):
    _fields_ = [("nx", C.c_long), ("ny", C.c_long), ("nz", C.c_long), ("nchem", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("gamma", C.c_double), ("bc", C.c_int * 6)]


class OrcChem(C.Structure):
    _fields_ = [("tables", _P), ("dbin", C.c_double), ("idbin", C.c_double),
                ("lb", C.c_double), ("nbins", C.c_int), ("tlo", C.c_double),
                ("thi", C.c_double), ("z", C.c_double)]


class OrcDirkOpts(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("t0", "tout", "tunit", "rtol", "atol", "nlscoef", "h0",
                                          "h0fac", "safety", "dgmax", "growth", "etamx1",
                                          "hmax")] + \
               [(k, C.c_int) for k in ("maxcor", "max_steps", "msbp", "maxnef", "maxncf",
                                       "nforcing")] + \
               [("tshift", C.c_double), ("tscale", C.c_double), ("fz", _P * 8),
                ("s", C.c_int), ("p", C.c_int), ("gamma", C.c_double), ("c", C.c_double * 7),
                ("a", (C.c_double * 7) * 7), ("e", C.c_double * 7), ("deduce", C.c_int)]


def _q(a, b):
    return float(a) / float(b)


def _dirk_tables():
    """The oracle's own copy of the two stiffly accurate ESDIRKs, by ARKODE table number, from
    the published coefficients (each rational as the double quotient of its integers):
    112 ARK4(3)7L[2]SA implicit part (Kennedy & Carpenter, Appl. Numer. Math. 136 (2019)
    183-205), 102 TR-BDF2 (Hosea & Shampine, Appl. Numer. Math. 20 (1996) 21-37).
    Returned as dicts of s, p, A (rows incl. the diagonal), c, b, bhat."""
    g = _q(1235, 10000)
    b = [0.0, 0.0, _q(9164257142617, 17756377923965), _q(-10812980402763, 74029279521829),
         _q(1335994250573, 5691609445217), _q(2273837961795, 8368240463276), _q(247, 2000)]
    A = [[0.0] * 7 for _ in range(7)]
    for i in range(1, 7):
        A[i][i] = g
    A[1][0] = g
    A[2][0] = A[2][1] = _q(624185399699, 4186980696204)
    A[3][0] = A[3][1] = _q(1258591069120, 10082082980243)
    A[3][2] = _q(-322722984531, 8455138723562)
    A[4][0] = A[4][1] = _q(-436103496990, 5971407786587)
    A[4][2] = _q(-2689175662187, 11046760208243)
    A[4][3] = _q(4431412449334, 12995360898505)
    A[5][0] = A[5][1] = _q(-2207373168298, 14430576638973)
    A[5][2] = _q(242511121179, 3358618340039)
    A[5][3] = _q(3145666661981, 7780404714551)
    A[5][4] = _q(5882073923981, 14490790706663)
    A[6][:6] = b[:6]
    ark437 = dict(s=7, p=3, A=A, b=b,
                  c=[0.0, _q(247, 1000), _q(4276536705230, 10142255878289), _q(67, 200),
                     _q(3, 40), _q(7, 10), 1.0],
                  bhat=[0.0, 0.0, _q(4469248916618, 8635866897933),
                        _q(-621260224600, 4094290005349), _q(696572312987, 2942599194819),
                        _q(1532940081127, 5565293938103), _q(2441, 20000)])
    rt2 = 1.4142135623730951
    gd, w = (2.0 - rt2) / 2.0, rt2 / 4.0
    trbdf2 = dict(s=3, p=3, A=[[0.0, 0.0, 0.0], [gd, gd, 0.0], [w, w, gd]], b=[w, w, gd],
                  c=[0.0, 2.0 - rt2, 1.0],
                  bhat=[(1.0 - w) / 3.0, (3.0 * w + 1.0) / 3.0, gd / 3.0])
    return {112: ark437, 102: trbdf2}


DIRK_TABLES = _dirk_tables()


# defaults of gbmv_dirk_opts_default (include/gbmv.h)
DIRK_DEFAULTS = dict(rtol=1e-6, atol=1e-10, nlscoef=0.1, h0=0.0, safety=0.9, dgmax=0.2,
                     growth=20.0, etamx1=10000.0, hmax=0.0, maxcor=3, max_steps=5000, msbp=20,
                     maxnef=7, maxncf=10, deduce=0)


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.orc_feuler.restype = C.c_int
        _lib.orc_block_newton_solve.restype = C.c_long
        _lib.orc_chem_dirk_evolve.restype = C.c_long
    return _lib


def grid(shape, nchem, bc, gamma=1.4, domain=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)):
    nx, ny, nz = shape
    g = OrcGrid()
    g.nx, g.ny, g.nz, g.nchem = nx, ny, nz, nchem
    # same expression as EulerData::SetupDecomp (src/euler3D.hpp:412-414)
    g.dx = (domain[1] - domain[0]) / nx
    g.dy = (domain[3] - domain[2]) / ny
    g.dz = (domain[5] - domain[4]) / nz
    g.gamma = gamma
    for i in range(6):
        g.bc[i] = bc[i]
    return g


def _threads(threads):
    return max(1, os.cpu_count() or 1) if threads in (None, 0) else max(1, int(threads))


def _chunks(n, parts):
    """[(lo, hi)] splitting range(n) into at most `parts` near-equal pieces."""
    parts = max(1, min(parts, n))
    edges = [n * i // parts for i in range(parts + 1)]
    return [(a, b) for a, b in zip(edges[:-1], edges[1:]) if b > a]


def feuler(fields, nchem, bc, gamma=1.4, force=None, domain=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0),
           threads=1):
    """fields: list of 5 arrays shaped (nz,ny,nx) and, if nchem>0, chem shaped (nz,ny,nx,nchem).
    Returns (status, list of output arrays of the same shapes).  threads > 1 (0 = every core)
    evaluates disjoint z-slabs of the output on that many threads (orc_feuler_slab; ctypes
    releases the interpreter lock during the calls); the values are those of one call."""
    nz, ny, nx = fields[0].shape
    g = grid((nx, ny, nz), nchem, bc, gamma, domain)
    ins = [np.ascontiguousarray(f, dtype=np.float64) for f in fields]
    outs = [np.zeros_like(f) for f in ins]
    inp = (_P * 6)(*[_ptr(a) for a in ins], *([None] * (6 - len(ins))))
    outp = (_P * 6)(*[_ptr(a) for a in outs], *([None] * (6 - len(outs))))
    fc = None
    if force is not None:
        fa = np.ascontiguousarray(force, dtype=np.float64)
        fc = _ptr(fa)
    nt = _threads(threads)
    if nt == 1:
        return lib().orc_feuler(C.byref(g), inp, outp, fc), outs
    L = lib()
    L.orc_feuler_slab.restype = C.c_int
    with cf.ThreadPoolExecutor(nt) as ex:
        sts = list(ex.map(lambda kk: L.orc_feuler_slab(C.byref(g), inp, outp, fc,
                                                       C.c_long(kk[0]), C.c_long(kk[1])),
                          _chunks(nz, 4 * nt)))
    st = -1 if any(sts) else 0
    if st:  # the whole-grid call writes nothing for an illegal state
        outs = [np.zeros_like(f) for f in ins]
    return st, outs


class Chem:
    """Oracle chemistry state: tables, per-cell scale/aux arrays and the temperature history."""

    def __init__(self, tables: np.ndarray, scale: np.ndarray, z: float = -1.0):
        self.tables = np.ascontiguousarray(tables, dtype=np.float64)
        self.c = OrcChem()
        lib().orc_chem_init(C.byref(self.c), _ptr(self.tables), C.c_double(z))
        self.scale = np.ascontiguousarray(scale, dtype=np.float64).reshape(-1)
        self.n = self.scale.size // 10
        self.inv_scale = 1.0 / self.scale
        self.mdens = np.zeros(self.n)
        self.imdens = np.zeros(self.n)
        self.cie = np.zeros(self.n)
        self.h2 = np.zeros(self.n)
        lib().orc_chem_aux(_ptr(self.scale), C.c_long(self.n), _ptr(self.mdens),
                           _ptr(self.imdens), _ptr(self.cie), _ptr(self.h2))
        self.Ts = np.full(self.n, 1000.0)
        self.dTs_ge = np.zeros(self.n)

    def _per_cell(self, fn, threads):
        """fn(lo, hi) over cell ranges, on `threads` threads (0 = every core).  The network is
        per cell (each cell reads and writes only its own entries), so chunks are disjoint."""
        nt = _threads(threads)
        if nt == 1:
            fn(0, self.n)
            return
        with cf.ThreadPoolExecutor(nt) as ex:
            list(ex.map(lambda r: fn(*r), _chunks(self.n, 4 * nt)))

    def rhs(self, y: np.ndarray, threads=1) -> np.ndarray:
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1)
        yd = np.zeros_like(y)
        L = lib()

        def part(a, b):
            L.orc_chem_rhs(C.byref(self.c), C.c_long(b - a), _ptr(y[10 * a:10 * b]),
                           _ptr(self.scale[10 * a:10 * b]), _ptr(self.inv_scale[10 * a:10 * b]),
                           _ptr(self.mdens[a:b]), _ptr(self.imdens[a:b]), _ptr(self.cie[a:b]),
                           _ptr(self.h2[a:b]), _ptr(self.Ts[a:b]), _ptr(self.dTs_ge[a:b]),
                           _ptr(yd[10 * a:10 * b]))
        self._per_cell(part, threads)
        return yd

    def jac(self, y: np.ndarray, threads=1) -> np.ndarray:
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1)
        J = np.zeros(self.n * 100)
        L = lib()

        def part(a, b):
            L.orc_chem_jac(C.byref(self.c), C.c_long(b - a), _ptr(y[10 * a:10 * b]),
                           _ptr(self.scale[10 * a:10 * b]), _ptr(self.inv_scale[10 * a:10 * b]),
                           _ptr(self.mdens[a:b]), _ptr(self.cie[a:b]), _ptr(self.h2[a:b]),
                           _ptr(self.Ts[a:b]), _ptr(self.dTs_ge[a:b]), _ptr(J[100 * a:100 * b]))
        self._per_cell(part, threads)
        return J.reshape(self.n, 10, 10)  # [cell][col][row]

    def dirk_evolve(self, y: np.ndarray, t0: float, tout: float, tunit: float, forcing=(),
                    tshift=0.0, tscale=1.0, table=112, **opts):
        """Per-cell adaptive ESDIRK integration from t0 to tout (orc_chem_dirk_evolve) with the
        table of ARKODE number `table` (112 ARK4(3)7L[2]SA, 102 TR-BDF2), with the MRI forcing
        sum_i tau^i forcing[i] (chemistry components) added to the RHS.
        Returns (y(tout), stats[n, 8], number of failed cells); Ts / dTs_ge carried."""
        o = dict(DIRK_DEFAULTS, **opts)
        O = OrcDirkOpts()
        T = DIRK_TABLES[table]
        O.s, O.p, O.gamma = T["s"], T["p"], T["A"][1][1]
        for i in range(T["s"]):
            O.c[i] = T["c"][i]
            O.e[i] = T["b"][i] - T["bhat"][i]
            for j in range(T["s"]):
                O.a[i][j] = T["A"][i][j]
        O.t0, O.tout, O.tunit = t0, tout, tunit
        keep = [np.ascontiguousarray(f, dtype=np.float64).reshape(-1) for f in forcing]
        O.nforcing, O.tshift, O.tscale = len(keep), tshift, tscale
        for q, f in enumerate(keep):
            O.fz[q] = _ptr(f)
        for k, v in o.items():
            setattr(O, k, v)
        O.h0fac = 0.5 * o["rtol"] ** (-2.0 / 3.0)
        y = np.array(y, dtype=np.float64).reshape(-1)
        stats = np.zeros((self.n, 8), dtype=np.int32)
        nf = lib().orc_chem_dirk_evolve(
            C.byref(self.c), C.c_long(self.n), _ptr(y), _ptr(self.scale), _ptr(self.inv_scale),
            _ptr(self.mdens), _ptr(self.imdens), _ptr(self.cie), _ptr(self.h2), _ptr(self.Ts),
            _ptr(self.dTs_ge), C.byref(O), stats.ctypes.data_as(C.POINTER(C.c_int)))
        return y, stats, int(nf)


def block_newton_solve(J: np.ndarray, gamma: float, b: np.ndarray, threads=1):
    """(I - gamma J_i) x_i = b_i per 10x10 block; returns (0 or 1 + first singular block, x)."""
    J = np.ascontiguousarray(J, dtype=np.float64).reshape(-1)
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
    x = np.zeros_like(b)
    n = b.size // 10
    L = lib()
    nt = _threads(threads)

    def part(r):
        a, e = r
        bad = L.orc_block_newton_solve(C.c_long(e - a), _ptr(J[100 * a:100 * e]),
                                       C.c_double(gamma), _ptr(b[10 * a:10 * e]),
                                       _ptr(x[10 * a:10 * e]))
        return a + bad if bad else 0
    if nt == 1:
        return int(part((0, n))), x
    with cf.ThreadPoolExecutor(nt) as ex:
        bads = [v for v in ex.map(part, _chunks(n, 4 * nt)) if v]
    return (int(min(bads)) if bads else 0), x


def fused_chem_hydro_step(fields, scale, chem, bc, gamma, energy_units, time_units,
                          newton_gamma, threads=1):
    """One fused chemistry-hydrodynamics stage over the oracle, the composition an IMEX /
    multirate stage calls (and the GPU's fused-step benchmark times):
      fexpl  (src/imex_chem_hydro_main.cpp:910-1000): physical chemistry = w5 * scale,
             et = ge / EnergyUnits + |m|^2 / (2 rho) written into the state, fEuler of all
             fields, the et tendency moved to the gas-energy slot (et tendency 0), w5 <-
             physical / scale (the reference's in-place scale / unscale round trip);
      fimpl  (:811-848) f = TimeUnits * f_chem(w5) (temperature state carried in `chem`);
      Jimpl  (:850-908) J = TimeUnits * df/dy, solved per block with I - newton_gamma J
             (the BDMPIMV solver, :1075-1194): x = (I - newton_gamma J)^{-1} f.
    `fields`: the six state arrays (modified in place: et and the chemistry round trip, as the
    GPU's FP64 form modifies them); `chem`: a Chem over `scale`.  Returns (status, [wdot_0..4,
    wdot_5, f, x]) with wdot_5 the chemistry tendency of the physical densities."""
    w = fields
    phys = w[5] * scale
    w[4][...] = phys[..., 9] * (1.0 / energy_units) + 0.5 / w[0] * (
        w[1] * w[1] + w[2] * w[2] + w[3] * w[3])
    st, out = feuler(list(w[:5]) + [phys], 10, bc, gamma, None, threads=threads)
    if st != 0:
        return st, None
    out[5][..., 9] = out[4]
    out[4][...] = 0.0
    w[5][...] = phys / scale
    y = w[5].reshape(-1)
    f = chem.rhs(y, threads) * time_units
    J = chem.jac(y, threads) * time_units
    bad, x = block_newton_solve(J, newton_gamma, f, threads)
    if bad:
        return 1, None
    return 0, out + [f, x]


class ImexChemHydro:
    """The IMEX callbacks of src/imex_chem_hydro_main.cpp over the oracle, in the problem
    protocol of the package's ARK-IMEX driver (fe, fi, setup, solve, norm, postprocess):
    fexpl (:910-1000: et from the physical gas energy, fEuler on the physical chemistry, the et
    tendency moved to the gas-energy slot, the in-place scale / unscale round trip of the
    chemistry component), its chemistry tendency converted to the scaled variables (species
    / scale, gas energy x EnergyUnits / scale) when forcing_units is "scaled", unconverted as
    the reference adds it when "reference"; fimpl (:811-848, TimeUnits x the source);
    Jimpl (:850-908, TimeUnits x J) with I - gamma J solved per block by orc_block_newton_solve
    (the BDMPIMV solver, :1075-1194); PostprocessStep (:1002-1051); WRMS norms with weights
    1 / (rtol |y| + atol).  `wl` holds bc, gamma and the per-entry scale."""

    def __init__(self, wl, tables, eu, tu, rtol, atol, forcing_units="reference"):
        self.forcing_units = forcing_units
        self.wl, self.eu, self.tu = wl, eu, tu
        self.rtol, self.atol = rtol, atol
        self.scale = wl["scale"]
        self.oc = Chem(tables, self.scale.reshape(-1))
        self.inv = 1.0 / self.scale
        self.J, self.g = None, None

    def _sync(self, y):
        phys = y[5] * self.scale
        y[4][...] = phys[..., 9] * (1.0 / self.eu) + 0.5 / y[0] * (
            y[1] * y[1] + y[2] * y[2] + y[3] * y[3])
        return phys

    def fe(self, t, y):
        phys = self._sync(y)
        st, out = feuler(y[:5] + [phys], 10, self.wl["bc"], self.wl["gamma"], None)
        if st != 0:
            raise RuntimeError("fexpl: illegal state")
        out[5][..., 9] = out[4]
        out[4][:] = 0.0
        y[5][...] = phys / self.scale
        if self.forcing_units == "scaled":
            out[5][..., :9] = out[5][..., :9] * self.inv[..., :9]
            out[5][..., 9] = out[5][..., 9] * (self.inv[..., 9] * self.eu)
        return out

    def fi(self, t, y):
        f = self.oc.rhs(y[5].reshape(-1)) * self.tu
        return [None] * 5 + [f.reshape(y[5].shape)]

    def setup(self, t, y, gamma):
        self.J = self.oc.jac(y[5].reshape(-1)) * self.tu
        self.g = gamma
        return 0

    def solve(self, b):
        bad, x = block_newton_solve(self.J, self.g, b[5].reshape(-1))
        if bad:
            raise RuntimeError("singular Newton block")
        return list(b[:5]) + [x.reshape(b[5].shape)]

    def norm(self, v, y):
        s = sum(float(((a * (1.0 / (self.rtol * np.abs(w) + self.atol))) ** 2).sum())
                for a, w in zip(v, y))
        return math.sqrt(s / sum(w.size for w in y))

    def postprocess(self, t, y):
        phys = self._sync(y)
        y[5][...] = phys / self.scale


# ---------------------------------------------------------------- reference build (here only)

def ref_available(nvar: int = 5) -> bool:
    return os.path.exists(os.path.join(REF, f"libref_nvar{nvar}.so"))


_ref_libs: dict[int, C.CDLL] = {}


def ref_lib(nvar: int):
    if nvar not in _ref_libs:
        path = os.path.join(REF, f"libref_nvar{nvar}.so")
        L = C.CDLL(path)
        L.ref_feuler.restype = C.c_int
        L.ref_chem_setup.restype = C.c_int
        L.ref_chem_rhs.restype = C.c_int
        L.ref_chem_jac.restype = C.c_int
        _ref_libs[nvar] = L
    return _ref_libs[nvar]


def ref_feuler(fields, nchem, bc, gamma=1.4, force=None, domain=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)):
    nz, ny, nx = fields[0].shape
    L = ref_lib(5 + nchem)
    ins = [np.ascontiguousarray(f, dtype=np.float64) for f in fields]
    outs = [np.zeros_like(f) for f in ins]
    inp = (_P * 6)(*[_ptr(a) for a in ins], *([None] * (6 - len(ins))))
    outp = (_P * 6)(*[_ptr(a) for a in outs], *([None] * (6 - len(outs))))
    dom = (C.c_double * 6)(*domain)
    bca = (C.c_int * 6)(*bc)
    fc = None
    if force is not None:
        fa = np.ascontiguousarray(force, dtype=np.float64)
        fc = _ptr(fa)
    sec = C.c_double()
    st = L.ref_feuler(C.c_long(nx), C.c_long(ny), C.c_long(nz), dom, bca, C.c_double(gamma),
                      C.c_double(0.0), fc, inp, outp, C.byref(sec))
    return st, outs


class RefChem:
    """The reference's chemistry network (compiled from its own source) with the same API."""

    def __init__(self, table_file: str, scale: np.ndarray, z: float = -1.0, nvar: int = 15):
        self.L = ref_lib(nvar)
        self.scale = np.ascontiguousarray(scale, dtype=np.float64).reshape(-1)
        self.n = self.scale.size // 10
        st = self.L.ref_chem_setup(table_file.encode(), C.c_long(self.n), _ptr(self.scale),
                                   C.c_double(z))
        if st != 0:
            raise RuntimeError("ref_chem_setup failed")

    def state(self):
        out = [np.zeros(self.n) for _ in range(5)]
        self.L.ref_chem_get_state(*[_ptr(a) for a in out])
        return dict(zip(["Ts", "dTs_ge", "mdens", "cie", "h2"], out))

    def set_Ts(self, Ts):
        Ts = np.ascontiguousarray(Ts, dtype=np.float64)
        self.L.ref_chem_set_Ts(_ptr(Ts))

    def rhs(self, y):
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1).copy()
        yd = np.zeros_like(y)
        self.L.ref_chem_rhs(C.c_double(0.0), _ptr(y), _ptr(yd), None)
        return yd

    def jac(self, y):
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1).copy()
        J = np.zeros(self.n * 100)
        self.L.ref_chem_jac(C.c_double(0.0), _ptr(y), _ptr(J), None)
        return J.reshape(self.n, 10, 10)


class RefGlue:
    """The reference's IMEX-program glue compiled from its own source (oracle/_ref/
    libref_glue.so, see ref_glue.cpp): fexpl, PostprocessStep and the static problem's Dengo
    scaling on one grid.  `scale` (10 per cell, the physical chemistry) goes through
    prepare_Dengo_structures; fields are [rho, mx, my, mz, et, chem] arrays."""

    def __init__(self, shape, bc, gamma, units, scale, table_dir):
        path = os.path.join(REF, "libref_glue.so")
        self.L = C.CDLL(path)
        self.L.ref_glue_energy_units.restype = C.c_double
        nz, ny, nx = shape
        phys = np.ascontiguousarray(scale, dtype=np.float64).reshape(-1).copy()
        st = self.L.ref_glue_setup(C.c_long(nx), C.c_long(ny), C.c_long(nz),
                                   (C.c_int * 6)(*bc), C.c_double(gamma),
                                   C.c_double(units["MassUnits"]),
                                   C.c_double(units["LengthUnits"]),
                                   C.c_double(units["TimeUnits"]), table_dir.encode(),
                                   _ptr(phys))
        if st != 0:
            raise RuntimeError(f"ref_glue_setup failed ({st})")
        self.prepared_chem = phys  # ones, as prepare_Dengo_structures leaves the solution

    @staticmethod
    def _arr(fields):
        return (C.c_void_p * 6)(*[f.ctypes.data for f in fields])

    def energy_units(self):
        return self.L.ref_glue_energy_units()

    def fexpl(self, t, fields):
        """(status, wdot); `fields` modified in place as the reference modifies them."""
        out = [np.zeros_like(f) for f in fields]
        st = self.L.ref_glue_fexpl(C.c_double(t), self._arr(fields), self._arr(out))
        return st, out

    def postprocess(self, t, fields):
        return self.L.ref_glue_postprocess(C.c_double(t), self._arr(fields))

    def scaling(self, fields, apply):
        return self.L.ref_glue_scaling(self._arr(fields), int(bool(apply)))
