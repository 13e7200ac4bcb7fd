"""The reference's input-file drivers over the drop-in entry points.

An input file in the reference's format -- `key = value` lines and '#' comments, read as
load_inputs reads them (src/io.cpp:226-298) -- with keyword overrides taking precedence as its
command-line options do (src/io.cpp:301-365), configures one of its three main programs:

  run_euler      src/euler3D_main.cpp               ERK hydrodynamics (fEuler = gbmv_feuler)
  run_imex       src/imex_chem_hydro_main.cpp       ARK-IMEX chemistry-hydrodynamics
  run_multirate  src/multirate_chem_hydro_main.cpp  MRI chemistry-hydrodynamics

each with the reference's output loop (src/euler3D_main.cpp:296-416): nout equal intervals
from t0 to tf; at t0 and after every interval the solution file output-%07i.hdf5 together
with restart_parameters.txt (output_solution, src/io.cpp:723), and with `showstats` the
conservation totals (check_conservation, src/io.cpp:504) and per-field RMS values
(print_stats, src/io.cpp:552) on the device.  `restart = r` (as written into
restart_parameters.txt) resumes from output-%07i.hdf5 number r (read_restart, src/io.cpp:946).

Initial conditions belong to the problem files (src/sod.cpp, src/rayleigh_taylor.cpp,
src/primordial_blast.cpp, ...); the caller passes `problem(inputs)`, returning a dict with
  fields  [rho, mx, my, mz, et, chem]: host arrays in code units, fluid [nz][ny][nx], chem
          [nz][ny][nx][nchem] (None for pure hydrodynamics);
  scale   (chemistry drivers) the Dengo scale, [nz][ny][nx][10], fields[5] holding the scaled
          values (prepare_Dengo_scaling, src/primordial_static.cpp:227);
  force   optional constant external force, 5 + nchem values (external_forces).

Methods: the reference selects SUNDIALS tables through order / etable / itable / mtable, and
so do these drivers, with the tables of gbmv_butcher_table (SUNDIALS is absent here; the host
integrators of integrate.py run them):
  run_euler      order != 0: ARKODE's default explicit table of that order (2 Heun-Euler,
                 3 Bogacki-Shampine, 4 Zonneveld, 5 Cash-Karp); else etable >= 0: that table;
                 else the order-4 default (src/euler3D_main.cpp:207-213);
  run_imex       ARKStepSetTableNum(itable, etable) (src/imex_chem_hydro_main.cpp:386): both
                 an additive pair (13 + 112 = ARK4(3)7L[2]SA, the primordial inputs'; 2 + 104 =
                 ARK3(2)4L[2]SA), itable alone a DIRK on the chemistry only, etable alone an ERK;
  run_multirate  the inner (fast) DIRK of itable (112 or 102; src/multirate_chem_hydro_main.
                 cpp:446-449), the slow coupling of mtable by SUNDIALS' ARKODE_MRITableID
                 numbers: -1 (MRIStep's default third-order explicit coupling) or 200 ->
                 MIS-KW3, 201 -> MRI-GARK-ERK33a.
Unknown table numbers are refused with ValueError.  adapt_method (0 PID, 1 PI, 2 I), k1-k3,
pq, safety, bias, growth, etamx1, etamxf and maxnef set ARKODE's step controller.  Options the
host integrators do not have (dense_order, mxhnil, hmin, predictor, fusedkernels,
localreduce) are read and written back unchanged but do not alter the run; a zero option
means "the integrator's default", as in the reference.  The chemistry drivers add the slow
(fexpl / fslow) chemistry tendency to the scaled chemistry unconverted, as the reference does
(forcing_units="reference"); forcing_units="scaled" converts it first (integrate.mri_evolve).
"""
from __future__ import annotations

import math
import re
import sys

import h5io
import integrate as I

# EulerData defaults (src/euler3D.hpp:277-287) of the keys load_inputs reads
UDATA_DEFAULTS = {
    "xl": 0.0, "xr": 1.0, "yl": 0.0, "yr": 1.0, "zl": 0.0, "zr": 1.0, "t0": 0.0, "tf": 1.0,
    "gamma": 1.4, "MassUnits": 1.0, "LengthUnits": 1.0, "TimeUnits": 1.0,
    "nx": 3, "ny": 3, "nz": 3, "xlbc": 0, "xrbc": 0, "ylbc": 0, "yrbc": 0, "zlbc": 0, "zrbc": 0,
    "cfl": 0.0, "nout": 10, "showstats": 0,
}
# ARKODEParameters defaults (src/euler3D.hpp:160-167) of the keys load_inputs reads
OPTS_DEFAULTS = {
    "order": 4, "dense_order": -1, "etable": -1, "itable": -1, "mtable": -1, "adapt_method": 0,
    "maxnef": 0, "mxhnil": 0, "mxsteps": 5000, "safety": 0.0, "bias": 0.0, "growth": 0.0,
    "pq": 0, "k1": 0.0, "k2": 0.0, "k3": 0.0, "etamx1": 0.0, "etamxf": 0.0, "h0": 0.0,
    "hmin": 0.0, "hmax": 0.0, "fixedstep": 0, "htrans": 0.0, "predictor": 0, "maxniters": 0,
    "nlconvcoef": 0.0, "rtol": 1e-8, "atol": 1e-12, "fusedkernels": 1, "localreduce": 1,
}
_INT_KEYS = {k for k, v in {**UDATA_DEFAULTS, **OPTS_DEFAULTS}.items() if isinstance(v, int)}
_INT_KEYS.add("restart")
_FLOAT = re.compile(r"[+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan)",
                    re.IGNORECASE)
_INT = re.compile(r"[+-]?(?:0[xX][0-9a-fA-F]+|0[0-7]*|[1-9][0-9]*)")


def _scan(text: str, integer: bool):
    """The value sscanf's %i / %lf reads from the start of `text` (None when it reads none):
    %i takes decimal, 0x hexadecimal and 0-prefixed octal; both stop at the first character
    that cannot continue the number."""
    text = text.lstrip()
    m = (_INT if integer else _FLOAT).match(text)
    if not m:
        return None
    tok = m.group(0)
    if not integer:
        return float(tok)
    sign = -1 if tok[0] == "-" else 1
    digits = tok.lstrip("+-")
    if digits[:2].lower() == "0x":
        return sign * int(digits, 16)
    if len(digits) > 1 and digits[0] == "0":
        return sign * int(digits, 8)
    return sign * int(digits)


def _match(line: str, key: str):
    """The text after '=' when `line` matches the sscanf format "key = ...": the key at the
    start of the line, any blanks, '='."""
    if not line.startswith(key):
        return None
    rest = line[len(key):].lstrip()
    return rest[1:] if rest.startswith("=") else None


class Inputs:
    """Parsed run parameters: `u` (EulerData fields), `o` (ARKODEParameters fields),
    `restart` (-1: start from the problem's initial conditions), `warnings` (lines with '='
    that no key read, which load_inputs reports on stderr)."""

    def __init__(self, u, o, restart, warnings):
        self.u, self.o, self.restart, self.warnings = u, o, restart, warnings

    def params(self) -> dict:
        """Every key of restart_parameters.txt, for h5io.write_parameters."""
        return {**self.u, **self.o, "restart": self.restart}

    @property
    def shape(self):
        return (self.u["nz"], self.u["ny"], self.u["nx"])

    @property
    def bc(self):
        u = self.u
        return (u["xlbc"], u["xrbc"], u["ylbc"], u["yrbc"], u["zlbc"], u["zrbc"])

    @property
    def domain(self):
        u = self.u
        return (u["xl"], u["xr"], u["yl"], u["yr"], u["zl"], u["zr"])

    def field_units(self):
        u = self.u
        return h5io.units(u["MassUnits"], u["LengthUnits"], u["TimeUnits"])


def load_inputs(path: str | None = None, **overrides) -> Inputs:
    """load_inputs (src/io.cpp:43-470) for one process: defaults, then the file's lines, then
    the keyword overrides (the command-line options).  Raises ValueError for an unknown
    override, non-positive units or nout, and fixed stepping without hmax > 0 (as the drivers
    refuse it, src/euler3D_main.cpp, src/imex_chem_hydro_main.cpp:186-190)."""
    u, o = dict(UDATA_DEFAULTS), dict(OPTS_DEFAULTS)
    restart = -1
    warnings = []
    keys = list(UDATA_DEFAULTS) + list(OPTS_DEFAULTS) + ["restart"]
    if path is not None:
        with open(path) as fh:
            for line in fh:
                read = 0
                for key in keys:
                    rest = _match(line, key)
                    if rest is None:
                        continue
                    v = _scan(rest, key in _INT_KEYS)
                    if v is None:
                        continue
                    read += 1
                    if key in u:
                        u[key] = v
                    elif key in o:
                        o[key] = v
                    else:
                        restart = v
                if read == 0 and "=" in line and not line.startswith("#"):
                    warnings.append(line.rstrip("\n"))
                    print("load_inputs Warning: parameter line was not interpreted:\n" + line,
                          end="" if line.endswith("\n") else "\n", file=sys.stderr)
    for key, v in overrides.items():
        if key in u:
            u[key] = int(v) if key in _INT_KEYS else float(v)
        elif key in o:
            o[key] = int(v) if key in _INT_KEYS else float(v)
        elif key == "restart":
            restart = int(v)
        else:
            raise ValueError(f"unknown option {key}")
    if min(u["MassUnits"], u["LengthUnits"], u["TimeUnits"]) <= 0.0:
        raise ValueError("MassUnits, LengthUnits and TimeUnits must be positive")
    if u["nout"] < 1:
        raise ValueError("nout must be at least 1")
    if o["fixedstep"] and o["hmax"] <= 0.0:
        raise ValueError(f"fixed time stepping requires hmax > 0 ({o['hmax']} given)")
    return Inputs(u, o, restart, warnings)


class RunResult:
    def __init__(self):
        self.t = 0.0                # final time
        self.h = 0.0                # step size at the last output
        self.outputs = []           # solution files written, in order
        self.conservation = []      # (t, total mass, total energy) per output (showstats)
        self.field_rms = []         # (t, per-field RMS in CGS units) per output (showstats)
        self.steps = 0              # integrator steps (slow steps for MRI)
        self.intervals = []         # per-interval integrator statistics objects


def _opt(value, default):
    """A zero option means the integrator's default."""
    return value if value > 0 else default


def _output_loop(inp: Inputs, hydro, w, t0: float, h0: float, outdir: str, evolve, log,
                 transient=None):
    """The shared loop: first batch at t0 (the restart file records opts.h0, as the reference
    writes it there), then nout intervals; evolve(t, tout, h) advances w in place from the
    step size h and returns (t, h_next, stats, steps); transient(t) -> t, when given, runs
    between the first batch and the first interval (fixedstep with htrans)."""
    u = inp.u
    res = RunResult()
    fu = inp.field_units()
    dx = (u["xr"] - u["xl"]) / u["nx"]
    dy = (u["yr"] - u["yl"]) / u["ny"]
    dz = (u["zr"] - u["zl"]) / u["nz"]
    vol = dx * dy * dz * u["LengthUnits"] ** 3
    first = []

    def report(t):
        if not u["showstats"]:
            return
        mass, energy = hydro.check_conservation(w, vol * fu[0], vol * fu[2])
        res.conservation.append((t, mass, energy))
        if not first:
            first.append((mass, energy))
            log(f"   Total mass   = {mass: .16e}")
            log(f"   Total energy = {energy: .16e}")
        else:
            m0, e0 = first[0]
            log(f"   Mass conservation relative change   = {abs(mass - m0) / m0:7.2e}")
            log(f"   Energy conservation relative change = {abs(energy - e0) / e0:7.2e}")
        rms = hydro.print_stats(w, fu)
        res.field_rms.append((t, rms))
        log(f"   t = {t:.6e}  rms = " + "  ".join(f"{v:.6e}" for v in rms))

    start = max(inp.restart, 0)
    t, h = t0, h0
    report(t)
    res.outputs.append(h5io.write_solution(outdir, start, t, w, inp.domain, fu))
    h5io.write_parameters(outdir, inp.params(), t, inp.o["h0"], start)
    dtout = (u["tf"] - t0) / u["nout"]
    tout = t0 + dtout
    if transient is not None:
        t = transient(t)
    for iout in range(start, start + u["nout"]):
        t, h, st, steps = evolve(t, tout, h)
        res.steps += steps
        res.intervals.append(st)
        tout = min(tout + dtout, u["tf"])
        report(t)
        res.outputs.append(h5io.write_solution(outdir, iout + 1, t, w, inp.domain, fu))
        h5io.write_parameters(outdir, inp.params(), t, h, iout + 1)
    res.t, res.h = t, h
    return res


def _initial_state(inp: Inputs, problem, nchem_needed, restart_dir):
    """(t0, host fields, problem dict) from the problem or, with restart >= 0, from
    output-%07i.hdf5 in restart_dir (the problem still supplies scale and force)."""
    pr = problem(inp)
    fields = list(pr["fields"]) + [None] * (6 - len(pr["fields"]))
    nchem = 0 if fields[5] is None else int(fields[5].shape[-1])
    if nchem_needed is not None and nchem != nchem_needed:
        raise ValueError(f"this driver needs {nchem_needed} chemical species ({nchem} given)")
    if fields[0].shape != inp.shape:
        raise ValueError(f"initial conditions of shape {fields[0].shape}, inputs {inp.shape}")
    t0 = inp.u["t0"]
    if inp.restart >= 0:
        t0, fields = h5io.read_restart(restart_dir, inp.restart, nchem, inp.domain, inp.shape,
                                       inp.field_units())
    return t0, fields, nchem, pr


def run_euler(inp: Inputs, problem, outdir: str = ".", restart_dir: str | None = None,
              precision: int | None = None, log=print) -> RunResult:
    """euler3D_main: adaptive ERK (or fixed steps of hmax with fixedstep, after an adaptive
    transient of htrans when given) of w' = fEuler(t, w), CFL-limited when cfl > 0, on the
    device; the loop of outputs above.  precision: gbmv.FP64 (default) or a mixed form."""
    import numpy as np
    import torch
    import gbmv
    gbmv.load()
    o = inp.o
    t0, fields, nchem, pr = _initial_state(inp, problem, None, restart_dir or outdir)
    prec = gbmv.FP64 if precision is None else precision
    hydro = gbmv.Hydro(inp.shape[::-1], nchem, inp.bc, inp.u["gamma"], force=pr.get("force"),
                       domain=inp.domain)
    n = int(np.prod(inp.shape))
    sizes = [n] * 5 + ([nchem * n] if nchem else [])
    y = torch.empty(sum(sizes), dtype=torch.float64, device="cuda")
    ydot = torch.empty_like(y)

    def split(v):
        parts = list(torch.split(v, sizes))
        out = [p.view(inp.shape) for p in parts[:5]]
        if nchem:
            out.append(parts[5].view(inp.shape + (nchem,)))
        return out

    w = split(y)
    for k in range(len(w)):
        w[k].copy_(torch.from_numpy(np.ascontiguousarray(fields[k], dtype=np.float64)))
    wdot = split(ydot)

    def rhs(t, v):
        if hydro.fEuler(t, split(v), wdot, prec) != 0:
            raise RuntimeError("fEuler: illegal state (solver failure, stopping integration)")
        return ydot.clone()

    cfl = inp.u["cfl"]
    stab = (lambda t, v: hydro.stability(split(v), cfl)) if cfl > 0 else None
    rtol, atol = o["rtol"], o["atol"]
    hmax = _opt(o["hmax"], math.inf)
    fixed = o["fixedstep"] != 0
    common = dict(max_steps=_opt(o["mxsteps"], 500), stability=stab, table=erk_table(o),
                  **_adapt(o))

    def evolve(t, tout, h):
        yt, st = I.erk_evolve(rhs, t, tout, y, rtol, atol, h0=h, hmax=hmax,
                              fixed_h=o["hmax"] if fixed else 0.0, **common)
        y.copy_(yt)
        return tout, st.h_next, st, st.steps

    def transient(t):  # adaptive over (t0, t0 + htrans], then fixed steps of hmax
        yt, _ = I.erk_evolve(rhs, t, t + o["htrans"], y, rtol, atol, h0=o["h0"], hmax=hmax,
                             **common)
        y.copy_(yt)
        return t + o["htrans"]

    h0 = o["hmax"] if fixed else o["h0"]
    return _output_loop(inp, hydro, w, t0, h0, outdir, evolve, log,
                        transient if (fixed and o["htrans"] > 0.0) else None)


def erk_table(o) -> int:
    """The explicit table euler3D_main selects: `order` overrides `etable`
    (src/euler3D_main.cpp:207-213); neither set -> ARKStep's order-4 default."""
    import gbmv
    if o["order"] != 0:
        tid = gbmv.erk_default_table(o["order"])
        if tid < 0:
            raise ValueError(f"order {o['order']}: no explicit table of that order here (2-5)")
        return tid
    tid = o["etable"] if o["etable"] >= 0 else gbmv.erk_default_table(4)
    gbmv.butcher_table(tid)  # refuses unknown numbers
    return tid


def _adapt(o) -> dict:
    """ARKODE step-controller options of the inputs (zero = the controller's default)."""
    kw = {"adapt_method": o["adapt_method"], "pq": o["pq"]}
    for key in ("k1", "k2", "k3", "safety", "bias", "growth", "etamx1", "etamxf"):
        if o[key] > 0:
            kw[key] = o[key]
    if o["maxnef"] > 0:
        kw["maxnef"] = o["maxnef"]
    return kw


def _chem_setup(inp: Inputs, problem, restart_dir, tables):
    import numpy as np
    import torch
    import gbmv
    gbmv.load()
    t0, fields, nchem, pr = _initial_state(inp, problem, 10, restart_dir)
    hydro = gbmv.Hydro(inp.shape[::-1], 10, inp.bc, inp.u["gamma"], force=pr.get("force"),
                       domain=inp.domain)
    chem = gbmv.Chem(int(np.prod(inp.shape)), tables)
    chem.set_scale(torch.from_numpy(np.ascontiguousarray(pr["scale"]).reshape(-1)).cuda())
    w = [torch.from_numpy(np.ascontiguousarray(f, dtype=np.float64)).cuda() for f in fields]
    return t0, hydro, chem, w


def run_imex(inp: Inputs, problem, tables, outdir: str = ".", restart_dir: str | None = None,
             precision: int | None = None, fused_newton: bool = False,
             forcing_units: str = "reference", log=print) -> RunResult:
    """imex_chem_hydro_main: ARK-IMEX with fe = fexpl and fi = fimpl, the block-diagonal
    direct solver, PostprocessStep after every step (integrate.ChemHydroImex), the method of
    ARKStepSetTableNum(itable, etable); rtol, atol, h0, hmax, fixedstep, the controller options,
    maxnef, maxniters (maxcor), nlconvcoef (nlscoef) and mxsteps as ARKStep takes them.
    tables: the 50 x 1024 rate table block (h5tables.load_table_block)."""
    import gbmv
    o = inp.o
    table = I.ark_table(o["etable"], o["itable"])  # refuses what ARKStepSetTableNum refuses
    t0, hydro, chem, w = _chem_setup(inp, problem, restart_dir or outdir, tables)
    u = inp.u
    eu = inp.field_units()[2]
    prec = gbmv.FP64 if precision is None else precision
    prob = I.ChemHydroImex(gbmv, hydro, chem, eu, u["TimeUnits"], o["rtol"], o["atol"], prec,
                           fused_newton=fused_newton, forcing_units=forcing_units)
    kw = dict(rtol=o["rtol"], atol=o["atol"], hmax=_opt(o["hmax"], math.inf),
              fixed_h=o["hmax"] if o["fixedstep"] else 0.0,
              max_steps=_opt(o["mxsteps"], 500), table=table, **_adapt(o))
    for key, name in (("maxniters", "maxcor"), ("nlconvcoef", "nlscoef")):
        if o[key] > 0:
            kw[name] = o[key]

    def evolve(t, tout, h):
        st = I.ark_imex_evolve(prob, t, tout, w, h0=h, **kw)
        return tout, st.h_next, st, st.steps

    def transient(t):  # adaptive over (t0, t0 + htrans], then fixed steps of hmax
        I.ark_imex_evolve(prob, t, t + o["htrans"], w, h0=o["h0"],
                          **{**kw, "fixed_h": 0.0})
        return t + o["htrans"]

    fixed = o["fixedstep"] != 0
    return _output_loop(inp, hydro, w, t0, o["hmax"] if fixed else o["h0"], outdir, evolve, log,
                        transient if (fixed and o["htrans"] > 0.0) else None)


MRI_TABLES = {-1: I.MRI_KW3, 200: I.MRI_KW3, 201: I.MRI_ERK33A}


def run_multirate(inp: Inputs, problem, tables, outdir: str = ".",
                  restart_dir: str | None = None, precision: int | None = None,
                  forcing_units: str = "reference", log=print) -> RunResult:
    """multirate_chem_hydro_main: MRI with a fixed slow step h0 (dTout when h0 is 0,
    src/multirate_chem_hydro_main.cpp:222), slow RHS fexpl, fast stages by
    gbmv_mri_fast_evolve (per-cell DIRK with rtol, atol, maxniters, nlconvcoef, hmax, safety,
    growth, etamx1, maxnef, mxsteps as the inner ARKStep takes them).  A slow step that would
    pass an output time is shortened to end on it, as MRIStep's stop time does.  The inner
    integrator's fixed-step mode (fixedstep) is not available and is refused.  The inner DIRK
    is the one of itable (112 ARK4(3)7L[2]SA, as the reference's multirate inputs select, or
    102 TR-BDF2); itable -1 (ARKODE's default inner DIRK, SDIRK 5(3)4) is not available and is
    refused."""
    o, u = inp.o, inp.u
    if o["mtable"] not in MRI_TABLES:
        raise ValueError(f"mtable {o['mtable']} is not available (-1, 200 MIS-KW3, 201 ERK33a)")
    if o["itable"] not in (102, 112):
        raise ValueError(f"itable {o['itable']}: the inner DIRK must be 112 or 102")
    if o["fixedstep"]:
        raise ValueError("fixedstep: the per-cell fast integrator has adaptive steps only")
    import gbmv
    table = MRI_TABLES[o["mtable"]]
    t0, hydro, chem, w = _chem_setup(inp, problem, restart_dir or outdir, tables)
    eu = inp.field_units()[2]
    prec = gbmv.FP64 if precision is None else precision
    dtout = (u["tf"] - t0) / u["nout"]
    hslow = o["h0"] if o["h0"] > 0 else dtout
    fast = dict(rtol=o["rtol"], atol=o["atol"], itable=o["itable"])
    for key, name in (("maxniters", "maxcor"), ("nlconvcoef", "nlscoef"), ("hmax", "hmax"),
                      ("safety", "safety"), ("growth", "growth"), ("etamx1", "etamx1"),
                      ("maxnef", "maxnef"), ("mxsteps", "max_steps")):
        if o[key] > 0:
            fast[name] = o[key]

    def evolve(t, tout, h):
        steps, failed = 0, 0
        nfull = int(math.floor((tout - t) / hslow * (1.0 + 1e-12)))
        tm = t + nfull * hslow
        if nfull >= 1:
            r = I.mri_evolve(gbmv, hydro, chem, w, t, tm, hslow, eu, u["TimeUnits"], table,
                             prec, forcing_units=forcing_units, **fast)
            steps, failed = r.slow_steps, r.fast_failed_cells
        rem = tout - tm
        if rem > 1e-12 * max(abs(tout), hslow):
            r = I.mri_evolve(gbmv, hydro, chem, w, tm, tout, rem, eu, u["TimeUnits"], table,
                             prec, forcing_units=forcing_units, **fast)
            steps, failed = steps + r.slow_steps, failed + r.fast_failed_cells
        if failed:
            raise RuntimeError(f"fast integration failed in {failed} cells")
        return tout, hslow, None, steps

    return _output_loop(inp, hydro, w, t0, hslow, outdir, evolve, log)
