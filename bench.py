"""Benchmark of the fused chemistry-hydrodynamics RHS step at 128^3 x (5 fluid + 10 species).

One step = one pass of the hot path over the whole grid, as an IMEX / multirate stage does it:
  1. fexpl (slow hydro RHS): Dengo scaling, et <- ge, WENO5 flux divergence of all 15
     fields with reflecting-x / periodic-y,z ghosts, ge tendency <- et tendency, unscale;
  2. fimpl (fast chemistry source) x TimeUnits;
  3. Jimpl (analytic chemistry Jacobian) x TimeUnits, Newton matrix I - gamma*J, batched LU;
  4. block-diagonal Newton solve of (I - gamma*J) x = fimpl.
metric: Mcells/s = cells / step time.  `value` is device-resident throughput; `e2e` includes
per-step host->device copies of the state from pinned memory and device->host copies of the
outputs (tendency vector and Newton update) through the public Python API.

  python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl gbmv|reference]
                  [--form best|fp64|mixed|mixed_fast|mixed_fast_concurrent|mixed_fast_queue]
--form best (default) times the plain FP64 form and the mixed-precision forms (the last with
the chemistry Newton on a second stream beside the WENO sweep inside the step's graph), checks
each mixed form's outputs against the FP64 form's (max-normalised per field), and reports the
fastest form whose error is <= 1e-6 as the headline.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "sundials-manyvector-demo_gb300")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

METRIC = "Mcells/s of fused WENO RHS+chem step at 128^3x15 vs plain FP64 GPU, at 1e-6 rel"
N = 128
GAMMA_NEWTON = 1e-4  # h * a_ii of the implicit stage, code time units
TABLES = os.path.join(ROOT, "tests", "golden", "primordial_tables.h5")
WORKLOAD = ("chem_hydro 128^3 x (5 fluid + 10 species): planar Sod-like interface along x, "
            "random primordial mass fractions, reflecting x / periodic y,z; fused step = "
            "fexpl WENO5 RHS + chem source + chem Jacobian + I-gamma*J LU + block solve")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gbmv", choices=["gbmv", "reference"])
    p.add_argument("--form", default="best",
                   choices=["best", "fp64", "mixed", "mixed_fast", "mixed_fast_concurrent",
                            "mixed_fast_queue"])
    p.add_argument("--n", type=int, default=N)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--newton-refine", type=int, default=None,
                   help="FP64-residual refinement cap of the fused Newton (default 2)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-parity", action="store_true",
                   help="skip the whole-grid comparisons with the oracle (all host cores)")
    p.add_argument("--dirk-n", type=int, default=64,
                   help="static-chemistry DIRK measurement on dirk_n^3 cells (0 = skip)")
    p.add_argument("--weno-n", default="128,256",
                   help="Rayleigh-Taylor WENO RHS throughput grids (comma list, '' = skip)")
    p.add_argument("--concurrent", action="store_true",
                   help="also time the mixed stage as two concurrent graph branches")
    p.add_argument("--no-sod", action="store_true", help="skip the Sod whole-run measurement")
    p.add_argument("--mri-n", type=int, default=128,
                   help="multirate time-to-t_f measurement on mri_n^3 x 15 (0 = skip)")
    p.add_argument("--imex-n", type=int, default=64,
                   help="ARK-IMEX time-to-t_f measurement on imex_n^3 x 15 (0 = skip)")
    p.add_argument("--imex-tf", type=float, default=4e-6)
    p.add_argument("--ad-n", type=int, default=96,
                   help="differentiation measurement on ad_n^3 x 9 fields (0 = skip)")
    p.add_argument("--dirk-only", action="store_true",
                   help="run only the DIRK measurement (prints its object)")
    p.add_argument("--dirk-form", default="all",
                   choices=["all", "fp64", "mixed", "fp64_deduce", "mixed_deduce"])
    return p.parse_args()


# ----------------------------------------------------------------- clocks during the timed region

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"gbmv_clocks_{os.getpid()}.csv")
        self.gpu = gpu_index

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}",
                                          f"--query-gpu={self.FIELDS}", "--format=csv,noheader",
                                          "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax = float(parts[2].split()[0])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- the GB300 arm

class FusedStep:
    """One fused step on device-resident state.

    form "fp64" : the plain FP64 GPU form -- the drop-in entry points in the order an ARKODE
                  IMEX/MRI stage calls them (fexpl, fimpl, Jimpl, SUNMatScaleAddI, LS setup,
                  LS solve), every kernel in FP64;
    form "mixed": the batched mixed-precision form -- float-float WENO face fluxes on the
                  FP32 pipes (FP64 per-cell primitives, FP64 divergence) and the fused
                  chemistry Newton kernel (FP64 source and Jacobian, FP32 LU with adaptive
                  FP64-residual refinement, no Jacobian in HBM), the whole stage captured as
                  one CUDA graph and replayed."""

    def __init__(self, torch, n, form, wl=None, concurrent=False, newton_bps=None):
        import gbmv
        import h5tables
        import workloads as W
        self.torch, self.gbmv, self.form = torch, gbmv, form
        self.concurrent = concurrent
        self.precision = {"mixed": gbmv.MIXED, "mixed_fast": gbmv.MIXED_FAST}.get(form, gbmv.FP64)
        wl = wl if wl is not None else W.chem_hydro(n=n)
        self.wl = wl
        self.n = n
        self.ncell = n ** 3
        self.units = wl["units"]
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        self.host = [np.ascontiguousarray(f) for f in wl["fields"]]
        self.w = [dev(f) for f in self.host]
        self.wdot = [torch.empty_like(f) for f in self.w]
        self.f = torch.empty(10 * self.ncell, dtype=torch.float64, device="cuda")
        self.x = torch.empty_like(self.f)
        self.J = (torch.empty(100 * self.ncell, dtype=torch.float64, device="cuda")
                  if form == "fp64" else None)
        self.hydro = gbmv.Hydro((n, n, n), 10, wl["bc"], wl["gamma"])
        self.chem = gbmv.Chem(self.ncell, h5tables.load_table_block(TABLES))
        self.chem.set_scale(dev(wl["scale"].reshape(-1)))
        self.ls = gbmv.BlockLinearSolver(self.ncell) if form == "fp64" else None
        self.status = torch.zeros(2, dtype=torch.int32, device="cuda")
        self.graph = None
        torch.cuda.synchronize()
        # the library's launch-shape autotuners on this state (results do not depend on them):
        # the face sweeps' threads per block, and the fused Newton's grid where it runs alone
        self.tuned = {"sweep_threads": self.hydro.autotune(self.w, self.precision)}
        if form != "fp64" and not concurrent:
            self.tuned["newton_blocks_per_sm"] = self.chem.newton_autotune(
                self.w[5].view(-1), GAMMA_NEWTON, self.units["TimeUnits"], gbmv.MIXED,
                NEWTON_REFINE)
        torch.cuda.synchronize()
        if form != "fp64":  # the whole stage as one CUDA graph (asynchronous entry points)
            self.chem_stream = torch.cuda.Stream()
            if concurrent:  # persistent Newton grid leaving room for the WENO sweep beside it,
                # and sweeps sized to share the SMs with it
                self.hydro.set_sweep_budget(True)
                self.tuned["sweeps"] = "shared"
                if concurrent == "queue":
                    self.queue = torch.zeros(1, dtype=torch.int64, device="cuda")
                if newton_bps is None:  # the Newton's resident blocks per SM and the sweeps'
                    # threads per block, by timing the two-branch graph (the state is restored
                    # after each trial)
                    trials = {}
                    for st in SWEEP_THREADS_CANDIDATES:
                        self.hydro.set_sweep_threads(self.precision, st)
                        for b in NEWTON_BPS_CANDIDATES:
                            trials[f"{st}x{b}"] = self._graph_ms(b)
                    best = min(trials, key=trials.get)
                    st, newton_bps = (int(v) for v in best.split("x"))
                    self.hydro.set_sweep_threads(self.precision, st)
                    self.tuned["sweep_threads"] = st
                    self.tuned["trials_ms (sweep threads x newton blocks per SM)"] = trials
                self.tuned["newton_blocks_per_sm"] = newton_bps
                self._set_narrow(newton_bps)
            self.graph = self._capture()
            # the captured launches keep their grid; eager calls (the per-kernel timings) use
            # the tuned (or default) grid again
            if concurrent:
                self.chem.set_newton_occupancy(0)

    def _capture(self):
        torch = self.torch
        self._stage_async()
        torch.cuda.synchronize()
        self.check_status()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=side):
            self._stage_async()
        torch.cuda.synchronize()
        return graph

    def _set_narrow(self, bps):
        if self.concurrent == "queue":
            self.narrow_bps = bps
        else:
            self.chem.set_newton_occupancy(bps)

    def _graph_ms(self, bps, reps=6):
        """Mean time of one replay of the concurrent stage with `bps` Newton blocks per SM."""
        torch = self.torch
        self._set_narrow(bps)
        graph = self._capture()
        graph.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            graph.replay()
        e1.record()
        torch.cuda.synchronize()
        del graph
        self.reset()
        return round(e0.elapsed_time(e1) / reps, 3)

    def _stage_async(self, t=0.0):
        g, torch = self.gbmv, self.torch
        EU, TU = self.units["EnergyUnits"], self.units["TimeUnits"]
        self.status.zero_()
        if not self.concurrent:
            g.fexpl_async(self.hydro, self.chem, t, self.w, self.wdot, EU, self.status[0:1],
                          self.precision)
            g.chem_newton_async(self.chem, t, self.w[5].view(-1), self.f, self.x, GAMMA_NEWTON,
                                TU, self.status[1:2], lu_precision=g.MIXED, refine=NEWTON_REFINE)
            return
        # two independent branches of the stage: the chemistry (FP64 pipe) beside the WENO
        # sweep (FP32 pipes); the mixed fexpl never writes w[5], so both may read it
        main = torch.cuda.current_stream()
        queue = self.concurrent == "queue"
        if queue:
            self.queue.zero_()
        fork = torch.cuda.Event()
        fork.record(main)
        self.chem_stream.wait_event(fork)
        y = self.w[5].view(-1)
        if queue:  # a narrow launch beside the sweep, a full-width one after it: one pass
            g.chem_newton_queue_async(self.chem, t, y, self.f, self.x, GAMMA_NEWTON, TU,
                                      self.status[1:2], self.queue, self.narrow_bps,
                                      lu_precision=g.MIXED, refine=NEWTON_REFINE,
                                      stream=self.chem_stream)
        else:
            g.chem_newton_async(self.chem, t, y, self.f, self.x, GAMMA_NEWTON, TU,
                                self.status[1:2], lu_precision=g.MIXED, refine=NEWTON_REFINE,
                                stream=self.chem_stream)
        g.fexpl_async(self.hydro, self.chem, t, self.w, self.wdot, EU, self.status[0:1],
                      self.precision)
        if queue:
            g.chem_newton_queue_async(self.chem, t, y, self.f, self.x, GAMMA_NEWTON, TU,
                                      self.status[1:2], self.queue, 0, lu_precision=g.MIXED,
                                      refine=NEWTON_REFINE)
        join = torch.cuda.Event()
        join.record(self.chem_stream)
        main.wait_event(join)

    def check_status(self):
        st = self.status.cpu().tolist()
        if st[0]:
            raise RuntimeError(f"illegal state mask {st[0]}")
        if st[1]:
            raise RuntimeError("singular Newton block")

    def reset(self):
        """Back to the initial state (fields and the chemistry temperature history)."""
        for d, h in zip(self.w, self.host):
            d.copy_(self.torch.from_numpy(h))
        self.chem.state("Ts").fill_(1000.0)
        self.torch.cuda.synchronize()

    def step(self, t=0.0):
        g = self.gbmv
        if self.graph is not None:
            self.graph.replay()
            return
        EU, TU = self.units["EnergyUnits"], self.units["TimeUnits"]
        rc = g.fexpl(self.hydro, self.chem, t, self.w, self.wdot, EU, self.precision)
        if rc != 0:
            raise RuntimeError(f"fexpl returned {rc}")
        y = self.w[5].view(-1)
        if self.form == "fp64":
            self.chem.calculate_rhs_cvklu(t, y, self.f, TU)
            self.chem.calculate_jacobian_cvklu(t, y, self.J, TU)
            g.form_newton_matrix(self.J, GAMMA_NEWTON)
            if self.ls.setup(self.J) != 0:
                raise RuntimeError("singular Newton block")
            self.ls.solve(self.J, self.x, self.f)
        else:
            if self.chem.newton_iteration(t, y, self.f, self.x, GAMMA_NEWTON, TU,
                                          lu_precision=g.MIXED, refine=NEWTON_REFINE) != 0:
                raise RuntimeError("singular Newton block")

    def outputs(self):
        self.check_status()
        outs = [t.cpu().numpy() for t in self.wdot]
        return outs + [self.f.cpu().numpy(), self.x.cpu().numpy()]

    def bytes_in(self):
        return sum(a.nbytes for a in self.host)

    def bytes_out(self):
        return sum(t.numel() * 8 for t in self.wdot) + self.x.numel() * 8


# FP32-LU refinement steps of the fused Newton in the mixed forms: each step costs ~0.4 ms at
# 128^3; two bring the Newton update within 1e-8 of the FP64 path (measured: 1 -> 3.5e-6,
# 2 -> 1.1e-8, 3 -> 3.6e-11, 4 -> 2.9e-12), far inside the 1e-6 budget.
NEWTON_REFINE = 2


def e2e_pipelined(torch, sets, pin_in, steps):
    """End-to-end steps with double-buffered device state: step k computes on set k % 2 while
    the inputs of step k+1 go up and the outputs of step k-1 come back on their own streams.
    Returns ms per step over `steps` steps (all copies inside the timed region)."""
    comp = torch.cuda.current_stream()
    h2d, d2h = torch.cuda.Stream(), torch.cuda.Stream()
    outs = [([torch.empty(t.shape, dtype=torch.float64).pin_memory() for t in s.wdot],
             torch.empty(s.x.shape, dtype=torch.float64).pin_memory()) for s in sets]
    ev = [{k: torch.cuda.Event() for k in ("ready", "done", "drained")} for _ in sets]

    def run(nsteps):
        for e in ev:
            e["drained"].record(comp)
        for k in range(nsteps):
            i = k % 2
            S, E = sets[i], ev[i]
            h2d.wait_event(E["drained"])
            with torch.cuda.stream(h2d):
                for d, h in zip(S.w, pin_in):
                    d.copy_(h, non_blocking=True)
            E["ready"].record(h2d)
            comp.wait_event(E["ready"])
            S.step()
            E["done"].record(comp)
            d2h.wait_event(E["done"])
            with torch.cuda.stream(d2h):
                for h, d in zip(outs[i][0], S.wdot):
                    h.copy_(d, non_blocking=True)
                outs[i][1].copy_(S.x, non_blocking=True)
            E["drained"].record(d2h)
        for e in ev:
            comp.wait_event(e["drained"])

    run(2)  # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(comp)
    h2d.wait_event(e0)
    d2h.wait_event(e0)
    run(steps)
    e1.record(comp)
    torch.cuda.synchronize()
    for s in sets:
        s.check_status()
    return e0.elapsed_time(e1) / steps


def time_steps(torch, fn, steps, warmup):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        fn()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


FAMILIES = ("face_flux", "divergence", "prims", "chem_rhs", "chem_jac", "chem_newton",
            "block_lu_factor", "block_lu_solve", "glue")


def algo_bytes(fam, n):
    """Algorithmic bytes per launch: inputs read once, outputs written once."""
    ncell, nvar = n ** 3, 15
    nf = (n + 1) * n * n
    return {
        "face_flux": 8 * nvar * (ncell + nf),           # FP64 form: state in, fluxes out
        "face_flux_mx": 4 * (16 * ncell + nvar * nf),   # mixed form: FP32 copies in, FP32 fluxes out
        "divergence": 8 * nvar * (3 * nf + ncell) + 8 * 5 * ncell,
        "prims": 8 * nvar * ncell + 4 * 16 * ncell,
        "chem_rhs": 368 * ncell,
        "chem_jac": (34 * 8 + 800) * ncell,
        "chem_newton": 456 * ncell,
        "block_lu_factor": 1640 * ncell,
        "block_lu_solve": 1000 * ncell,
        "glue": 0,
    }[fam]


# Arithmetic per unit of each kernel family, counted by ncu on these kernels
# (smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma} or {fadd,fmul,ffma}: adds + muls +
# 2 x FMAs, per face or cell, on a 112^3 grid) -- the numerator of the compute
# roofline; the denominator is the FMA rate measured by gbmv_diag_fma_rate.
FP_COUNTS = {
    ("fp64", "face_flux"): ("fp64", 3841.3, "face"),
    ("fp64", "chem_rhs"): ("fp64", 2440.9, "cell"),
    ("fp64", "chem_jac"): ("fp64", 957.0, "cell"),
    ("fp64", "block_lu_factor"): ("fp64", 759.0, "cell"),
    ("mixed", "face_flux"): ("fp32", 25990.0, "face"),
    ("mixed", "chem_newton"): ("fp64", 1671.1, "cell"),
    ("mixed_fast", "face_flux"): ("fp32", 16190.0, "face"),
    ("mixed_fast", "chem_newton"): ("fp64", 1671.1, "cell"),
}


# DRAM bytes per unit of the dominant kernels, from ncu captures with the state larger than
# L2 (dram__bytes_read.sum + dram__bytes_write.sum per face or cell on a 112^3 grid), scaled by
# the units of one 128^3 launch for the roofline's `traffic`.
DRAM_TRAFFIC = {
    ("fp64", "face_flux"): (248.2, "face"),    # mean of the x / y / z sweeps
    ("mixed", "face_flux"): (296.5, "face"),
    ("mixed", "chem_newton"): (471.4, "cell"),
    ("mixed_fast", "face_flux"): (355.6, "face"),
    ("mixed_fast", "chem_newton"): (471.4, "cell"),
    ("fp64", "chem_rhs"): (357.3, "cell"),
}


def timed_form(torch, gbmv, fs, steps, warmup):
    for _ in range(warmup):
        fs.step()
    torch.cuda.synchronize()
    gbmv.profile_reset()
    gbmv.profile_enable(True)
    l0 = gbmv.launch_count()
    with ClockSampler(0) as clk:
        ms = time_steps(torch, fs.step, steps, 0)
    launches = gbmv.launch_count() - l0
    gbmv.profile_enable(False)
    fam = {f: gbmv.profile_get(f) for f in FAMILIES}
    return ms, fam, launches, clk.summary()


def run_gbmv(args):
    import torch
    import gbmv
    import build_lib
    import workloads as W
    if not os.path.exists(build_lib.LIB):
        build_lib.build()
    gbmv.load()
    torch.cuda.set_device(0)
    wl = W.chem_hydro(n=args.n)
    global NEWTON_REFINE
    if args.newton_refine is not None:
        NEWTON_REFINE = args.newton_refine
    forms = (["fp64", "mixed", "mixed_fast", "mixed_fast_concurrent", "mixed_fast_queue"]
             if args.form == "best" else [args.form])
    if args.concurrent and "mixed" in forms:
        forms.append("mixed_concurrent")

    def make_fs(form):
        base = form.replace("_concurrent", "").replace("_queue", "")
        mode = "queue" if form.endswith("_queue") else form.endswith("_concurrent")
        return FusedStep(torch, args.n, base, wl, concurrent=mode)

    res = {}
    for form in forms:
        fs = make_fs(form)
        ms, fam, launches, clk = timed_form(torch, gbmv, fs, args.steps, args.warmup)
        fam_steps = args.steps
        if fs.graph is not None:  # graph replays bypass the per-call timing events: time eagerly
            g_ms = ms
            graph, fs.graph = fs.graph, None
            fam_steps = max(2, args.steps // 2)
            _, fam, el, _ = timed_form(torch, gbmv, fs, fam_steps, 1)
            # replays launch the captured kernels: the eager count per step times the steps
            launches = el // fam_steps * args.steps
            fs.graph = graph
            ms = g_ms
        fs.reset()
        fs.step()
        torch.cuda.synchronize()
        res[form] = dict(fs=fs, ms=ms, fam=fam, fam_steps=fam_steps, launches=launches, clocks=clk,
                         out=fs.outputs(), tuned=fs.tuned)
        if form != forms[-1]:
            del fs.J
            res[form]["fs"] = None
            torch.cuda.empty_cache()
    ncell = args.n ** 3
    def form_errs(form):
        names = ["rho", "mx", "my", "mz", "et", "chem", "fimpl", "newton_x"]
        ref, mx = res["fp64"]["out"], res[form]["out"]
        errs = {}
        for nm, a, b in zip(names, mx, ref):
            if nm in ("chem", "fimpl", "newton_x"):
                a2, b2 = a.reshape(-1, 10), b.reshape(-1, 10)
                e = max(float(np.max(np.abs(a2[:, s] - b2[:, s])) / max(np.max(np.abs(b2[:, s])), 1e-300))
                        for s in range(10))
            else:
                e = float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
            errs[nm] = e
        return errs

    all_errs = {f: form_errs(f) for f in res if f.startswith("mixed")} if "fp64" in res else {}
    ok = [f for f, e in all_errs.items() if max(e.values()) <= 1e-6]
    head = min(ok, key=lambda f: res[f]["ms"]) if ok else forms[0]
    errs = all_errs.get(head) if head != "fp64" else None
    R = res[head]
    ms, fam = R["ms"], R["fam"]
    value = ncell / (ms * 1e-3) / 1e6
    dom = max(fam, key=lambda k: fam[k][0])
    hbm_peak, peak_kind = measured_peaks()
    fp64_peak = gbmv.fma_rate(True) / 1e12
    dt_ms, nl = fam[dom]
    avg_ms = dt_ms / max(nl, 1)
    hform = head.replace("_concurrent", "").replace("_queue", "")
    key = "face_flux_mx" if (dom == "face_flux" and hform != "fp64") else dom
    achieved = algo_bytes(key, args.n) / (avg_ms * 1e-3) / 1e9 if avg_ms > 0 else 0.0
    traffic, traffic_note = None, None
    if (hform, dom) in DRAM_TRAFFIC:
        per, unit = DRAM_TRAFFIC[(hform, dom)]
        units = (args.n + 1) * args.n * args.n if unit == "face" else ncell
        traffic = round(per * units, 0)
        traffic_note = (f"bytes per launch: {per} B/{unit} (ncu dram__bytes_read+write, 112^3 "
                        f"capture, state > L2) x {units} {unit}s")
    pipe = None
    if (hform, dom) in FP_COUNTS:
        pname, per_unit, unit = FP_COUNTS[(hform, dom)]
        units = (args.n + 1) * args.n * args.n if unit == "face" else ncell
        peak_pipe = gbmv.fma_rate(pname == "fp64") / 1e12
        ach = per_unit * units / (avg_ms * 1e-3) / 1e12
        pipe = {"name": pname, "achieved": round(ach, 4), "peak": round(peak_pipe, 4),
                "unit": "TFLOP/s", "frac": round(ach / peak_pipe, 4),
                "flops_per_unit": per_unit, "per": unit,
                "peak_kind": "measured (gbmv_diag_fma_rate FMA probe)"}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mcells/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64",
                  "mixed_fast": ("f64 state; float-float WENO with f32 weights on differences, "
                                 "f32 LU + f64 refinement")}.get(
            hform, "f64 state; f32 + float-float WENO, f32 LU + f64 refinement"),
        "data": "synthetic (seeded numpy PCG64; rate tables from the reference's primordial_tables.h5)",
        "config": {"workload": WORKLOAD, "grid": [args.n] * 3, "nvar": 15, "cells": ncell,
                   "form": head, "newton_gamma": GAMMA_NEWTON, "newton_refine": NEWTON_REFINE,
                   "l2": "inputs larger than L2 (state 252 MB)"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2),
                     "peak": hbm_peak, "unit": "GB/s", "frac": round(achieved / hbm_peak, 5),
                     "peak_kind": f"{peak_kind} hbm_gbs", "traffic": traffic,
                     "traffic_note": traffic_note,
                     "avg_launch_ms": round(avg_ms, 4),
                     "fp64_peak_tflops_measured": round(fp64_peak, 4),
                     "pipe": pipe},
        "kernel_ms_per_step": {k: round(v[0] / R["fam_steps"], 4) for k, v in fam.items() if v[1]},
        "kernel_ms_per_step_fp64_form": ({k: round(v[0] / res["fp64"]["fam_steps"], 4)
                                          for k, v in res["fp64"]["fam"].items() if v[1]}
                                         if "fp64" in res else None),
        "gpu_launches": int(R["launches"]),
        "clocks": R["clocks"],
        "forms": {f: {"ms_per_step": round(r["ms"], 4),
                      "value": round(ncell / (r["ms"] * 1e-3) / 1e6, 3),
                      "autotuned": r["tuned"]} for f, r in res.items()},
    }
    if head.endswith("_concurrent") or head.endswith("_queue"):
        bps = R["tuned"].get("newton_blocks_per_sm")
        line["config"]["schedule"] = (
            "one CUDA graph per step with two branches: the chemistry Newton on a second stream "
            f"(persistent grid, {bps} one-warp blocks per SM, chosen by timing the graph) beside "
            "the WENO sweep (its register budget sized to share the SMs)"
            + ("; both Newton launches take 32-cell chunks from one counter, the second, a full-"
               "width launch after the sweep, drains what the first has not taken"
               if head.endswith("_queue") else "")
            + "; outputs bit-identical to the serial graph; kernel_ms_per_step and roofline time "
            "each kernel alone (eager, serial), so their sum exceeds ms_per_step by the overlap")
    if errs is not None:
        line["mixed_vs_fp64_maxnorm_err"] = {k: float(f"{v:.3e}") for k, v in errs.items()}
        line["speedup_vs_fp64_form"] = round(res["fp64"]["ms"] / res[head]["ms"], 3)
        line["forms_maxnorm_err_vs_fp64"] = {f: float(f"{max(e.values()):.3e}")
                                             for f, e in all_errs.items()}

    if not args.no_parity:
        line["parity"] = fused_parity(wl, {f: r["out"] for f, r in res.items()}, head)

    if not args.no_e2e:
        fs = R["fs"] if R["fs"] is not None else make_fs(head)
        pin_in = [torch.from_numpy(a).pin_memory() for a in fs.host]
        pin_out = [torch.empty(t.shape, dtype=torch.float64).pin_memory() for t in fs.wdot]
        pin_x = torch.empty(fs.x.shape, dtype=torch.float64).pin_memory()

        def e2e_step():
            for d, h in zip(fs.w, pin_in):
                d.copy_(h, non_blocking=True)
            fs.step()
            for h, d in zip(pin_out, fs.wdot):
                h.copy_(d, non_blocking=True)
            pin_x.copy_(fs.x, non_blocking=True)

        e2e_steps = max(10, args.steps)
        ms_serial = statistics.median(time_steps(torch, e2e_step, e2e_steps, 1)
                                      for _ in range(3))
        sets = [fs, make_fs(head)]
        ms_pipe = statistics.median(e2e_pipelined(torch, sets, pin_in, e2e_steps)
                                    for _ in range(3))
        ms_e2e = min(ms_serial, ms_pipe)
        line["e2e"] = {"value": round(ncell / (ms_e2e * 1e-3) / 1e6, 3), "unit": "Mcells/s",
                       "h2d_bytes_per_step": fs.bytes_in(), "d2h_bytes_per_step": fs.bytes_out(),
                       "ms_per_step": round(ms_e2e, 4),
                       "ms_per_step_serial_copies": round(ms_serial, 4),
                       "ms_per_step_pipelined": round(ms_pipe, 4),
                       "repeats": "median of 3 runs of max(10, steps) steps each",
                       "note": ("every step copies its inputs from pinned host memory and its "
                                "tendencies and Newton update back inside the timed region; "
                                "pipelined = two device state sets, copies of one step overlap "
                                "the compute of its neighbour on separate copy streams")}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_port(sample_n=(128, 128, 32))
    if args.weno_n:
        for r in res.values():
            r["fs"] = None
        fs = None
        torch.cuda.empty_cache()
        line["weno_rhs"] = _guarded(run_weno, torch, gbmv,
                                    [int(x) for x in args.weno_n.split(",") if x],
                                    parity=not args.no_parity)
    if not args.no_sod:
        line["sod"] = _guarded(run_sod, torch, gbmv, not args.no_cpu_baseline)
    if args.mri_n > 0:
        for r in res.values():
            r["fs"] = None
        fs = None
        torch.cuda.empty_cache()
        line["multirate"] = _guarded(run_mri, torch, gbmv, args.mri_n)
    if args.imex_n > 0:
        for r in res.values():
            r["fs"] = None
        fs = None
        torch.cuda.empty_cache()
        line["imex"] = _guarded(run_imex, torch, gbmv, args.imex_n, args.imex_tf,
                                not args.no_cpu_baseline)
    if args.ad_n > 0:
        for r in res.values():
            r["fs"] = None
        fs = None
        torch.cuda.empty_cache()
        line["differentiation"] = _guarded(run_ad, torch, gbmv, args.ad_n)
    if args.dirk_n > 0:
        for k in ("fs",):
            for r in res.values():
                r[k] = None
        fs = None
        torch.cuda.empty_cache()
        line["chem_dirk"] = _guarded(run_dirk, torch, gbmv, args.dirk_n,
                                     not args.no_cpu_baseline, args.dirk_form)
    print(json.dumps(line))


def _guarded(fn, torch, *a, **kw):
    """A secondary measurement: its failure is recorded in the line instead of losing it."""
    try:
        return fn(torch, *a, **kw)
    except Exception as e:  # noqa: BLE001 (reported, not hidden)
        import traceback
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        return {"error": f"{type(e).__name__}: {e}",
                "where": traceback.format_exc().strip().splitlines()[-3:]}


# ----------------------------------------------------------------- whole-grid parity

OUT_NAMES = ["rho", "mx", "my", "mz", "et", "chem", "fimpl", "newton_x"]


def _maxnorm(a, b):
    """max |a - b| / max |b| (NaN positions must coincide)."""
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return float("inf")
    m = ~nb
    if not m.any():
        return 0.0
    sc = float(np.max(np.abs(b[m])))
    d = float(np.max(np.abs(a[m] - b[m])))
    return d / sc if sc > 0 else d


def _out_errs(outs, refs, names):
    e = {}
    for nm, a, b in zip(names, outs, refs):
        if nm in ("chem", "fimpl", "newton_x"):
            a2, b2 = a.reshape(-1, 10), b.reshape(-1, 10)
            e[nm] = max(_maxnorm(a2[:, k], b2[:, k]) for k in range(10))
        else:
            e[nm] = _maxnorm(a, b)
    return {k: float(f"{v:.3e}") for k, v in e.items()}


def fused_parity(wl, form_outs, head):
    """Every timed form's outputs of one stage at the full grid against the oracle's
    composition of the same stage (fexpl + fimpl + Jimpl + block solve), evaluated on all
    host cores (z-slabs and cell ranges on threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import h5tables
    import oracle_py as O
    t0 = time.time()
    fields = [np.array(f, copy=True) for f in wl["fields"]]
    oc = O.Chem(h5tables.load_table_block(TABLES), wl["scale"].reshape(-1))
    st, ref = O.fused_chem_hydro_step(fields, wl["scale"], oc, wl["bc"], wl["gamma"],
                                      wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"],
                                      GAMMA_NEWTON, threads=0)
    secs = time.time() - t0
    if st != 0:
        return {"error": f"oracle status {st}"}
    errs = {f: _out_errs(o, ref, OUT_NAMES) for f, o in form_outs.items()}
    out = {"what": ("one fused stage from the initial state, every output of every timed form "
                    "against the CPU oracle at the full grid (per field max|gpu - oracle| / "
                    "max|oracle|; chemistry, fimpl and the Newton update per species)"),
           "oracle_threads": os.cpu_count(), "oracle_s": round(secs, 2),
           "bars": {"fp64": "1e-12 (Newton update 1e-10)", "mixed forms": "1e-6"},
           "maxnorm_err_vs_oracle": {f: max(e.values()) for f, e in errs.items()},
           "per_output": {f: errs[f] for f in ("fp64", head) if f in errs}}
    out["fp64_maxnorm_err_vs_oracle"] = out["maxnorm_err_vs_oracle"].get("fp64")
    out["mixed_maxnorm_err_vs_oracle"] = out["maxnorm_err_vs_oracle"].get(head)
    return out


# ----------------------------------------------------------------- WENO RHS throughput (RT)

def run_weno(torch, gbmv, grids, steps=3, warmup=2, parity=True):
    """Rayleigh-Taylor WENO RHS (fEuler alone) at NVAR 15, the FP64 and both mixed forms: RHS
    evaluations per second, cell updates per second, algorithmic HBM GB/s (read w + write wdot
    = 240 B/cell) and the FP64 form's FP64-pipe fraction from the counted flops per face; with
    `parity`, each form's output against the CPU oracle at the full grid (all host cores)."""
    import workloads as W
    if parity:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py as O
    fp64_peak = gbmv.fma_rate(True) / 1e12
    hbm_peak, peak_kind = measured_peaks()
    out = {"workload": "Rayleigh-Taylor: rho = 1.5 + 0.5 tanh((z-0.5)/0.02), hydrostatic p "
                       "(g = -0.1, p(1) = 2.5), velocities U[-1e-2, 1e-2], 10 tracers U[0,1] rho; "
                       "periodic x,y, reflecting z; constant force -0.1 on z-momentum",
           "nvar": 15, "hbm_peak_gbs": hbm_peak, "fp64_peak_tflops": round(fp64_peak, 4),
           "grids": {}}
    for n in grids:
        wl = W.rayleigh_taylor(n=n, nchem=10)
        h = gbmv.Hydro((n, n, n), 10, wl["bc"], wl["gamma"], wl["force"])
        w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
        wdot = [torch.empty_like(f) for f in w]
        ref = None
        if parity:
            t0 = time.time()
            st, ref = O.feuler(wl["fields"], 10, wl["bc"], wl["gamma"], wl["force"], threads=0)
            oracle_s = time.time() - t0
            if st != 0:
                raise RuntimeError("oracle: illegal state")
        del wl
        ncell = n ** 3
        faces = 3 * (n + 1) * n * n
        g = {}
        perr = {}
        for name, prec in (("fp64", gbmv.FP64), ("mixed", gbmv.MIXED),
                           ("mixed_fast", gbmv.MIXED_FAST)):
            def rhs():
                if h.fEuler(0.0, w, wdot, prec) != 0:
                    raise RuntimeError("fEuler failed")
            ms = time_steps(torch, rhs, steps, warmup)
            if ref is not None:
                perr[name] = float(f"{max(_maxnorm(a.cpu().numpy(), b) for a, b in zip(wdot, ref)):.3e}")
            r = {"ms_per_rhs": round(ms, 3), "rhs_per_s": round(1e3 / ms, 2),
                 "Mcell_updates_per_s": round(ncell / (ms * 1e-3) / 1e6, 2),
                 "algorithmic_GBps": round(240.0 * ncell / (ms * 1e-3) / 1e9, 1),
                 "hbm_frac": round(240.0 * ncell / (ms * 1e-3) / 1e9 / hbm_peak, 5)}
            if name == "fp64":
                fl = FP_COUNTS[("fp64", "face_flux")][1] * faces + 158.4 * ncell
                r["fp64_pipe_frac"] = round(fl / (ms * 1e-3) / 1e12 / fp64_peak, 4)
            g[name] = r
        g["speedup_mixed_vs_fp64"] = round(g["fp64"]["ms_per_rhs"] / g["mixed"]["ms_per_rhs"], 3)
        g["speedup_mixed_fast_vs_fp64"] = round(g["fp64"]["ms_per_rhs"] /
                                                g["mixed_fast"]["ms_per_rhs"], 3)
        if ref is not None:
            g["parity"] = {"maxnorm_err_vs_oracle": perr, "oracle_threads": os.cpu_count(),
                           "oracle_s": round(oracle_s, 2),
                           "bars": {"fp64": 1e-12, "mixed": 1e-6, "mixed_fast": 1e-6}}
        out["grids"][f"{n}^3"] = g
        del h, w, wdot, ref
        torch.cuda.empty_cache()
    return out


# ----------------------------------------------------------------- Sod whole run

SOD_TABLE = 3  # ARKODE's default order-4 ERK (input_sod.txt: order = 4)


def sod_errors(yg, shape, x, t=0.2, gamma=1.4):
    """L-infinity and RMS errors of the five conserved fields against the exact Riemann
    solution over the whole grid, as the reference's Sod output_diagnostics forms them
    (src/sod.cpp:385-469: rho, mx, my, mz, et)."""
    import integrate as I
    r, u, p = I.sod_exact(x, t, gamma)
    exact = [r, r * u, 0.0 * r, 0.0 * r, p / (gamma - 1.0) + 0.5 * r * u * u]
    names = ["rho", "mx", "my", "mz", "et"]
    linf, rms = {}, {}
    for v, (nm, e) in enumerate(zip(names, exact)):
        d = np.abs(yg[v].reshape(shape) - e[None, None, :])
        linf[nm] = float(f"{float(d.max()):.3e}")
        rms[nm] = float(f"{float(np.sqrt(np.mean(d * d))):.3e}")
    return {"linf": linf, "rms": rms,
            "note": "shocks and contacts are smeared over a few cells, so the L-infinity errors "
                    "are of the jump's size there; the RMS errors carry the convergence"}


def run_sod(torch, gbmv, with_cpu):
    """Sod shock tube 128x3x3 (reflecting x, periodic y,z, gamma 1.4) to t_f = 0.2 with the
    adaptive ERK of the Sod inputs (order 4: ARKODE's Zonneveld 5-3-4, PID controller; rtol
    1e-6, atol 1e-11) over the GPU FP64 RHS: time to t_f, steps, L1 error of density against
    the exact Riemann solution; the oracle-driven run on one host core beside it."""
    import integrate as I
    import workloads as W
    nx = 128
    wl = W.sod(nx, 3, 3)
    shape = wl["fields"][0].shape
    n = int(np.prod(shape))
    h = gbmv.Hydro((nx, 3, 3), 0, wl["bc"], wl["gamma"])
    wdot = torch.empty((5, n), dtype=torch.float64, device="cuda")

    def rhs_gpu(t, y):
        w = [y[i].view(shape) for i in range(5)]
        d = [wdot[i].view(shape) for i in range(5)]
        if h.fEuler(t, w, d) != 0:
            raise RuntimeError("illegal state")
        return wdot.clone()

    y0 = np.stack([f.reshape(-1) for f in wl["fields"]])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h0 = 1e-4
    yl, stl = I.erk_evolve(rhs_gpu, 0.0, 0.2, torch.from_numpy(y0).cuda(), 1e-6, 1e-11,
                           table=SOD_TABLE, h0=h0)
    torch.cuda.synchronize()
    dt_loop = time.perf_counter() - t0

    # the same integration with every step one CUDA graph (stages, device WRMS norm, device
    # controller), replayed in batches of 16 with one 128-byte read per batch
    def graph_run(precision):
        status = torch.zeros(1, dtype=torch.int32, device="cuda")

        def rhs_async(y, o):
            v, d = y.view(5, n), o.view(5, n)
            h.fEuler_async(0.0, [v[i].view(shape) for i in range(5)],
                           [d[i].view(shape) for i in range(5)], status, precision)

        def norm_async(v, y, o):
            a, b = v.view(5, n), y.view(5, n)
            h.wrms_norm_async([a[i].view(shape) for i in range(5)],
                              [b[i].view(shape) for i in range(5)], 1e-6, 1e-11, o)

        yd = torch.from_numpy(y0.copy()).cuda().view(-1)
        ge = I.GraphERK(rhs_async, norm_async, yd, table=SOD_TABLE, batch=16,
                        status=lambda: int(status.item()))
        ge.evolve(0.0, 1e-12, h0)  # capture (and one tiny eager step) outside the timed region
        yd.copy_(torch.from_numpy(y0).cuda().view(-1))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = ge.evolve(0.0, 0.2, h0)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, st, yd.view(5, n).cpu().numpy()

    dt, st, yg = graph_run(gbmv.FP64)
    dt_m, st_m, yg_m = graph_run(gbmv.MIXED)
    x = (np.arange(nx) + 0.5) / nx
    r, _, _ = I.sod_exact(x, 0.2)
    rho = yg[0].reshape(shape)[1, 1]
    out = {"workload": "Sod 128x3x3, reflecting x / periodic y,z, gamma 1.4, t_f 0.2, "
                       "adaptive Zonneveld 4(3) (order 4, PID) rtol 1e-6 atol 1e-11, FP64 RHS",
           "s_to_tf": round(dt, 4), "steps": st.steps, "error_test_fails": st.fails,
           "rhs_evals": st.nfe, "form": "every step one CUDA graph (integrate.GraphERK)",
           "host_loop": {"s_to_tf": round(dt_loop, 3), "steps": stl.steps,
                         "note": "integrate.erk_evolve: one host synchronisation per step"},
           "graph_vs_host_loop_maxnorm_diff": float(f"{max(float(np.max(np.abs(yg[v] - yl.cpu().numpy()[v]))) / max(float(np.max(np.abs(yl.cpu().numpy()[v]))), 1e-300) for v in range(5)):.3e}"),
           "l1_density_err_vs_exact": float(f"{np.mean(np.abs(rho - r)):.3e}"),
           "vs_exact": sod_errors(yg, shape, x),
           "mixed_form": {
               "s_to_tf": round(dt_m, 4), "steps": st_m.steps,
               "rhs": "GBMV_MIXED (float-float face fluxes: the per-face chain on the FP32 "
                      "pipes; the 128x3x3 grid is too small to fill the GPU, so each RHS is "
                      "latency-bound by one warp's face)",
               "vs_fp64_graph_run_maxnorm_diff": float(f"{max(float(np.max(np.abs(yg_m[v] - yg[v]))) / max(float(np.max(np.abs(yg[v]))), 1e-300) for v in range(5)):.3e}"),
               "vs_exact": sod_errors(yg_m, shape, x)}}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py as O

        def rhs_cpu(t, y):
            s_, o = O.feuler([y[i].reshape(shape) for i in range(5)], 0, wl["bc"], wl["gamma"],
                             None)
            return np.stack([a.reshape(-1) for a in o])

        t0 = time.perf_counter()
        yc, stc = I.erk_evolve(rhs_cpu, 0.0, 0.2, y0, 1e-6, 1e-11, table=SOD_TABLE, h0=h0)
        dtc = time.perf_counter() - t0
        # max-normalised per field; fields that stay zero (the y, z momenta here) give 0
        diff = max(float(np.max(np.abs(yg[v] - yc[v]))) /
                   max(float(np.max(np.abs(yc[v]))), 1e-300) for v in range(5))
        out["cpu_baseline"] = {"s_to_tf": round(dtc, 3), "cores": 1, "kind": "port",
                               "steps": stc.steps, "max_rel_diff_vs_gpu_run": float(f"{diff:.3e}")}
    return out


# ----------------------------------------------------------------- multirate time-to-t_f

MRI_H, MRI_STEPS = 2e-6, 2   # slow step (code time units) and slow steps to t_f
MRI_FAST = dict(rtol=1e-6, atol=1e-10, maxcor=10, nlscoef=0.01, itable=112)


def run_mri(torch, gbmv, n):
    """Multirate chemistry-hydrodynamics to t_f = MRI_STEPS * MRI_H on the chem_hydro state
    (integrate.mri_evolve: WENO slow stages, persistent batched DIRK fast stages) with the
    reference's default third-order MIS-KW3 coupling in the FP64 and the mixed form (the
    latter also with the fast DIRK's intermediate stage derivatives deduced), and the
    second-order MRI-GARK-ERK22b coupling in the mixed form; time-to-t_f and max-normalised
    differences per field."""
    import h5tables
    import integrate
    import workloads as W
    wl = W.chem_hydro(n=n)
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    tables = h5tables.load_table_block(TABLES)
    out = {"workload": (f"chem_hydro {n}^3 x 15, explicit MRI-GARK (MIS-KW3: third order; "
                        f"ERK22b: explicit midpoint coupling), fixed slow step {MRI_H} x 1e11 s, "
                        f"{MRI_STEPS} steps, fast DIRK ARK4(3)7L[2]SA (itable 112) rtol 1e-6 "
                        "atol 1e-10; slow chemistry tendency added unconverted, as the "
                        "reference"), "forms": {}}
    finals = {}
    for name, prec, table, extra in (("fp64", gbmv.FP64, integrate.MRI_KW3, {}),
                                     ("mixed", gbmv.MIXED, integrate.MRI_KW3, {}),
                                     ("mixed_deduce", gbmv.MIXED, integrate.MRI_KW3,
                                      {"deduce": 1}),
                                     ("mixed_erk22b", gbmv.MIXED, integrate.MRI_ERK22B, {})):
        hy = gbmv.Hydro((n, n, n), 10, wl["bc"], wl["gamma"])
        c = gbmv.Chem(n ** 3, tables)
        c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
        w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
        # every slow step one CUDA graph (integrate.GraphMRI): the first step runs eagerly
        # (allocations, the DIRK block autotuner) and the graph is captured, outside the timed
        # region; then the state goes back to the start and all steps replay the graph
        gm = integrate.GraphMRI(gbmv, hy, c, w, MRI_H, eu, tu, table, prec, **MRI_FAST, **extra)
        gm.evolve(0.0, MRI_H)
        for x, f in zip(w, wl["fields"]):
            x.copy_(torch.from_numpy(np.ascontiguousarray(f)))
        c.state("Ts").fill_(1000.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = gm.evolve(0.0, MRI_H * MRI_STEPS)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        finals[name] = [x.cpu().numpy() for x in w]
        out["forms"][name] = {"s_to_tf": round(dt, 3),
                              "Mcells_per_s": round(n ** 3 * MRI_STEPS / dt / 1e6, 4),
                              "coupling": table["name"], "slow_steps": r.slow_steps,
                              "schedule": "each slow step one CUDA graph (fexpl, forcing, "
                                          "persistent-DIRK fast evolves of all stages)",
                              "slow_rhs": r.slow_rhs, "failed_cells": r.fast_failed_cells}
        del hy, c, w
        torch.cuda.empty_cache()
    def errs(x, y):
        e = {}
        for nm, a, b in zip(["rho", "mx", "my", "mz", "et", "chem"], x, y):
            if nm == "chem":
                a2, b2 = a.reshape(-1, 10), b.reshape(-1, 10)
                e[nm] = float(f"{max(float(np.max(np.abs(a2[:, s] - b2[:, s]) / max(np.max(np.abs(b2[:, s])), 1e-300))) for s in range(10)):.3e}")
            else:
                e[nm] = float(f"{float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)):.3e}")
        return e
    out["mixed_vs_fp64_maxnorm_err"] = errs(finals["mixed"], finals["fp64"])
    # both forms against the same slow steps with the fast problems solved to a tight
    # tolerance (FP64, rtol 1e-9, atol 1e-13): the error each form's inner integration makes.
    # The mixed-against-FP64 difference is of that size (adaptive inner steps at rtol 1e-6
    # that part on a rounding difference), and both forms' errors are alike.
    hy = gbmv.Hydro((n, n, n), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(n ** 3, tables)
    c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    tight = dict(MRI_FAST, rtol=1e-9, atol=1e-13)
    gm = integrate.GraphMRI(gbmv, hy, c, w, MRI_H, eu, tu, integrate.MRI_KW3, gbmv.FP64, **tight)
    t0 = time.perf_counter()
    r = gm.evolve(0.0, MRI_H * MRI_STEPS)
    torch.cuda.synchronize()
    ref = [x.cpu().numpy() for x in w]
    out["vs_tight_inner_tolerance"] = {
        "reference": "FP64 form, MIS-KW3, the same slow steps, fast DIRK rtol 1e-9 atol 1e-13",
        "reference_s": round(time.perf_counter() - t0, 3),
        "reference_failed_cells": r.fast_failed_cells,
        "fp64_maxnorm_err": errs(finals["fp64"], ref),
        "mixed_maxnorm_err": errs(finals["mixed"], ref),
        "mixed_deduce_maxnorm_err": errs(finals["mixed_deduce"], ref)}
    del hy, c, w, gm
    torch.cuda.empty_cache()
    # the coupling's own contribution (second- against third-order MRI at the same slow step)
    out["erk22b_vs_kw3_maxnorm_diff"] = errs(finals["mixed_erk22b"], finals["mixed"])
    out["speedup_mixed_vs_fp64"] = round(out["forms"]["fp64"]["s_to_tf"] /
                                         out["forms"]["mixed"]["s_to_tf"], 3)
    out["speedup_mixed_deduce_vs_fp64"] = round(out["forms"]["fp64"]["s_to_tf"] /
                                                out["forms"]["mixed_deduce"]["s_to_tf"], 3)
    return out


NEWTON_BPS_CANDIDATES = (3, 4, 5)  # the concurrent stage's Newton blocks per SM, timed
SWEEP_THREADS_CANDIDATES = (64, 128)  # and its sweeps' threads per block


IMEX_OPTS = dict(rtol=1e-6, atol=1e-10, maxcor=10, nlscoef=0.01, safety=0.99, bias=2.0,
                 growth=2.0, adapt_method=2)  # the reference's primordial IMEX inputs
IMEX_PAIR = (13, 112)  # ARK4(3)7L[2]SA: etable 13, itable 112 of those inputs


def run_imex(torch, gbmv, n, tf, with_cpu):
    """ARK-IMEX chemistry-hydrodynamics to t_f on the chem_hydro state (integrate.ark_imex_evolve
    over integrate.ChemHydroImex: ARK3(2)4L[2]SA, WENO explicit, chemistry implicit, device
    WRMS norms; the reference IMEX inputs' step control): the FP64 and the GBMV_MIXED_FAST
    explicit RHS with ARKODE's modified Newton over the FP64 Jacobian and block LU, and
    GBMV_MIXED_FAST with full Newton corrections from the fused per-cell kernel: time-to-t_f,
    step and solver statistics, max-normalised differences from the FP64 run; the
    oracle-driven run of the same driver on an 8x6x5 sample on one host core beside it."""
    import h5tables
    import integrate
    import workloads as W
    wl = W.chem_hydro(n=n)
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    tables = h5tables.load_table_block(TABLES)
    table = integrate.ark_table(*IMEX_PAIR)
    opts = dict(IMEX_OPTS, table=table)
    out = {"workload": (f"chem_hydro {n}^3 x 15 to t_f = {tf} x 1e11 s, ARK4(3)7L[2]SA IMEX "
                        "(etable 13 / itable 112; WENO explicit, chemistry implicit), rtol 1e-6 "
                        "atol 1e-10, maxcor 10, nlscoef 0.01, I controller safety 0.99 bias 2 "
                        "growth 2; fexpl chemistry tendency added unconverted, as the reference"),
           "forms": {}}
    finals = {}
    # fp64 / mixed_fast: ARKODE's modified Newton over fimpl, Jimpl and the block LU;
    # mixed_fast_fused: full Newton stage corrections from the fused per-cell kernel (FP64
    # factor)
    for name, prec, fused in (("fp64", gbmv.FP64, False), ("mixed_fast", gbmv.MIXED_FAST, False),
                              ("mixed_fast_fused", gbmv.MIXED_FAST, True)):
        hy = gbmv.Hydro((n, n, n), 10, wl["bc"], wl["gamma"])
        c = gbmv.Chem(n ** 3, tables)
        c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
        w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
        prob = integrate.ChemHydroImex(gbmv, hy, c, eu, tu, IMEX_OPTS["rtol"], IMEX_OPTS["atol"],
                                       prec, fused_newton=fused)
        wc = [x.clone() for x in w]  # warm-up on a copy (allocations)
        integrate.ark_imex_evolve(prob, 0.0, tf * 1e-17, wc, **opts)  # a few steps
        c.state("Ts").fill_(1000.0)
        del wc
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = integrate.ark_imex_evolve(prob, 0.0, tf, w, **opts)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        finals[name] = [x.cpu().numpy() for x in w]
        out["forms"][name] = {"s_to_tf": round(dt, 3), "steps": st.steps,
                              "attempts": st.attempts, "error_test_fails": st.netf,
                              "newton_fails": st.ncf, "newton_iters": st.nni,
                              "setups": st.nsetups, "fe_evals": st.nfe, "fi_evals": st.nfi,
                              "Mcell_steps_per_s": round(n ** 3 * st.steps / dt / 1e6, 4)}
        del hy, c, w, prob
        torch.cuda.empty_cache()
    for form in ("mixed_fast", "mixed_fast_fused"):
        errs = {}
        for nm, a, b in zip(["rho", "mx", "my", "mz", "et", "chem"], finals[form],
                            finals["fp64"]):
            errs[nm] = float(f"{float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)):.3e}")
        out[f"{form}_vs_fp64_maxnorm_err"] = errs
        out[f"speedup_{form}_vs_fp64"] = round(out["forms"]["fp64"]["s_to_tf"] /
                                               out["forms"][form]["s_to_tf"], 3)
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py as O
        sw = W.chem_hydro(shape=(8, 6, 5))
        y = [f.copy() for f in sw["fields"]]
        prob = O.ImexChemHydro(sw, tables, sw["units"]["EnergyUnits"],
                               sw["units"]["TimeUnits"], IMEX_OPTS["rtol"], IMEX_OPTS["atol"])
        t0 = time.perf_counter()
        st = integrate.ark_imex_evolve(prob, 0.0, tf, y, **opts)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"Mcell_steps_per_s": round(240 * st.steps / dt / 1e6, 6),
                               "s_to_tf": round(dt, 3), "steps": st.steps, "cores": 1,
                               "kind": "port", "sample": "8x6x5 cells of the same workload"}
    return out


# ----------------------------------------------------------------- differentiation

def run_ad(torch, gbmv, n, ndir=16, h=1e-7, nsteps=50, every=10):
    """Smooth periodic flow (rho = 1 + 0.2 sin(2 pi (x+y+z)), p = 1, velocities U[-0.1, 0.1],
    4 tracers) on n^3 x 9 fields: times of the FP64 RHS, its JVP and VJP; their agreement with
    central differences (h = 1e-7) on `ndir` seeded directions; the gradient of the integral of
    rho^2 after `nsteps` RK4 steps with checkpoints every `every` steps (autograd wrapper of
    tests/ad_harness.py over the C ABI) against a central difference of the loss."""
    import workloads as W
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import ad_harness as AD
    wl = W.smooth_periodic(n=n, nchem=4)
    hy = gbmv.Hydro((n, n, n), 4, wl["bc"], wl["gamma"])
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    del wl
    out = [torch.empty_like(x) for x in w]
    rng = np.random.default_rng(20261203 + 5)

    def dirs():
        return [torch.from_numpy(rng.standard_normal(tuple(x.shape))).cuda() *
                float(x.abs().max()) for x in w]

    def rhs(ws, o):
        if hy.fEuler(0.0, ws, o, 0) != 0:
            raise RuntimeError("fEuler failed")

    d0 = dirs()
    t_rhs = time_steps(torch, lambda: rhs(w, out), 3, 2)
    t_jvp = time_steps(torch, lambda: hy.fEuler_jvp(0.0, w, d0, out), 3, 2)
    t_vjp = time_steps(torch, lambda: hy.fEuler_vjp(0.0, w, d0, out), 3, 2)
    dot = lambda a, b: sum(float((x * y).sum()) for x, y in zip(a, b))
    fp = [torch.empty_like(x) for x in w]
    fm = [torch.empty_like(x) for x in w]
    jv = [torch.empty_like(x) for x in w]
    u = [torch.empty_like(x) for x in w]
    fd_checks = {}
    ncell = n ** 3
    mask = torch.empty(ncell, dtype=torch.uint8, device="cuda")
    for hh in (h, 1e-9):
        jmax, jl2, verr, nbad, ntot = 0.0, 0.0, 0.0, 0, 0
        jmax_s, verr_s, nmask = 0.0, 0.0, 0
        for _ in range(ndir):
            d = dirs()
            hy.fEuler_jvp(0.0, w, d, jv)
            rhs([a + hh * b for a, b in zip(w, d)], fp)
            rhs([a - hh * b for a, b in zip(w, d)], fm)
            # cells whose faces keep their Lax-Friedrichs branch over w -+ hh d
            hy.kink_mask(w, d, hh, mask)
            keep = (mask == 0).view(w[0].shape)
            nmask += ncell - int(keep.sum())
            num, den = 0.0, 0.0
            for a, b, c in zip(jv, fp, fm):
                fd = (b - c) / (2 * hh)
                err = (a - fd).abs()
                scale = max(float(fd.abs().max()), 1e-300)
                jmax = max(jmax, float(err.max()) / scale)
                kk = keep if a.dim() == 3 else keep.unsqueeze(-1)
                jmax_s = max(jmax_s, float((err * kk).max()) / scale)
                nbad += int((err > 1e-6 * scale).sum())
                ntot += err.numel()
                num += float((err * err).sum())
                den += float((fd * fd).sum())
            jl2 = max(jl2, (num / max(den, 1e-300)) ** 0.5)
            v = dirs()
            hy.fEuler_vjp(0.0, w, v, u)
            lhs, r = dot(u, d), (dot(v, fp) - dot(v, fm)) / (2 * hh)
            verr = max(verr, abs(lhs - r) / max(abs(r), 1e-300))
            vs = [x * (keep if x.dim() == 3 else keep.unsqueeze(-1)) for x in dirs()]
            hy.fEuler_vjp(0.0, w, vs, u)
            lhs, r = dot(u, d), (dot(vs, fp) - dot(vs, fm)) / (2 * hh)
            verr_s = max(verr_s, abs(lhs - r) / max(abs(r), 1e-300))
        fd_checks[f"h={hh:g}"] = {"jvp_maxnorm_err": float(f"{jmax:.3e}"),
                                  "jvp_rel_l2_err": float(f"{jl2:.3e}"),
                                  "jvp_entries_above_1e-6": f"{nbad} of {ntot}",
                                  "vjp_rel_err": float(f"{verr:.3e}"),
                                  "smooth_cells": {
                                      "what": ("cells none of whose six faces changes its "
                                               "Lax-Friedrichs branch (maximising stencil "
                                               "point, sign of its velocity) over w -+ h d "
                                               "(gbmv_feuler_kink_mask)"),
                                      "masked_cells": f"{nmask} of {ndir * ncell}",
                                      "jvp_maxnorm_err": float(f"{jmax_s:.3e}"),
                                      "vjp_rel_err": float(f"{verr_s:.3e}")}}
    dx = 1.0 / n
    dt, vol = 0.2 * dx / 1.4, dx ** 3
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L, g = AD.loss_and_grad(hy, w, dt, nsteps, vol, checkpoint_every=every)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    t0 = time.perf_counter()
    AD.loss_only(hy, w, dt, nsteps, vol)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    gerr = {}
    for hh in (h, 1e-9):
        e = 0.0
        for _ in range(2):
            d = dirs()
            ad = dot(g, d)
            fd = (AD.loss_only(hy, [a + hh * b for a, b in zip(w, d)], dt, nsteps, vol) -
                  AD.loss_only(hy, [a - hh * b for a, b in zip(w, d)], dt, nsteps, vol)) / (2 * hh)
            e = max(e, abs(ad - fd) / abs(fd))
        gerr[f"h={hh:g}"] = float(f"{e:.3e}")
    return {"workload": f"smooth periodic flow {n}^3 x 9 (rho = 1 + 0.2 sin(2 pi (x+y+z)), p = 1, "
                        "velocities U[-0.1, 0.1], 4 tracers U[0,1] rho)",
            "ms_rhs": round(t_rhs, 3), "ms_jvp": round(t_jvp, 3), "ms_vjp": round(t_vjp, 3),
            "central_differences": fd_checks, "directions": ndir,
            "note": ("the flux has kinks (|u| and the stencil max of |u|+c in the Lax-Friedrichs "
                     "speed; the velocities are random per cell): the few entries whose "
                     "difference stencil crosses a kink differ at O(1), their number scales "
                     "with h, the exact derivatives (JVP, VJP = its transpose to 1e-12) take "
                     "the branch of the unperturbed state; `smooth_cells` holds the same "
                     "checks with the cells whose difference crosses a branch masked"),
            "gradient": {"loss": "integral of rho^2 at t_f", "rk4_steps": nsteps,
                         "checkpoint_every": every, "s_forward_only": round(t_fwd, 3),
                         "s_forward_and_gradient": round(t_grad, 3),
                         "vs_central_diff_rel_err": gerr}}


# ----------------------------------------------------------------- static chemistry (DIRK)

DIRK_TOUT = 1e-3      # code time units (TimeUnits = 1e11 s): 1e8 s of chemistry
DIRK_OPTS = dict(rtol=1e-6, atol=1e-10, maxcor=10, nlscoef=0.01)  # Newton settings of the inputs
DIRK_TABLE = 112  # ARK4(3)7L[2]SA, the `itable` of the reference's chemistry inputs


def _dirk_summary(st):
    nni = st[:, 1]
    q = np.percentile(nni, [50, 90, 99])
    edges = np.unique(np.round(np.geomspace(max(nni.min(), 1), nni.max() + 1, 13)).astype(int))
    cnt, _ = np.histogram(nni, bins=edges)
    return {"steps_mean": round(float(st[:, 0].mean()), 2), "steps_max": int(st[:, 0].max()),
            "newton_iters": {"mean": round(float(nni.mean()), 2), "p50": float(q[0]),
                             "p90": float(q[1]), "p99": float(q[2]), "max": int(nni.max())},
            "newton_iters_hist": {"edges": edges.tolist(), "counts": cnt.tolist()},
            "error_test_fails_mean": round(float(st[:, 2].mean()), 3),
            "newton_fails_mean": round(float(st[:, 3].mean()), 3),
            "setups_mean": round(float(st[:, 4].mean()), 2),
            "f_evals_mean": round(float(st[:, 6].mean()), 2), "failed": int(st[:, 7].sum())}


def run_dirk(torch, gbmv, n1, with_cpu, forms="all"):
    """Static primordial chemistry on n1^3 cells integrated to DIRK_TOUT by the persistent
    batched DIRK kernel, FP64 form and mixed form (equilibrated FP32 LU, FP32 temperature
    iterations), each with the intermediate stage derivatives evaluated (ARKODE's default)
    and deduced from the stage equations (`_deduce`); per-cell Newton-iteration histograms;
    every form against a tight-tolerance solution; oracle port timed on a sample."""
    import h5tables
    import workloads as W
    tables = h5tables.load_table_block(TABLES)
    n = n1 ** 3
    y, _ = W.primordial(n, seed=W.SEED_BASE + 2)
    scale = torch.from_numpy(y.reshape(-1).copy()).cuda()
    out = {"workload": (f"static primordial chemistry {n1}^3: uniform rho = 1e2 m_H, log-uniform "
                        "mass fractions in [1e-10, 1], log-uniform T in [10, 1e4] K; per-cell "
                        "adaptive ARK4(3)7L[2]SA ESDIRK (the inputs' itable 112) + modified "
                        "Newton, rtol 1e-6, atol 1e-10, maxcor 10, nlscoef 0.01, "
                        f"t in [0, {DIRK_TOUT}] x 1e11 s"),
           "cells": n, "tout": DIRK_TOUT, "table": DIRK_TABLE, "forms": {}}
    finals = {}
    for name, prec, deduce in (("fp64", gbmv.FP64, 0), ("mixed", gbmv.MIXED, 0),
                               ("fp64_deduce", gbmv.FP64, 1), ("mixed_deduce", gbmv.MIXED, 1)):
        if forms not in ("all", name):
            continue
        c = gbmv.Chem(n, tables)
        c.set_scale(scale)
        z = torch.ones(10 * n, dtype=torch.float64, device="cuda")
        st = torch.zeros(8 * n, dtype=torch.int32, device="cuda")
        # warm-up call over the full interval: the block-size autotuner times its candidates
        # on this call's work, which must be representative of the timed one
        c.dirk_evolve(0.0, DIRK_TOUT, z, 1e11, precision=prec, table=DIRK_TABLE, deduce=deduce,
                      **DIRK_OPTS)
        z.fill_(1.0)
        c.state("Ts").fill_(1000.0)
        torch.cuda.synchronize()
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(0) as clk:
            e0.record(s)
            nf = c.dirk_evolve(0.0, DIRK_TOUT, z, 1e11, stats=st, precision=prec,
                               table=DIRK_TABLE, deduce=deduce, **DIRK_OPTS)
            e1.record(s)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        stn = st.view(n, 8).cpu().numpy().astype(np.int64)
        finals[name] = z.view(n, 10).cpu().numpy()
        out["forms"][name] = {"ms": round(ms, 2), "value": round(n / (ms * 1e-3) / 1e6, 4),
                              "unit": "Mcells/s (cells integrated to tout per second)",
                              "block": c.dirk_block(prec), "failed_cells": int(nf),
                              "clocks": clk.summary(), **_dirk_summary(stn)}
        if prec == gbmv.MIXED:  # cells the FP32 pass left to the FP64-factor pass, their cost
            rc = c.dirk_retried()
            out["forms"][name]["second_pass"] = {
                "cells": int(rc.size),
                "newton_iters_max": int(stn[rc, 1].max()) if rc.size else 0,
                "f_evals_max": int(stn[rc, 6].max()) if rc.size else 0}
        del c
        torch.cuda.empty_cache()
    if "mixed" in finals and "fp64" in finals:
        a, b = finals["mixed"], finals["fp64"]
        e = np.abs(a - b) / (np.abs(b) + DIRK_OPTS["atol"] / DIRK_OPTS["rtol"])
        out["mixed_vs_fp64_relerr"] = {"median": float(f"{np.median(e):.3e}"),
                                       "p99": float(f"{np.percentile(e, 99):.3e}"),
                                       "max": float(f"{e.max():.3e}")}
        out["speedup_mixed_vs_fp64"] = round(out["forms"]["fp64"]["ms"] /
                                             out["forms"]["mixed"]["ms"], 3)
    for name in ("fp64_deduce", "mixed_deduce"):
        if name in finals and "fp64" in finals:
            out[f"speedup_{name}_vs_fp64"] = round(out["forms"]["fp64"]["ms"] /
                                                   out["forms"][name]["ms"], 3)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py as O
    # both forms against a tight-tolerance FP64 solution (the oracle at rtol 1e-10) on a sample
    # of cells: the error each form makes, and where the two forms part
    ns_t = 512
    t0 = time.perf_counter()
    oc = O.Chem(tables, y[:ns_t].reshape(-1))
    zt, _, nft = oc.dirk_evolve(np.ones(10 * ns_t), 0.0, DIRK_TOUT, 1e11, rtol=1e-10,
                                atol=1e-14, maxcor=10, nlscoef=0.01, max_steps=500000,
                                table=DIRK_TABLE)
    zt = zt.reshape(ns_t, 10)
    floor = DIRK_OPTS["atol"] / DIRK_OPTS["rtol"]
    tight = {"sample": f"the first {ns_t} cells", "reference": "oracle FP64 at rtol 1e-10, "
             "atol 1e-14", "reference_failed_cells": int(nft),
             "oracle_s": round(time.perf_counter() - t0, 2)}
    for name, z in finals.items():
        e = (np.abs(z[:ns_t] - zt) / (np.abs(zt) + floor)).max(axis=1)
        tight[f"{name}_relerr"] = {"median": float(f"{np.median(e):.3e}"),
                                   "p99": float(f"{np.percentile(e, 99):.3e}"),
                                   "max": float(f"{e.max():.3e}")}
    if "mixed" in finals and "fp64" in finals:
        d = (np.abs(finals["mixed"][:ns_t] - finals["fp64"][:ns_t]) /
             (np.abs(finals["fp64"][:ns_t]) + floor)).max(axis=1)
        tight["mixed_vs_fp64_relerr_max"] = float(f"{d.max():.3e}")
    out["vs_tight_tolerance_solution"] = tight
    if len(finals) >= 2:
        # the cells where the forms disagree most (over all cells), against the same tight
        # solution: which form a large disagreement comes from
        names = list(finals)
        base = finals[names[0]]
        dis = np.zeros(n)
        for name in names[1:]:
            dis = np.maximum(dis, (np.abs(finals[name] - base) / (np.abs(base) + floor)).max(axis=1))
        nh = 32
        idx = np.sort(np.argsort(dis)[-nh:])
        t0 = time.perf_counter()
        oc = O.Chem(tables, y[idx].reshape(-1))
        zh, _, nfh = oc.dirk_evolve(np.ones(10 * nh), 0.0, DIRK_TOUT, 1e11, rtol=1e-10,
                                    atol=1e-14, maxcor=10, nlscoef=0.01, max_steps=500000,
                                    table=DIRK_TABLE)
        zh = zh.reshape(nh, 10)
        hard = {"sample": f"the {nh} cells of largest disagreement between the forms (largest "
                          f"{dis.max():.3e}, smallest {dis[idx].min():.3e}, against {names[0]})",
                "reference_failed_cells": int(nfh),
                "oracle_s": round(time.perf_counter() - t0, 2)}
        for name, z in finals.items():
            e = (np.abs(z[idx] - zh) / (np.abs(zh) + floor)).max(axis=1)
            hard[f"{name}_relerr"] = {"median": float(f"{np.median(e):.3e}"),
                                      "max": float(f"{e.max():.3e}")}
        out["vs_tight_tolerance_solution_hardest"] = hard
    if with_cpu:
        ns = 256
        oc = O.Chem(tables, y[:ns].reshape(-1))
        t0 = time.perf_counter()
        oc.dirk_evolve(np.ones(10 * ns), 0.0, DIRK_TOUT, 1e11, table=DIRK_TABLE, **DIRK_OPTS)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(ns / dt / 1e6, 6), "unit": "Mcells/s", "cores": 1,
                               "kind": "port",
                               "sample": f"the first {ns} cells of the same inputs ({dt:.2f} s), "
                                         "1 thread, FP64 LU"}
    return out


# ----------------------------------------------------------------- CPU baseline (oracle port)

def _cpu_fused_step(shape, seed_offset=0):
    """One fused step of the oracle (plain-C port of the reference path) on a sub-grid of the
    same workload; returns (cells, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import h5tables
    import oracle_py as O
    import workloads as W
    wl = W.chem_hydro(shape=shape, seed=W.SEED_BASE + 3 + seed_offset)
    tables = h5tables.load_table_block(TABLES)
    u = wl["units"]
    fields = [f.copy() for f in wl["fields"]]
    scale = wl["scale"]
    chem = O.Chem(tables, scale.reshape(-1))
    t0 = time.perf_counter()
    # fexpl: scale, et <- ge, fEuler, ge tendency <- et tendency, unscale
    phys = fields[5] * scale
    fields[4] = phys[..., 9] / u["EnergyUnits"] + 0.5 / fields[0] * (
        fields[1] ** 2 + fields[2] ** 2 + fields[3] ** 2)
    st, out = O.feuler(fields[:5] + [phys], 10, wl["bc"], wl["gamma"], None)
    out[5][..., 9] = out[4]
    out[4][:] = 0.0
    y = (phys / scale).reshape(-1)
    f = chem.rhs(y) * u["TimeUnits"]
    J = chem.jac(y) * u["TimeUnits"]
    bad, x = O.block_newton_solve(J, GAMMA_NEWTON, f)
    dt = time.perf_counter() - t0
    return int(np.prod(shape)), dt


def cpu_baseline_port(sample_n=(32, 32, 32)):
    cells, dt = _cpu_fused_step(sample_n)
    return {"value": round(cells / dt / 1e6, 5), "unit": "Mcells/s", "cores": 1, "kind": "port",
            "sample": f"one fused step on a {sample_n[0]}x{sample_n[1]}x{sample_n[2]} sub-grid of "
                      f"the same workload ({cells} cells, {dt:.2f} s), 1 thread"}


def _ref_worker(args):
    shape, seed, steps = args
    tot_cells, tot_t = 0, 0.0
    for s in range(steps):
        c, t = _cpu_fused_step(shape, seed * 100 + s)
        tot_cells += c
        tot_t += t
    return tot_cells, tot_t


def run_reference(args):
    """Reference arm: the reference's path as the plain-C oracle port (the reference's own
    build needs its source tree, which is not present where the benchmark runs), on all host
    cores as independent z-slabs (one process per core, like the reference's MPI ranks)."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    slab = (args.n, 32, 4)  # per-core sample per step: 16K cells
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_ref_worker, [(slab, i, 1) for i in range(cores)])  # warm-up (imports, build)
        t0 = time.perf_counter()
        res = pool.map(_ref_worker, [(slab, i, args.steps) for i in range(cores)])
        wall = time.perf_counter() - t0
    cells = sum(r[0] for r in res)
    value = cells / wall / 1e6
    sample = (f"{args.steps} steps x {cores} processes, each one fused step on a "
              f"{slab[0]}x{slab[1]}x{slab[2]} slab of the workload per step")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": "Mcells/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(wall / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": [args.n] * 3, "nvar": 15,
                       "sample_cells_per_step": cells // args.steps},
            "cpu_baseline": {"value": round(value, 5), "unit": "Mcells/s", "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 5), "unit": "Mcells/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.dirk_only:
        import torch
        import gbmv
        import build_lib
        if not os.path.exists(build_lib.LIB):
            build_lib.build()
        gbmv.load()
        print(json.dumps({"chem_dirk": run_dirk(torch, gbmv, args.dirk_n,
                                                not args.no_cpu_baseline, args.dirk_form)}))
    else:
        run_gbmv(args)


if __name__ == "__main__":
    main()
