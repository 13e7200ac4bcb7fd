"""Generate the golden fixtures in this directory from the reference's own code.

The reference ships no golden vectors, so they are produced by running its hot-path sources
(src/utilities.cpp, src/euler3D.hpp, src/raja_primordial_network.cpp, and the IMEX program's
glue with the static problem's Dengo scaling: src/imex_chem_hydro_main.cpp,
src/primordial_static.cpp), compiled unmodified
against the one-rank shims by oracle/build_ref.sh, on seeded synthetic inputs.  This needs the
reference tree (it runs only where it exists); the fixtures it writes are committed and the
tests read only them.

    python tests/golden/make_golden.py [REFERENCE_ROOT] [--glue-only]
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "sundials-manyvector-demo_gb300"))

import oracle_py as O  # noqa: E402
import workloads as W  # noqa: E402

TABLES = os.path.join(HERE, "primordial_tables.h5")

# (name, workload builder) for the flux-divergence fixtures: every boundary type on each
# face, NVAR 5/7/9/11/15, odd extents, the minimum extent 3, forcing on and off.
BC_SETS = {
    "periodic": (0, 0, 0, 0, 0, 0),
    "neumann": (1, 1, 1, 1, 1, 1),
    "dirichlet": (2, 2, 2, 2, 2, 2),
    "reflecting": (3, 3, 3, 3, 3, 3),
    "mixed": (1, 3, 0, 0, 3, 2),
    "mixed2": (3, 1, 2, 3, 0, 0),
}


def hydro_cases():
    cases = []
    wl = W.sod()
    cases.append(("sod_128x3x3", wl))
    wl = W.rayleigh_taylor(shape=(10, 9, 8), nchem=10)
    cases.append(("rt_10x9x8_nchem10", wl))
    for nchem in (0, 2, 4, 6, 10):
        for bname, bc in BC_SETS.items():
            wl = W.rayleigh_taylor(shape=(7, 5, 6), nchem=nchem, seed=W.SEED_BASE + 50 + nchem)
            wl["bc"] = bc
            cases.append((f"bc_{bname}_nchem{nchem}", wl))
    wl = W.rayleigh_taylor(shape=(3, 3, 3), nchem=2, seed=W.SEED_BASE + 60)
    wl["bc"] = (3, 3, 1, 1, 0, 0)
    cases.append(("minimum_3x3x3", wl))
    wl = W.smooth_periodic(shape=(12, 12, 12), nchem=4)
    cases.append(("smooth_12_nchem4", wl))
    wl = W.chem_hydro(shape=(8, 6, 5))
    wl["fields"][5] = wl["fields"][5] * wl["scale"]  # physical tracers, as fslow passes them
    cases.append(("chemhydro_8x6x5", wl))
    # illegal state: one cell with negative pressure -> fEuler returns -1
    wl = W.rayleigh_taylor(shape=(6, 5, 4), nchem=0, seed=W.SEED_BASE + 70)
    wl["fields"][4][2, 3, 1] = 1e-9
    cases.append(("illegal_pressure", wl))
    return cases


def main(ref_root=None):
    cmd = [os.path.join(ROOT, "oracle", "build_ref.sh")]
    if ref_root:
        cmd.append(ref_root)
    subprocess.check_call(cmd)
    out = {}
    for name, wl in hydro_cases():
        st, res = O.ref_feuler(wl["fields"], wl["nchem"], wl["bc"], wl["gamma"], wl["force"])
        out[f"{name}/status"] = np.array(st)
        out[f"{name}/nchem"] = np.array(wl["nchem"])
        out[f"{name}/bc"] = np.array(wl["bc"])
        out[f"{name}/gamma"] = np.array(wl["gamma"])
        out[f"{name}/force"] = (np.zeros(5 + wl["nchem"]) if wl["force"] is None
                                else np.asarray(wl["force"]))
        for i, f in enumerate(wl["fields"]):
            out[f"{name}/w{i}"] = f
            if st == 0:
                out[f"{name}/wdot{i}"] = res[i]
    np.savez_compressed(os.path.join(HERE, "feuler_cases.npz"), **out)

    # chemistry: 3 successive source/Jacobian calls (the temperature carries over)
    n = 384
    y, _ = W.primordial(n, seed=W.SEED_BASE + 80)
    rng = np.random.Generator(np.random.PCG64(W.SEED_BASE + 81))
    scale = y.reshape(-1).copy()
    rc = O.RefChem(TABLES, scale)
    st = rc.state()
    ch = {"scale": scale, "mdens": st["mdens"], "cie": st["cie"], "h2": st["h2"]}
    for call in range(3):
        state = 1.0 + rng.uniform(-0.02, 0.02, size=10 * n)
        ydot = rc.rhs(state)
        s = rc.state()
        J = rc.jac(state)
        ch[f"y{call}"] = state
        ch[f"ydot{call}"] = ydot
        ch[f"Ts{call}"] = s["Ts"]
        ch[f"dTs_ge{call}"] = s["dTs_ge"]
        ch[f"J{call}"] = J
    np.savez_compressed(os.path.join(HERE, "chem_cases.npz"), **ch)
    glue_fixtures()
    print("wrote feuler_cases.npz, chem_cases.npz and glue_cases.npz")


def glue_fixtures():
    """The IMEX program's glue run from the reference's own source (oracle/_ref/
    libref_glue.so): prepare_Dengo_structures, fexpl (twice in a row: the state it rewrites
    feeds the second call), PostprocessStep, apply / unapply_Dengo_scaling, on two
    chemistry-hydrodynamics grids."""
    g = {}
    cases = [("ch_8x6x5", W.chem_hydro(shape=(8, 6, 5)), None),
             ("ch_7x5x6_mixedbc", W.chem_hydro(shape=(7, 5, 6), seed=W.SEED_BASE + 90),
              (1, 3, 0, 0, 3, 3))]
    rng = np.random.Generator(np.random.PCG64(W.SEED_BASE + 91))
    for name, wl, bc in cases:
        if bc is not None:
            wl["bc"] = bc
        u = wl["units"]
        ref = O.RefGlue(wl["fields"][0].shape, wl["bc"], wl["gamma"], u, wl["scale"], HERE)
        g[f"{name}/bc"] = np.array(wl["bc"])
        g[f"{name}/gamma"] = np.array(wl["gamma"])
        for k in ("MassUnits", "LengthUnits", "TimeUnits"):
            g[f"{name}/{k}"] = np.array(u[k])
        g[f"{name}/EnergyUnits"] = np.array(ref.energy_units())
        g[f"{name}/scale"] = wl["scale"].copy()
        g[f"{name}/prepared_chem"] = ref.prepared_chem.copy()
        f = [np.ascontiguousarray(x.copy()) for x in wl["fields"]]
        for i, x in enumerate(f):
            g[f"{name}/w{i}"] = x.copy()
        for call in range(2):
            st, out = ref.fexpl(0.0, f)
            assert st == 0
            for i in range(6):
                g[f"{name}/fexpl{call}_wdot{i}"] = out[i]
                g[f"{name}/fexpl{call}_w{i}"] = f[i].copy()
        p = [np.ascontiguousarray(x.copy()) for x in wl["fields"]]
        p[4] = p[4] * (1.0 + rng.uniform(-0.1, 0.1, size=p[4].shape))  # stale et
        p[5] = p[5] * (1.0 + rng.uniform(-0.01, 0.01, size=p[5].shape))
        for i, x in enumerate(p):
            g[f"{name}/post_in{i}"] = x.copy()
        assert ref.postprocess(0.0, p) == 0
        for i, x in enumerate(p):
            g[f"{name}/post_out{i}"] = x.copy()
        s = [np.ascontiguousarray(x.copy()) for x in wl["fields"]]
        assert ref.scaling(s, True) == 0
        g[f"{name}/applied_chem"] = s[5].copy()
        assert ref.scaling(s, False) == 0
        g[f"{name}/unapplied_chem"] = s[5].copy()
    g["cases"] = np.array([c[0] for c in cases])
    np.savez_compressed(os.path.join(HERE, "glue_cases.npz"), **g)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if "--glue-only" in sys.argv:  # keep the other fixtures, (re)write glue_cases.npz
        cmd = [os.path.join(ROOT, "oracle", "build_ref.sh")] + args[:1]
        subprocess.check_call(cmd)
        glue_fixtures()
    else:
        main(args[0] if args else None)
