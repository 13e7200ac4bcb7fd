"""Generate the golden fixtures in this directory from the reference's own code.

The reference ships no golden vectors, so they are produced by running its hot-path sources
(src/utilities.cpp, src/euler3D.hpp, src/raja_primordial_network.cpp), compiled unmodified
against the one-rank shims by oracle/build_ref.sh, on seeded synthetic inputs.  This needs the
reference tree (it runs only where it exists); the fixtures it writes are committed and the
tests read only them.

    python tests/golden/make_golden.py [REFERENCE_ROOT]
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
    print("wrote feuler_cases.npz and chem_cases.npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
