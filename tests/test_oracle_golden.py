"""The oracle restatement against fixtures produced by the reference's own code (CPU)."""
import numpy as np
import pytest

import oracle_py as O
from conftest import case_fields, feuler_case_names, maxnorm_err


def test_feuler_cases_bit_exact(golden_feuler):
    g = golden_feuler
    names = feuler_case_names(g)
    assert len(names) >= 30
    for name in names:
        w, nchem, bc, gamma, force = case_fields(g, name)
        st, out = O.feuler(w, nchem, bc, gamma, force)
        assert st == int(g[f"{name}/status"]), name
        if st != 0:
            continue
        for i, o in enumerate(out):
            ref = g[f"{name}/wdot{i}"]
            # oracle and reference evaluate the same expressions in the same order: bit-exact
            assert np.array_equal(o, ref, equal_nan=True), (name, i, maxnorm_err(o, ref))


def test_illegal_state_reported(golden_feuler):
    assert int(golden_feuler["illegal_pressure/status"]) == -1


def test_chem_sequence_bit_exact(golden_chem, tables):
    g = golden_chem
    c = O.Chem(tables, g["scale"])
    assert np.array_equal(c.mdens, g["mdens"])
    assert np.array_equal(c.cie, g["cie"])
    assert np.array_equal(c.h2, g["h2"])
    for call in range(3):
        ydot = c.rhs(g[f"y{call}"])
        assert np.array_equal(ydot, g[f"ydot{call}"], equal_nan=True), call
        assert np.array_equal(c.Ts, g[f"Ts{call}"]), call
        assert np.array_equal(c.dTs_ge, g[f"dTs_ge{call}"]), call
        J = c.jac(g[f"y{call}"])
        assert np.array_equal(J, g[f"J{call}"], equal_nan=True), call


def test_temperature_history_matters(golden_chem, tables):
    """The temperature Newton starts from the previous call's T (ten fixed iterations), so a
    fresh state (T=1000 K) gives different sources than the third call of the sequence."""
    g = golden_chem
    c = O.Chem(tables, g["scale"])
    ydot_fresh = c.rhs(g["y2"])
    assert not np.array_equal(ydot_fresh, g["ydot2"])


def test_block_newton_solve_matches_dense_lapack(golden_chem):
    """The block LU solve has no reference test (MAGMA/KLU are absent): pin it against
    numpy's LAPACK solve of I - gamma*J on the oracle Jacobians."""
    g = golden_chem
    J = g["J0"]
    n = J.shape[0]
    rng = np.random.default_rng(7)
    b = rng.normal(size=10 * n)
    for gamma in (1e-3, 0.1, 10.0):
        bad, x = O.block_newton_solve(J, gamma, b)
        assert bad == 0
        A = np.eye(10)[None] - gamma * np.transpose(J, (0, 2, 1))  # [cell][row][col]
        xr = np.linalg.solve(A, b.reshape(n, 10, 1))[..., 0].reshape(-1)
        res = np.einsum("nij,nj->ni", A, x.reshape(n, 10)) - b.reshape(n, 10)
        rel = np.abs(res).max(axis=1) / (np.abs(A).max(axis=(1, 2)) * np.abs(x.reshape(n, 10)).max(axis=1) + 1e-300)
        assert rel.max() < 1e-12
        assert np.allclose(x, xr, rtol=1e-8, atol=1e-12 * np.abs(xr).max())


def test_block_solve_singular_flagged():
    J = np.zeros((4, 10, 10))
    bad, _ = O.block_newton_solve(J, 1.0, np.ones(40))
    assert bad == 0  # I - 0 is regular
    J[2] = np.eye(10)  # I - 1*I = 0 -> singular block 2
    bad, _ = O.block_newton_solve(J, 1.0, np.ones(40))
    assert bad == 3


def _glue_cases():
    import os
    from conftest import GOLDEN
    g = np.load(os.path.join(GOLDEN, "glue_cases.npz"))
    return g, [str(c) for c in g["cases"]]


def test_oracle_glue_matches_the_reference_program(tables):
    """The oracle's composition of the IMEX program's callbacks (oracle_py.ImexChemHydro with
    the reference's unconverted forcing) against the program's own fexpl and PostprocessStep
    and the static problem's Dengo scaling, compiled from the reference's source
    (tests/golden/glue_cases.npz): bit for bit, two fexpl calls in a row (the state the first
    rewrites feeds the second)."""
    g, cases = _glue_cases()
    for name in cases:
        w = [g[f"{name}/w{i}"].copy() for i in range(6)]
        wl = {"bc": tuple(int(b) for b in g[f"{name}/bc"]), "gamma": float(g[f"{name}/gamma"]),
              "scale": g[f"{name}/scale"]}
        eu, tu = float(g[f"{name}/EnergyUnits"]), float(g[f"{name}/TimeUnits"])
        assert np.all(g[f"{name}/prepared_chem"] == 1.0)
        p = O.ImexChemHydro(wl, tables, eu, tu, 1e-6, 1e-10, forcing_units="reference")
        for call in range(2):
            out = p.fe(0.0, w)
            for i in range(6):
                assert np.array_equal(out[i], g[f"{name}/fexpl{call}_wdot{i}"]), (name, call, i)
                assert np.array_equal(w[i], g[f"{name}/fexpl{call}_w{i}"]), (name, call, i)
        q = [g[f"{name}/post_in{i}"].copy() for i in range(6)]
        p.postprocess(0.0, q)
        for i in range(6):
            assert np.array_equal(q[i], g[f"{name}/post_out{i}"]), (name, "post", i)
        chem = g[f"{name}/w5"] * wl["scale"]
        assert np.array_equal(chem, g[f"{name}/applied_chem"])
        assert np.array_equal(chem / wl["scale"], g[f"{name}/unapplied_chem"])
