"""ARK-IMEX chemistry-hydrodynamics integration on the GPU (integrate.ark_imex_evolve over
integrate.ChemHydroImex: fexpl, fimpl, Jimpl + block LU, PostprocessStep, device WRMS norms)
against the same driver over the oracle (the oracle's fEuler with the reference's fexpl glue,
chemistry source and Jacobian, dense per-block Newton solves, numpy norms); and the device
WRMS norm against numpy."""
import math

import numpy as np
import pytest

import oracle_py as O
import workloads as W
from conftest import maxnorm_err

pytestmark = pytest.mark.gpu
OPTS = dict(rtol=1e-6, atol=1e-10, maxcor=10, nlscoef=0.01, safety=0.99, bias=2.0, growth=2.0)


def _gpu_problem(torch, wl, tables, eu, tu, precision=0, **kw):
    import gbmv
    import integrate
    nz, ny, nx = wl["fields"][0].shape
    hy = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(nx * ny * nz, tables)
    c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    prob = integrate.ChemHydroImex(gbmv, hy, c, eu, tu, OPTS["rtol"], OPTS["atol"], precision,
                                   **kw)
    return hy, prob, w


def test_wrms_norm_matches_numpy(cuda):
    torch = cuda
    import gbmv
    rng = np.random.default_rng(7)
    shape = (6, 5, 7)
    hy = gbmv.Hydro(shape[::-1], 10, (0,) * 6, 1.4)
    v = [rng.standard_normal(shape) for _ in range(5)] + [rng.standard_normal(shape + (10,))]
    y = [rng.standard_normal(shape) * 10.0 ** rng.integers(-8, 8, size=shape) for _ in range(5)]
    y.append(rng.standard_normal(shape + (10,)))
    for rtol, atol in ((1e-6, 1e-10), (1e-3, 0.0), (0.0, 1.0)):
        ref = math.sqrt(sum(float(((a * (1.0 / (rtol * np.abs(b) + atol))) ** 2).sum())
                            for a, b in zip(v, y)) / (15 * np.prod(shape)))
        got = hy.wrms_norm([torch.from_numpy(a).cuda() for a in v],
                           [torch.from_numpy(b).cuda() for b in y], rtol, atol)
        assert abs(got - ref) <= 1e-14 * ref, (rtol, atol)
    zero = [torch.zeros_like(torch.from_numpy(a)).cuda() for a in v]
    assert hy.wrms_norm(zero, [torch.from_numpy(b).cuda() for b in y], 1e-6, 1e-10) == 0.0
    with pytest.raises(Exception):
        hy.wrms_norm(zero, zero, 0.0, 0.0)


@pytest.mark.parametrize("pair,units,adapt", [((2, 104), "scaled", 0),
                                               ((13, 112), "reference", 2),
                                               ((13, 112), "scaled", 0)],
                         ids=["ark324-scaled-pid", "ark437-reference-i", "ark437-scaled-pid"])
def test_imex_fp64_matches_oracle_driven_run(cuda, tables, pair, units, adapt):
    """ARK3(2)4L[2]SA and the primordial inputs' ARK4(3)7L[2]SA (etable 13, itable 112), the
    fexpl chemistry tendency unconverted as the reference adds it or converted to the scaled
    variables, the PID and I controllers."""
    torch = cuda
    import integrate
    wl = W.chem_hydro(shape=(8, 6, 5))
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    tf = 4e-6
    opts = dict(OPTS, table=integrate.ark_table(*pair), adapt_method=adapt)
    y_ref = [f.copy() for f in wl["fields"]]
    oracle_prob = O.ImexChemHydro(wl, tables, eu, tu, OPTS["rtol"], OPTS["atol"],
                                  forcing_units=units)
    st_ref = integrate.ark_imex_evolve(oracle_prob, 0.0, tf, y_ref, **opts)
    _, prob, w = _gpu_problem(torch, wl, tables, eu, tu, forcing_units=units)
    st = integrate.ark_imex_evolve(prob, 0.0, tf, w, **opts)
    torch.cuda.synchronize()
    got = [x.cpu().numpy() for x in w]
    # the same step sequence, then the same states to well inside the tolerance
    assert (st.steps, st.netf, st.ncf) == (st_ref.steps, st_ref.netf, st_ref.ncf)
    assert st.steps >= 3 and st.nsetups >= 1
    for k in range(5):
        assert maxnorm_err(got[k], y_ref[k]) <= 1e-10, k
    n = got[5].size // 10
    a, b = got[5].reshape(n, 10), y_ref[5].reshape(n, 10)
    for s in range(10):  # the same steps; rounding amplified over the run, far inside rtol
        assert maxnorm_err(a[:, s], b[:, s]) <= 1e-7, s
    for k in range(6):  # the run moved the state
        assert not np.array_equal(got[k], wl["fields"][k])


def test_imex_mixed_fexpl_matches_fp64(cuda, tables):
    """The float-float WENO in the explicit part changes the run by far less than the
    integration tolerance."""
    torch = cuda
    import integrate
    wl = W.chem_hydro(shape=(12, 10, 8))
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    runs = []
    for precision in (0, 2):
        _, prob, w = _gpu_problem(torch, wl, tables, eu, tu, precision)
        st = integrate.ark_imex_evolve(prob, 0.0, 4e-6, w, **OPTS)
        runs.append(([x.cpu().numpy() for x in w], st))
    (a, sa), (b, sb) = runs
    assert abs(sa.steps - sb.steps) <= max(2, sa.steps // 20)
    for k in range(6):
        assert maxnorm_err(b[k], a[k]) <= 1e-6, k


def test_imex_fused_newton_matches_modified(cuda, tables):
    """Stage solves by the fused per-cell kernel (full Newton with the FP64 factor) against
    ARKODE's modified Newton over the separate entries: the same solution to well inside the
    integration tolerance, in fewer Newton iterations."""
    torch = cuda
    import integrate
    wl = W.chem_hydro(shape=(12, 10, 8))
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    runs = []
    for fused in (False, True):
        _, prob, w = _gpu_problem(torch, wl, tables, eu, tu, 0, fused_newton=fused)
        st = integrate.ark_imex_evolve(prob, 0.0, 4e-6, w, **OPTS)
        runs.append(([x.cpu().numpy() for x in w], st))
    (a, sa), (b, sb) = runs
    assert sb.ncf == 0 and sb.nni <= sa.nni
    for k in range(6):
        assert maxnorm_err(b[k], a[k]) <= 1e-6, k


def test_imex_newton_krylov_matches_direct(cuda, tables):
    """Matrix-free Newton-Krylov: the stage corrections by batched per-cell GMRES over
    gbmv_chem_jvp (no Jacobian formed or factored) against the block-direct solver: the
    linear solves agree to ~1e-10 and the IMEX runs to well inside the tolerance."""
    torch = cuda
    import gbmv
    import integrate
    wl = W.chem_hydro(shape=(8, 6, 5))
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    # one linear solve: (I - gamma J) x = b
    _, pd, w = _gpu_problem(torch, wl, tables, eu, tu)
    _, pk, _ = _gpu_problem(torch, wl, tables, eu, tu, linear_solver="gmres")
    pk.chem, pk.hydro = pd.chem, pd.hydro
    pd.fi(0.0, w)
    pk.fi(0.0, w)
    gam = 2e-6 * 0.1235
    assert pd.setup(0.0, w, gam) == 0 and pk.setup(0.0, w, gam) == 0
    rng = np.random.default_rng(8)
    b = [torch.from_numpy(rng.standard_normal(tuple(x.shape))).cuda() for x in w]
    xd, xk = pd.solve(b)[5].cpu().numpy(), pk.solve(b)[5].cpu().numpy()
    n = xd.size // 10
    for s in range(10):
        assert maxnorm_err(xk.reshape(n, 10)[:, s], xd.reshape(n, 10)[:, s]) <= 1e-9, s
    # whole runs with the primordial inputs' method pair
    runs = []
    for lsolver in ("direct", "gmres"):
        _, prob, w = _gpu_problem(torch, wl, tables, eu, tu, linear_solver=lsolver)
        st = integrate.ark_imex_evolve(prob, 0.0, 4e-6, w, table=integrate.ark_table(13, 112),
                                       **OPTS)
        runs.append(([x.cpu().numpy() for x in w], st, prob.krylov_iters))
    (a, sa, _), (b_, sb, kit) = runs
    assert sb.steps == sa.steps and kit > 0
    for k in range(6):
        assert maxnorm_err(b_[k], a[k]) <= 1e-6, k
