"""Mixed-precision and fused forms against the FP64 oracle (GPU).

Tolerance: the 1e-6 relative error budget against the FP64 oracle, measured per field
as max|mixed - oracle| / max|oracle| over the grid.
"""
import numpy as np
import pytest

import oracle_py as O
import workloads as W
from conftest import maxnorm_err

pytestmark = pytest.mark.gpu
TOL_MIXED = 1e-6


def _run(torch, wl, precision):
    import gbmv
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), wl["nchem"], wl["bc"], wl["gamma"], wl["force"])
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    wdot = [torch.full_like(f, np.nan) for f in w]
    st = h.fEuler(0.0, w, wdot, precision)
    torch.cuda.synchronize()
    return st, [x.cpu().numpy() for x in wdot]


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("case", ["rt", "chemhydro", "smooth", "sod"])
def test_mixed_weno_within_1e6_of_oracle(cuda, precision, case):
    if case == "rt":
        wl = W.rayleigh_taylor(shape=(32, 24, 20), nchem=10, seed=W.SEED_BASE + 300)
    elif case == "chemhydro":
        wl = W.chem_hydro(shape=(24, 16, 16))
        wl["fields"][5] = wl["fields"][5] * wl["scale"]
    elif case == "smooth":
        wl = W.smooth_periodic(shape=(24, 24, 24), nchem=4)
    else:
        wl = W.sod(64, 3, 3)
    st0, ref = O.feuler(wl["fields"], wl["nchem"], wl["bc"], wl["gamma"], wl["force"])
    st1, out = _run(cuda, wl, precision)
    assert st0 == st1 == 0
    errs = [maxnorm_err(a, b) for a, b in zip(out, ref)]
    assert max(errs) <= TOL_MIXED, errs


def test_mixed_illegal_state_flagged(cuda):
    wl = W.rayleigh_taylor(shape=(6, 5, 4), nchem=0)
    wl["fields"][4][1, 1, 1] = -1.0
    st, _ = _run(cuda, wl, 1)
    assert st == -1


def _status_mask(torch, wl, precision):
    import gbmv
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), wl["nchem"], wl["bc"], wl["gamma"], wl["force"])
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    wdot = [torch.zeros_like(f) for f in w]
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    h.fEuler_async(0.0, w, wdot, status, precision)
    torch.cuda.synchronize()
    return int(status.item())


@pytest.mark.parametrize("plant", ["none", "rho", "et", "p", "rho_and_p"])
def test_mixed_legal_state_mask_matches_fp64(cuda, plant):
    """The float-float forms set the legal-state bits (1 density, 2 energy, 4 pressure;
    legal_state, src/euler3D.hpp:1398-1414) in their primitives pass; the mask must equal the
    FP64 form's for states away from p = 0 within rounding."""
    wl = W.rayleigh_taylor(shape=(7, 6, 5), nchem=10, seed=W.SEED_BASE + 310)
    rho, mx, my, mz, et = wl["fields"][:5]
    ke = 0.5 * (mx * mx + my * my + mz * mz) / rho
    if plant in ("rho", "rho_and_p"):
        rho[1, 2, 3] = -1.0
    if plant == "et":
        et[4, 1, 2] = -0.5
    if plant in ("p", "rho_and_p"):
        et[2, 4, 1] = 0.25 * ke[2, 4, 1]  # positive energy below the kinetic energy
    masks = [_status_mask(cuda, wl, prec) for prec in (0, 1, 2)]
    expect = {"none": 0, "rho": 1, "et": 6, "p": 4, "rho_and_p": 5}[plant]
    assert masks == [expect] * 3, masks


def _chem_setup(torch, tables, n, seed):
    import gbmv
    y, _ = W.primordial(n, seed=seed)
    c = gbmv.Chem(n, tables)
    c.set_scale(torch.from_numpy(y.reshape(-1).copy()).cuda())
    rng = np.random.default_rng(seed)
    state = 1.0 + rng.uniform(-1e-3, 1e-3, size=10 * n)
    return c, y.reshape(-1), state


@pytest.mark.parametrize("lu", [0, 1])
def test_fused_newton_matches_separate_path(cuda, tables, lu):
    """gbmv_chem_newton == rhs + jac + (I - gamma J) + factor + solve."""
    torch = cuda
    import gbmv
    n, gamma, tu = 4096, 1e-4, 1.0e11
    c1, y, state = _chem_setup(torch, tables, n, 401)
    c2, _, _ = _chem_setup(torch, tables, n, 401)
    ys = torch.from_numpy(state).cuda()
    f1 = torch.empty_like(ys)
    J = torch.empty(100 * n, dtype=torch.float64, device="cuda")
    x1 = torch.empty_like(ys)
    c1.calculate_rhs_cvklu(0.0, ys, f1, tu)
    c1.calculate_jacobian_cvklu(0.0, ys, J, tu)
    gbmv.form_newton_matrix(J, gamma)
    ls = gbmv.BlockLinearSolver(n)
    assert ls.setup(J) == 0
    ls.solve(J, x1, f1)
    f2, x2 = torch.empty_like(ys), torch.empty_like(ys)
    assert c2.newton_iteration(0.0, ys, f2, x2, gamma, tu, lu_precision=lu, refine=4) == 0
    torch.cuda.synchronize()
    a, b = f1.cpu().numpy().reshape(n, 10), f2.cpu().numpy().reshape(n, 10)
    ftol = 1e-12 if lu == 0 else 1e-9  # mixed: temperature iterations 1-8 in FP32
    for s in range(10):
        assert maxnorm_err(b[:, s], a[:, s]) <= ftol, (s, maxnorm_err(b[:, s], a[:, s]))
    xa, xb = x1.cpu().numpy().reshape(n, 10), x2.cpu().numpy().reshape(n, 10)
    # the fused kernel forms I - gamma*J with a different rounding order (row factors), so
    # even the FP64 LU differs by conditioning x 1e-16; FP32 LU + two FP64-residual
    # refinements: ~(kappa * 6e-8)^3 relative -- both far inside the 1e-6 budget
    tol = 1e-10 if lu == 0 else 1e-8
    for s in range(10):
        assert maxnorm_err(xb[:, s], xa[:, s]) <= tol, (s, maxnorm_err(xb[:, s], xa[:, s]))
    if lu == 0:
        assert torch.equal(c1.state("Ts"), c2.state("Ts"))
    else:
        t1, t2 = c1.state("Ts").cpu().numpy(), c2.state("Ts").cpu().numpy()
        assert np.max(np.abs(t1 - t2) / t1) <= 1e-12


@pytest.mark.parametrize("lu", [0, 1])
def test_newton_stage_matches_separate_path(cuda, tables, lu):
    """gbmv_chem_newton_stage == rhs + jac + (I - gamma J) + factor + solve of b + gamma f."""
    torch = cuda
    import gbmv
    n, gamma, tu = 4096, 1e-4, 1.0e11
    c1, y, state = _chem_setup(torch, tables, n, 402)
    c2, _, _ = _chem_setup(torch, tables, n, 402)
    rng = np.random.default_rng(402)
    ys = torch.from_numpy(state).cuda()
    f1, x1 = torch.empty_like(ys), torch.empty_like(ys)
    J = torch.empty(100 * n, dtype=torch.float64, device="cuda")
    c1.calculate_rhs_cvklu(0.0, ys, f1, tu)
    c1.calculate_jacobian_cvklu(0.0, ys, J, tu)
    # b = a - z of an implicit stage: of the size of h times the stage derivatives
    b = torch.from_numpy(rng.uniform(0.2, 0.4, size=10 * n)).cuda() * (gamma * f1)
    gbmv.form_newton_matrix(J, gamma)
    ls = gbmv.BlockLinearSolver(n)
    assert ls.setup(J) == 0
    ls.solve(J, x1, b + gamma * f1)
    f2, x2 = torch.empty_like(ys), torch.empty_like(ys)
    assert c2.newton_stage(0.0, ys, b, f2, x2, gamma, tu, lu_precision=lu, refine=4) == 0
    torch.cuda.synchronize()
    a_, b_ = f1.cpu().numpy().reshape(n, 10), f2.cpu().numpy().reshape(n, 10)
    xa, xb = x1.cpu().numpy().reshape(n, 10), x2.cpu().numpy().reshape(n, 10)
    # the kernel forms b + gamma f with one rounding (fma) and I - gamma J with row factors;
    # the blocks' conditioning carries those roundings into x
    ftol, xtol = (1e-12, 1e-9) if lu == 0 else (1e-9, 1e-8)
    for s in range(10):
        assert maxnorm_err(b_[:, s], a_[:, s]) <= ftol, s
        assert maxnorm_err(xb[:, s], xa[:, s]) <= xtol, (s, maxnorm_err(xb[:, s], xa[:, s]))


def test_fused_newton_against_oracle(cuda, tables):
    torch = cuda
    n, gamma, tu = 512, 3e-5, 1.0e11
    c, y, state = _chem_setup(torch, tables, n, 402)
    ys = torch.from_numpy(state).cuda()
    f, x = torch.empty_like(ys), torch.empty_like(ys)
    assert c.newton_iteration(0.0, ys, f, x, gamma, tu, lu_precision=1, refine=4) == 0
    torch.cuda.synchronize()
    oc = O.Chem(tables, y)
    fr = oc.rhs(state) * tu
    Jr = oc.jac(state) * tu
    bad, xr = O.block_newton_solve(Jr, gamma, fr)
    assert bad == 0
    fo, xo = f.cpu().numpy().reshape(n, 10), x.cpu().numpy().reshape(n, 10)
    for s in range(10):
        assert maxnorm_err(fo[:, s], fr.reshape(n, 10)[:, s]) <= 1e-9
        assert maxnorm_err(xo[:, s], xr.reshape(n, 10)[:, s]) <= 1e-8


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("bc", [(2, 2, 0, 0, 1, 3), (1, 3, 2, 1, 0, 0), (3, 1, 1, 3, 2, 2)])
def test_mixed_every_boundary_type(cuda, precision, bc):
    """Mixed forms on every boundary type, homogeneous Dirichlet included: there the reference's
    ghost density is negative and its fluxes are NaN; the mixed forms take their FP64 path on
    those faces and must put NaN exactly where the oracle does, and agree to 1e-6 elsewhere."""
    wl = W.rayleigh_taylor(shape=(10, 9, 8), nchem=4, seed=W.SEED_BASE + 320)
    wl["bc"] = bc
    st0, ref = O.feuler(wl["fields"], wl["nchem"], wl["bc"], wl["gamma"], wl["force"])
    st1, out = _run(cuda, wl, precision)
    assert st0 == st1 == 0
    errs = [maxnorm_err(a, b) for a, b in zip(out, ref)]  # NaN positions must coincide
    assert max(errs) <= TOL_MIXED, errs
