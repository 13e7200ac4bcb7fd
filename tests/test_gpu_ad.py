"""Derivatives of the right-hand side on the GPU (differentiation workload: periodic smooth
flow, rho = 1 + 0.2 sin(2 pi (x+y+z)), p = 1, velocities U[-0.1, 0.1], 4 passive tracers):

* WENO RHS JVP (dual numbers) and VJP (hand-written reverse mode) against central finite
  differences, h = 1e-7, on 16 seeded random directions: agreement to 1e-6 (max-normalised);
* the VJP against the JVP by the dot-product identity <v, J dw> = <J^T v, dw> (exact
  derivatives on both sides: agreement to rounding) on periodic, Neumann, reflecting and
  mixed boundaries, NVAR 5 / 9 / 15;
* chemistry-source JVP and VJP against the Jacobian of the oracle (bit-exact with the
  reference's calculate_jacobian_cvklu), the JVP assembling it column by column;
* the gradient of the integral of rho^2 after 50 RK4 steps, recomputed from checkpoints every
  10 steps, against a central finite difference of the loss along random directions.
"""
import numpy as np
import pytest

import oracle_py as O
import workloads as W
from conftest import maxnorm_err

pytestmark = pytest.mark.gpu
H = 1e-7


def _setup(torch, wl):
    import gbmv
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), wl["nchem"], wl["bc"], wl["gamma"], wl.get("force"))
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    return h, w


def _rhs(h, w):
    import torch
    out = [torch.empty_like(x) for x in w]
    assert h.fEuler(0.0, w, out, 0) == 0
    return out


def _dirs(torch, w, rng):
    return [torch.from_numpy(rng.standard_normal(tuple(x.shape)) * np.abs(x.cpu().numpy()).max())
            .cuda() for x in w]


def _dot(a, b):
    return sum(float((x * y).sum()) for x, y in zip(a, b))


@pytest.mark.parametrize("case", ["smooth", "rt"])
def test_weno_jvp_vjp_vs_central_differences(cuda, case):
    torch = cuda
    if case == "smooth":
        wl = W.smooth_periodic(shape=(16, 12, 10), nchem=4)
    else:
        wl = W.rayleigh_taylor(shape=(10, 8, 12), nchem=4, seed=W.SEED_BASE + 600)
    h, w = _setup(torch, wl)
    # the RT interface (width 0.02) is a near-jump on a 12-cell column: there the central
    # difference itself carries ~1e-6 truncation error from the switching WENO weights, while
    # the smooth flow (the differentiation workload) is held to the 1e-6 target
    tol = 1e-6 if case == "smooth" else 1e-5
    rng = np.random.default_rng(20261203 + 5)
    for k in range(16):
        d = _dirs(torch, w, rng)
        jv = [torch.empty_like(x) for x in w]
        h.fEuler_jvp(0.0, w, d, jv)
        fp = _rhs(h, [a + H * b for a, b in zip(w, d)])
        fm = _rhs(h, [a - H * b for a, b in zip(w, d)])
        fd = [(a - b) / (2 * H) for a, b in zip(fp, fm)]
        for i, (a, b) in enumerate(zip(jv, fd)):
            assert maxnorm_err(a.cpu().numpy(), b.cpu().numpy()) <= tol, (k, i)
        # VJP: <J^T v, d> against the difference quotient of <v, f>
        v = _dirs(torch, w, rng)
        u = [torch.empty_like(x) for x in w]
        h.fEuler_vjp(0.0, w, v, u)
        lhs = _dot(u, d)
        rhs = (_dot(v, fp) - _dot(v, fm)) / (2 * H)
        assert abs(lhs - rhs) <= tol * max(abs(rhs), 1e-300) + tol * np.sqrt(
            _dot(u, u) * _dot(d, d)), (k, lhs, rhs)


@pytest.mark.parametrize("nchem,bc", [
    (0, (0, 0, 0, 0, 0, 0)),
    (4, (1, 1, 0, 0, 3, 3)),
    (10, (3, 1, 1, 3, 0, 0)),
    (2, (1, 3, 3, 1, 1, 1)),
])
def test_weno_vjp_dot_product_identity(cuda, nchem, bc):
    """<v, J dw> == <J^T v, dw> to rounding: the hand-written adjoint is the exact transpose
    of the dual-number linearisation, ghost rules included."""
    torch = cuda
    wl = W.rayleigh_taylor(shape=(9, 7, 8), nchem=nchem, seed=W.SEED_BASE + 610 + nchem)
    wl["bc"] = bc
    h, w = _setup(torch, wl)
    rng = np.random.default_rng(611 + nchem)
    for _ in range(4):
        d = _dirs(torch, w, rng)
        v = _dirs(torch, w, rng)
        jv = [torch.empty_like(x) for x in w]
        u = [torch.empty_like(x) for x in w]
        h.fEuler_jvp(0.0, w, d, jv)
        h.fEuler_vjp(0.0, w, v, u)
        a, b = _dot(v, jv), _dot(u, d)
        scale = np.sqrt(_dot(v, v) * _dot(jv, jv)) + np.sqrt(_dot(u, u) * _dot(d, d))
        assert abs(a - b) <= 1e-12 * scale, (a, b)


def test_chem_jvp_vjp_against_reference_jacobian(cuda, tables):
    torch = cuda
    import gbmv
    wl = W.chem_hydro(shape=(32, 32, 32))
    n = 32 ** 3
    TU = wl["units"]["TimeUnits"]
    scale = wl["scale"].reshape(-1)
    y = wl["fields"][5].reshape(-1).copy()
    c = gbmv.Chem(n, tables)
    c.set_scale(torch.from_numpy(scale.copy()).cuda())
    yd = torch.from_numpy(y).cuda()
    f = torch.empty_like(yd)
    c.calculate_rhs_cvklu(0.0, yd, f, TU)  # temperature state, as before a Jacobian call
    oc = O.Chem(tables, scale)
    oc.rhs(y)
    Jr = oc.jac(y) * TU                      # [cell][col][row]
    rng = np.random.default_rng(620)
    v = rng.standard_normal(10 * n)
    u = torch.empty_like(yd)
    c.vjp(0.0, yd, torch.from_numpy(v).cuda(), u, TU)
    ref_vjp = np.einsum("ncr,nr->nc", Jr, v.reshape(n, 10))
    got = u.cpu().numpy().reshape(n, 10)
    for s in range(10):
        assert maxnorm_err(got[:, s], ref_vjp[:, s]) <= 1e-12, s
    # JVP with unit directions assembles J column by column
    for col in range(10):
        e = np.zeros((n, 10))
        e[:, col] = 1.0
        jv = torch.empty_like(yd)
        c.jvp(0.0, yd, torch.from_numpy(e.reshape(-1)).cuda(), jv, TU)
        got = jv.cpu().numpy().reshape(n, 10)
        for r in range(10):
            assert maxnorm_err(got[:, r], Jr[:, col, r]) <= 1e-12, (col, r)


def test_gradient_through_50_rk4_steps_with_checkpoints(cuda):
    torch = cuda
    import ad_harness as AD
    n = 24
    wl = W.smooth_periodic(shape=(n, n, n), nchem=4)
    h, w0 = _setup(torch, wl)
    dx = 1.0 / n
    dt = 0.2 * dx / 1.4
    vol = dx ** 3
    L, g = AD.loss_and_grad(h, w0, dt, 50, vol, checkpoint_every=10)
    L2, g2 = AD.loss_and_grad(h, w0, dt, 50, vol, checkpoint_every=None)
    assert abs(L - L2) <= 1e-14 * abs(L)
    for a, b in zip(g, g2):  # recomputation from checkpoints reproduces the stored-stage grad
        assert torch.equal(a, b)
    rng = np.random.default_rng(630)
    for _ in range(3):
        d = _dirs(torch, w0, rng)
        ad = _dot(g, d)
        Lp = AD.loss_only(h, [a + H * b for a, b in zip(w0, d)], dt, 50, vol)
        Lm = AD.loss_only(h, [a - H * b for a, b in zip(w0, d)], dt, 50, vol)
        fd = (Lp - Lm) / (2 * H)
        assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)


def test_weno_jvp_vjp_vs_central_differences_at_96cube_masked(cuda):
    """The differentiation workload at its stated size (96^3 x 9 fields, h = 1e-7, 16 seeded
    directions): on every cell whose six faces keep their Lax-Friedrichs branch between
    w - h d, w and w + h d (gbmv_feuler_kink_mask), the central difference differentiates one
    smooth branch and must match the exact JVP to 1e-6 (max-normalised per field); the VJP
    identity <u, d> = <v, J d> with v supported on those cells likewise.  The masked cells are
    counted: a few per million, growing with h."""
    torch = cuda
    wl = W.smooth_periodic(n=96, nchem=4)
    h, w = _setup(torch, wl)
    rng = np.random.default_rng(W.SEED_BASE + 96)
    ncell = 96 ** 3
    mask = torch.empty(ncell, dtype=torch.uint8, device="cuda")
    jv = [torch.empty_like(x) for x in w]
    u = [torch.empty_like(x) for x in w]
    masked = 0
    for _ in range(16):
        d = _dirs(torch, w, rng)
        h.fEuler_jvp(0.0, w, d, jv)
        fp = _rhs(h, [a + H * b for a, b in zip(w, d)])
        fm = _rhs(h, [a - H * b for a, b in zip(w, d)])
        h.kink_mask(w, d, H, mask)
        keep = (mask == 0).view(w[0].shape)
        masked += int(ncell - int(keep.sum()))
        for k, (a, p, m) in enumerate(zip(jv, fp, fm)):
            fd = (p - m) / (2 * H)
            kk = keep if a.dim() == 3 else keep.unsqueeze(-1)
            err = float(((a - fd).abs() * kk).max()) / float(fd.abs().max())
            assert err <= 1e-6, (k, err)
        v = [x * (keep if x.dim() == 3 else keep.unsqueeze(-1)) for x in _dirs(torch, w, rng)]
        h.fEuler_vjp(0.0, w, v, u)
        lhs = _dot(u, d)
        r = (_dot(v, fp) - _dot(v, fm)) / (2 * H)
        assert abs(lhs - r) <= 1e-6 * abs(r), (lhs, r)
    assert masked < 16 * ncell * 1e-3, masked
