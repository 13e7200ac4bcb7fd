"""Host time integration for whole-run checks (SUNDIALS is not available here).

An adaptive explicit Runge-Kutta driver with ARKODE's error control conventions -- WRMS norm
of the embedded error with weights 1 / (rtol |y| + atol), step accepted when the norm is
<= 1, step-size update h * min(etamax, max(etamin, safety * err^(-1/q))) -- running the
Dormand-Prince 5(4) pair (FSAL).  The driver is array-library agnostic: `y` may be a numpy
array or a torch tensor (the GPU RHS keeps everything on the device); `rhs(t, y)` returns
dy/dt of the same kind.  It plays the role of ARKStep in euler3D_main.cpp's pure-hydro runs;
its step sequence is not SUNDIALS', so whole-run comparisons are made within the integration
tolerance.
"""
from __future__ import annotations

import math

# Dormand-Prince 5(4) (J. R. Dormand, P. J. Prince, J. Comput. Appl. Math. 6 (1980) 19-26)
_C = [0.0, 1 / 5, 3 / 10, 4 / 5, 8 / 9, 1.0, 1.0]
_A = [
    [],
    [1 / 5],
    [3 / 40, 9 / 40],
    [44 / 45, -56 / 15, 32 / 9],
    [19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
    [9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
    [35 / 384, 0.0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84],
]
_B = [35 / 384, 0.0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84, 0.0]
_BSTAR = [5179 / 57600, 0.0, 7571 / 16695, 393 / 640, -92097 / 339200, 187 / 2100, 1 / 40]
_E = [b - bs for b, bs in zip(_B, _BSTAR)]


def _wrms(e, y, rtol, atol):
    w = e / (rtol * abs(y) + atol)
    n = w.numel() if hasattr(w, "numel") else w.size
    return math.sqrt(float((w * w).sum()) / n)


class ERKResult:
    def __init__(self):
        self.steps = 0
        self.fails = 0
        self.nfe = 0


def erk_evolve(rhs, t0, tf, y0, rtol=1e-6, atol=1e-11, h0=0.0, safety=0.9, etamax=5.0,
               etamin=0.2, hmax=math.inf, max_steps=100000):
    """Integrate dy/dt = rhs(t, y) from t0 to tf; returns (y(tf), stats)."""
    st = ERKResult()
    y = y0.clone() if hasattr(y0, "clone") else y0.copy()
    t = t0
    k1 = rhs(t, y)
    st.nfe += 1
    if h0 <= 0.0:  # initial step from the derivative size (ARKODE estimates similarly)
        d0 = _wrms(y, y, rtol, atol)
        d1 = _wrms(k1, y, rtol, atol)
        h0 = 0.01 * d0 / d1 if d0 > 1e-5 and d1 > 1e-5 else 1e-6
    h = min(h0, tf - t0, hmax)
    while t < tf:
        if st.steps + st.fails > max_steps:
            raise RuntimeError("erk_evolve: too many steps")
        h = min(h, tf - t)
        ks = [k1]
        for s in range(1, 7):
            ys = y
            for j, a in enumerate(_A[s]):
                if a != 0.0:
                    ys = ys + (h * a) * ks[j]
            ks.append(rhs(t + _C[s] * h, ys))
            st.nfe += 1
        ynew = y
        for b, k in zip(_B, ks):
            if b != 0.0:
                ynew = ynew + (h * b) * k
        err = None
        for e, k in zip(_E, ks):
            if e != 0.0:
                err = (h * e) * k if err is None else err + (h * e) * k
        en = _wrms(err, ynew, rtol, atol)
        if not math.isfinite(en):
            en = 1e10
        if en <= 1.0:
            t += h
            y = ynew
            k1 = ks[6]  # FSAL
            st.steps += 1
        else:
            st.fails += 1
        fac = etamax if en == 0.0 else min(etamax, max(etamin, safety * en ** (-1.0 / 5.0)))
        h = min(h * fac, hmax)
    return y, st


def sod_exact(x, t, gamma=1.4, left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1), x0=0.5):
    """Exact solution of the Riemann problem (rho, u, p) at positions x and time t: the star
    pressure from Newton's method on the two-shock/rarefaction pressure functions, then the
    self-similar wave pattern (as in standard texts on Riemann solvers)."""
    import numpy as np
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = math.sqrt(gamma * pl / rl), math.sqrt(gamma * pr / rr)

    def fk(p, rk, pk, ck):
        if p > pk:  # shock
            A, B = 2.0 / ((gamma + 1) * rk), (gamma - 1) / (gamma + 1) * pk
            f = (p - pk) * math.sqrt(A / (p + B))
            df = math.sqrt(A / (B + p)) * (1 - (p - pk) / (2 * (B + p)))
        else:  # rarefaction
            f = 2 * ck / (gamma - 1) * ((p / pk) ** ((gamma - 1) / (2 * gamma)) - 1)
            df = 1 / (rk * ck) * (p / pk) ** (-(gamma + 1) / (2 * gamma))
        return f, df

    p = 0.5 * (pl + pr)
    for _ in range(100):
        f1, d1 = fk(p, rl, pl, cl)
        f2, d2 = fk(p, rr, pr, cr)
        dp = (f1 + f2 + ur - ul) / (d1 + d2)
        p = max(p - dp, 1e-12)
        if abs(dp) < 1e-14 * p:
            break
    f1, _ = fk(p, rl, pl, cl)
    f2, _ = fk(p, rr, pr, cr)
    us = 0.5 * (ul + ur) + 0.5 * (f2 - f1)
    g1, g2 = (gamma - 1) / (gamma + 1), (gamma - 1) / (2 * gamma)
    rsl = rl * (p / pl) ** (1 / gamma)                      # left rarefaction star density
    rsr = rr * ((p / pr) + g1) / (g1 * (p / pr) + 1)         # right shock star density
    csl = cl * (p / pl) ** g2
    shead, stail = ul - cl, us - csl
    sshock = ur + cr * math.sqrt((gamma + 1) / (2 * gamma) * p / pr + g2)
    xi = (np.asarray(x) - x0) / max(t, 1e-300)
    rho = np.empty_like(xi); u = np.empty_like(xi); pp = np.empty_like(xi)
    for n, s in enumerate(xi):
        if s < shead:
            rho[n], u[n], pp[n] = rl, ul, pl
        elif s < stail:  # inside the left rarefaction fan
            uf = 2 / (gamma + 1) * (cl + (gamma - 1) / 2 * ul + s)
            cf = 2 / (gamma + 1) * (cl + (gamma - 1) / 2 * (ul - s))
            rho[n], u[n], pp[n] = rl * (cf / cl) ** (2 / (gamma - 1)), uf, pl * (cf / cl) ** (2 * gamma / (gamma - 1))
        elif s < us:
            rho[n], u[n], pp[n] = rsl, us, p
        elif s < sshock:
            rho[n], u[n], pp[n] = rsr, us, p
        else:
            rho[n], u[n], pp[n] = rr, ur, pr
    return rho, u, pp


def scaled_forcing(g5, inv_scale, energy_units):
    """Slow chemistry tendency (physical densities; gas-energy slot = etdot in code units) to
    the scaled fast variables, in place: species * inv_scale, gas energy * EnergyUnits *
    inv_scale."""
    g5[:, :9].mul_(inv_scale[:, :9])
    g5[:, 9].mul_(inv_scale[:, 9] * energy_units)


class MRIResult:
    def __init__(self):
        self.slow_steps = 0
        self.slow_rhs = 0
        self.fast_failed_cells = 0


def mri_erk22b_evolve(gbmv, hydro, chem, w, t0, tf, h, energy_units, time_units,
                      precision=0, slow_rhs=None, **fast_opts):
    """Multirate chemistry-hydrodynamics integration (the MRIStep driver of
    src/multirate_chem_hydro_main.cpp) with a fixed slow step h: second-order explicit
    MRI-GARK coupling of the slow explicit midpoint rule (stage abscissae 0, 1/2, 1; inner
    forcings g1 = fs(Y1) on [t, t+h/2] and g2 = 2 fs(Y2) - fs(Y1) on [t+h/2, t+h], constant
    in time), the slow RHS fs = fexpl (WENO hydro + glue, `precision`), each fast problem
    w' = ffast(t, w) + g integrated by gbmv_mri_fast_evolve (persistent batched DIRK for the
    chemistry, exact forcing integral for the fluid).  With ffast = 0 it is the explicit
    midpoint rule, with fs = 0 the fast integrator alone.  `w` (six torch CUDA tensors) is
    advanced in place; returns an MRIResult.

    Units of the slow chemistry forcing: fexpl returns the chemistry tendency of the physical
    densities, with the total-energy tendency (code units) in the gas-energy slot, as the
    reference's fslow does (src/multirate_chem_hydro_main.cpp:1061-1074, TUnitScale = 1),
    while the fast variables are the scaled ones (chemistry / scale).  The reference adds the
    two as they are; here the forcing is converted to the scaled variables first -- species
    tendencies divided by scale, the gas-energy slot EnergyUnits * etdot / scale -- so that the
    coupling is dimensionally consistent (`scaled_forcing`)."""
    import torch
    res = MRIResult()
    fs0 = slow_rhs or (lambda t, y, out: gbmv.fexpl(hydro, chem, t, y, out, energy_units,
                                                    precision))
    inv_scale = chem.state("inv_scale").view(-1, 10)

    def fs(t, y, out):
        rc = fs0(t, y, out)
        if rc == 0:
            scaled_forcing(out[5].view(-1, 10), inv_scale, energy_units)
        return rc
    g1 = [torch.empty_like(x) for x in w]
    g2 = [torch.empty_like(x) for x in w]
    nsteps = int(round((tf - t0) / h))
    if nsteps < 1 or abs(nsteps * h - (tf - t0)) > 1e-12 * max(abs(tf), 1.0):
        raise ValueError("tf - t0 must be a whole number of slow steps")
    t = t0
    for n in range(nsteps):
        t_mid, t_end = t0 + (n + 0.5) * h, t0 + (n + 1) * h
        if fs(t, w, g1) != 0:
            raise RuntimeError("slow RHS failed (illegal state)")
        nf = gbmv.mri_fast_evolve(hydro, chem, t, t_mid, w, time_units, [g1], t, 1.0,
                                  precision=precision, **fast_opts)
        res.fast_failed_cells += nf
        if fs(t_mid, w, g2) != 0:
            raise RuntimeError("slow RHS failed (illegal state)")
        for a, b in zip(g2, g1):
            a.mul_(2.0).sub_(b)
        nf = gbmv.mri_fast_evolve(hydro, chem, t_mid, t_end, w, time_units, [g2], t_mid, 1.0,
                                  precision=precision, **fast_opts)
        res.fast_failed_cells += nf
        res.slow_rhs += 2
        res.slow_steps += 1
        t = t_end
    return res
