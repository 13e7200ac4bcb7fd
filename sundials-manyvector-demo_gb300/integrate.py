"""Host time integration over the drop-in entry points (SUNDIALS is not available here).

The ARKStep / MRIStep configurations the reference's main programs select, array-library
agnostic (`y` may be numpy arrays or torch tensors; the GPU problems keep everything on the
device):

  erk_evolve        adaptive (or fixed-step) explicit Runge-Kutta, any explicit table of
                    gbmv_butcher_table (ARKStepSetOrder / ARKStepSetTableNum with an explicit
                    table, src/euler3D_main.cpp:207-213);
  ark_imex_evolve   additive Runge-Kutta with modified Newton on the implicit stages, any
                    explicit / implicit / additive pair (ARKStepSetTableNum,
                    src/imex_chem_hydro_main.cpp:386);
  mri_gark_evolve   explicit MRI-GARK slow stepping over an inner fast integrator (MRIStep,
                    src/multirate_chem_hydro_main.cpp:529-560).

Error control is ARKODE's: WRMS norm of the embedded difference with weights
1 / (rtol |y| + atol), accepted when <= 1, step factor from its adaptivity controllers (PID,
PI or I, `adapt_method` 0 / 1 / 2, with its default gains, safety, bias and growth bounds).
The Butcher tables come from the library (gbmv_butcher_table), the single copy of the
coefficients the GPU integrator uses too.
"""
from __future__ import annotations

import math

def butcher(table_id):
    """Table `table_id` of the library (a dict of name, s, q, p, c, A, b, bhat)."""
    import gbmv
    return gbmv.butcher_table(table_id)


# ARKODE's adaptivity controllers (arkode_adapt.c): eta = safety * e_n^(-k1/k) e_{n-1}^(k2/k)
# e_{n-2}^(-k3/k), e = bias * dsm, k the embedding order, with the default gains of each
# method: 0 PID (0.58, 0.21, 0.10), 1 PI (0.8, 0.31), 2 I (1.0)
_ADAPT_GAINS = {0: (0.58, 0.21, 0.10), 1: (0.8, 0.31, 0.0), 2: (1.0, 0.0, 0.0)}


class Controller:
    """ARKODE's step-size adaptivity for an embedded pair of order p (ARKStep defaults:
    safety 0.96, bias 1.5, growth 20, etamx1 10^4 on the first step, etamxf 0.3 after small_nef
    error failures in one step, step factor kept at 1 inside [1, 1.5) to keep the Newton
    matrix, at least 0.1).  adapt_method 0 PID (default), 1 PI, 2 I; k1..k3 0 = the method's
    default gains; pq = 1 uses the method order q instead of p."""

    def __init__(self, p, q=None, adapt_method=0, k1=0.0, k2=0.0, k3=0.0, pq=0, safety=0.96,
                 bias=1.5, growth=20.0, etamx1=1e4, etamxf=0.3, small_nef=2):
        if adapt_method not in _ADAPT_GAINS:
            raise ValueError(f"adapt_method {adapt_method} is not available (0 PID, 1 PI, 2 I)")
        g = _ADAPT_GAINS[adapt_method]
        self.k = [k1 or g[0], (k2 or g[1]) if adapt_method < 2 else 0.0,
                  (k3 or g[2]) if adapt_method == 0 else 0.0]
        self.ord = q if (pq and q) else p
        self.safety, self.bias, self.growth = safety, bias, growth
        self.etamx1, self.etamxf, self.small_nef = etamx1, etamxf, small_nef
        self.ehist = [1.0, 1.0]  # bias * dsm of the last two accepted steps

    def _eta(self, dsm):
        e1 = max(self.bias * dsm, 1e-10)
        k = self.ord
        eta = e1 ** (-self.k[0] / k)
        if self.k[1]:
            eta *= self.ehist[0] ** (self.k[1] / k)
        if self.k[2]:
            eta *= self.ehist[1] ** (-self.k[2] / k)
        return self.safety * eta

    def accepted(self, dsm, first, after_failure):
        """Step factor after an accepted step with error norm dsm."""
        eta = min(self._eta(dsm), self.etamx1 if first else self.growth)
        if after_failure:
            eta = min(eta, 1.0)
        if 1.0 <= eta < 1.5:
            eta = 1.0
        eta = max(eta, 0.1)
        self.ehist = [max(self.bias * dsm, 1e-10), self.ehist[0]]
        return eta

    def rejected(self, dsm, nef):
        """Step factor after the nef-th error-test failure of a step."""
        eta = max(0.1, min(1.0, self.safety * max(self.bias * dsm, 1e-10) ** (-1.0 / self.ord)))
        if nef >= self.small_nef:
            eta = min(eta, self.etamxf)
        return eta


def _wrms(e, y, rtol, atol):
    w = e / (rtol * abs(y) + atol)
    n = w.numel() if hasattr(w, "numel") else w.size
    return math.sqrt(float((w * w).sum()) / n)


class ERKResult:
    def __init__(self):
        self.steps = 0
        self.fails = 0
        self.nfe = 0
        self.h_next = 0.0  # the step the controller proposes after the last one


def erk_evolve(rhs, t0, tf, y0, rtol=1e-6, atol=1e-11, h0=0.0, hmax=math.inf,
               max_steps=100000, fixed_h=0.0, stability=None, table=8, maxnef=7, **adapt):
    """Integrate dy/dt = rhs(t, y) from t0 to tf with the explicit table `table` (an ARKODE
    table number of gbmv_butcher_table, or a table dict; default Dormand-Prince 5(4)); returns
    (y(tf), stats).  A table whose last row is b with c = 1 reuses its last stage derivative
    as the next step's first (FSAL).  fixed_h > 0: steps of fixed_h (the last one shortened to
    reach tf) without error control, as ARKStep's fixed step mode.  stability(t, y): an
    explicitly stable step bound applied to every adaptive step (ARKStepSetStabilityFn, as
    the reference's CFL function `stability` is used).  adapt: Controller options
    (adapt_method, k1, k2, k3, pq, safety, bias, growth, etamx1, etamxf, small_nef)."""
    T = butcher(table) if not isinstance(table, dict) else table
    A, b, c, bh = T["A"], T["b"], T["c"], T["bhat"]
    ns = T["s"]
    e = [bi - bhi for bi, bhi in zip(b, bh)]
    fsal = c[-1] == 1.0 and list(A[-1][:ns - 1]) == list(b[:ns - 1]) and b[-1] == 0.0
    ctl = Controller(T["p"], T["q"], **adapt)
    st = ERKResult()
    y = y0.clone() if hasattr(y0, "clone") else y0.copy()
    t = t0
    k1 = rhs(t, y)
    st.nfe += 1
    if h0 <= 0.0:  # ARKODE's initial-step rule, on the explicit problem
        h0 = _initial_step(_ExplicitProblem(rhs, rtol, atol), t0, tf, [y], [k1], atol)
    h = fixed_h if fixed_h > 0.0 else min(h0, tf - t0, hmax)
    first, nef_s = True, 0
    while t < tf:
        if st.steps + st.fails > max_steps:
            raise RuntimeError("erk_evolve: too many steps")
        if stability is not None and fixed_h <= 0.0:
            h = min(h, stability(t, y))
        hp = h  # proposal before the cut to tf
        h = min(h, tf - t)
        cut = h < hp
        if fixed_h > 0.0 and h <= 1e-14 * max(abs(tf), 1.0):  # roundoff sliver of a fixed grid
            t = tf
            break
        ks = [k1]
        for i in range(1, ns):
            ys = y
            for j in range(i):
                if A[i][j] != 0.0:
                    ys = ys + (h * A[i][j]) * ks[j]
            ks.append(rhs(t + c[i] * h, ys))
            st.nfe += 1
        ynew = y
        for bj, k in zip(b, ks):
            if bj != 0.0:
                ynew = ynew + (h * bj) * k
        err = None
        for ej, k in zip(e, ks):
            if ej != 0.0:
                err = (h * ej) * k if err is None else err + (h * ej) * k
        en = 0.0 if (fixed_h > 0.0 or err is None) else _wrms(err, y, rtol, atol)
        if not math.isfinite(en):
            en = 1e10
        if en <= 1.0:
            t = tf if h == tf - t else t + h
            y = ynew
            k1 = ks[-1] if fsal else rhs(t, y)
            if not fsal:
                st.nfe += 1
            st.steps += 1
            if fixed_h > 0.0:
                h = fixed_h
                st.h_next = fixed_h
                continue
            eta = ctl.accepted(en, first, nef_s > 0)
            first, nef_s = False, 0
            h = min(h * eta, hmax)
            # a step cut short to land on tf does not shrink the proposal for the next interval
            st.h_next = max(h, hp) if cut else h
        else:
            st.fails += 1
            nef_s += 1
            if nef_s >= maxnef:
                raise RuntimeError("erk_evolve: too many error-test failures in one step")
            h *= ctl.rejected(en, nef_s)
            st.h_next = h
    return y, st


class GraphERK:
    """erk_evolve with every step one CUDA graph: the stages (right-hand sides and linear
    combinations), the embedded error's WRMS norm, ARKODE's controller and the accept / reject
    selection all run on the device (gbmv_step_begin / _end / _select, gbmv_wrms_norm_async),
    captured once and replayed; the host replays `batch` steps at a time and reads the step
    state (16 doubles) between batches, so no step waits for the host.

      rhs_async(y, out)        enqueue out = f(y) on the current stream (flat CUDA float64
                               tensors; graph-capturable; illegal states reported through
                               the caller's own device status word, read by `status()`)
      norm_async(v, y, out)    enqueue the WRMS norm of v with weights from y into out[0]
    `y` (a flat CUDA float64 tensor) is advanced in place.  The table is any explicit table
    of gbmv_butcher_table (default ARKODE's order-4 Zonneveld 5-3-4); the stage derivative at
    the step start is evaluated in every step graph (no FSAL reuse).  adapt: Controller
    options (adapt_method, k1, k2, k3, pq, safety, bias, growth, etamx1, etamxf, small_nef).
    Replays after the end time are no-ops apart from their launches (at most batch - 1).
    The graph is captured at the first `evolve` (its first step run eagerly outside the
    capture) and reused by later calls with the same controller settings, whatever the
    interval."""

    def __init__(self, rhs_async, norm_async, y, table=3, hmax=0.0, fixed_h=0.0, batch=16,
                 max_attempts=100000, maxnef=7, status=None, **adapt):
        import torch
        import gbmv
        self.g, self.torch = gbmv, torch
        self.T = butcher(table) if not isinstance(table, dict) else table
        T = self.T
        ctl = Controller(T["p"], T["q"], **adapt)
        self.rhs, self.norm, self.y, self.batch = rhs_async, norm_async, y, batch
        self.status_fn = status
        self.fixed_h, self.hmax = fixed_h, hmax
        self.ctl, self.max_attempts, self.maxnef = ctl, max_attempts, maxnef
        s = T["s"]
        coef = [T["A"][i][j] for i in range(s) for j in range(s)] + list(T["b"]) + \
               [bi - bhi for bi, bhi in zip(T["b"], T["bhat"])]
        dev = y.device
        self.coef = torch.tensor(coef, dtype=torch.float64, device=dev)
        self.hc = torch.empty_like(self.coef)
        self.k = [torch.empty_like(y) for _ in range(s)]
        self.ys, self.ynew, self.err = (torch.empty_like(y) for _ in range(3))
        self.dsm = torch.zeros(1, dtype=torch.float64, device=dev)
        self.state = torch.zeros(gbmv.STEP_STATE, dtype=torch.float64, device=dev)
        self.graph, self.params = None, None

    def _body(self):
        g, T, s = self.g, self.T, self.T["s"]
        A, b = T["A"], T["b"]
        e = [bi - bhi for bi, bhi in zip(T["b"], T["bhat"])]
        g.step_begin(self.state, self.params)
        ST = g.ST
        self.torch.mul(self.coef, self.state[ST["h_used"]:ST["h_used"] + 1], out=self.hc)
        hc = self.hc
        self.rhs(self.y, self.k[0])
        for i in range(1, s):
            self.ys.copy_(self.y)
            for j in range(i):
                if A[i][j] != 0.0:
                    self.ys.addcmul_(self.k[j], hc[i * s + j])
            self.rhs(self.ys, self.k[i])
        self.ynew.copy_(self.y)
        for j in range(s):
            if b[j] != 0.0:
                self.ynew.addcmul_(self.k[j], hc[s * s + j])
        self.err.zero_()
        for j in range(s):
            if e[j] != 0.0:
                self.err.addcmul_(self.k[j], hc[s * s + s + j])
        self.norm(self.err, self.y, self.dsm)
        g.step_end(self.state, self.dsm, self.params)
        g.step_select(self.state, self.y, self.ynew)

    def evolve(self, t0, tf, h0):
        """Advance y from t0 to tf starting with step h0 (> 0); returns an ERKResult."""
        torch, g = self.torch, self.g
        c = self.ctl
        fixed = self.fixed_h > 0.0
        p = g.step_params(c.ord, hmax=self.hmax if self.hmax < math.inf else 0.0,
                          safety=c.safety, bias=c.bias, growth=c.growth, etamx1=c.etamx1,
                          etamxf=c.etamxf, k1=c.k[0], k2=c.k[1], k3=c.k[2],
                          small_nef=c.small_nef, maxnef=self.maxnef,
                          max_attempts=self.max_attempts, fixed=fixed)
        st0 = [0.0] * g.STEP_STATE
        ST = g.ST
        st0[ST["t"]], st0[ST["tf"]] = t0, tf
        st0[ST["h"]] = self.fixed_h if fixed else h0
        st0[ST["first"]], st0[ST["e1"]], st0[ST["e2"]] = 1.0, 1.0, 1.0
        self.state.copy_(torch.tensor(st0, dtype=torch.float64))
        if self.graph is None or self.params is None or \
                bytes(self.params) != bytes(p):  # (re)capture for these parameters
            self.params = p
            y_save = self.y.clone()
            self._body()  # eager first step: first-use allocations happen outside the capture
            torch.cuda.synchronize()
            self.y.copy_(y_save)
            self.state.copy_(torch.tensor(st0, dtype=torch.float64))
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=side):
                self._body()
            torch.cuda.synchronize()
        res = ERKResult()
        while True:
            for _ in range(self.batch):
                self.graph.replay()
            st = self.state.cpu().tolist()
            if self.status_fn is not None and self.status_fn():
                raise RuntimeError("right-hand side reported an illegal state")
            if st[ST["status"]] < 0:
                raise RuntimeError("GraphERK: " + ("too many error-test failures in one step"
                                                   if st[ST["status"]] == -1 else
                                                   "max_attempts reached"))
            if st[ST["done"]] != 0.0:
                break
        res.steps = int(st[ST["steps"]])
        res.fails = int(st[ST["fails"]])
        res.nfe = int(st[ST["attempts"]]) * self.T["s"]
        res.h_next = st[ST["h"]]
        return res


class _ExplicitProblem:
    """The problem protocol of _initial_step for one explicit right-hand side."""

    def __init__(self, rhs, rtol, atol):
        self.rhs, self.rtol, self.atol = rhs, rtol, atol

    def fe(self, t, y):
        return [self.rhs(t, y[0])]

    def fi(self, t, y):
        return [None]

    def norm(self, v, y):
        return _wrms(v[0], y[0], self.rtol, self.atol)


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
            rho[n], u[n], pp[n] = (rl * (cf / cl) ** (2 / (gamma - 1)), uf,
                                   pl * (cf / cl) ** (2 * gamma / (gamma - 1)))
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


# Explicit MRI-GARK coupling tables (A. Sandu, SIAM J. Sci. Comput. 41 (2019) A2260-A2292): slow
# abscissae c and coefficient matrices G[k][i-1][j] -- the inner problem of stage i (from
# T_{i-1} = t + c_{i-1} h to T_i) is v' = ffast(v) + r_i(tau), r_i(tau) = (1/dc_i) sum_k tau^k
# sum_j G[k][i-1][j] fs(Y_j), tau = (t - T_{i-1}) / (dc_i h) in [0, 1], dc_i = c_i - c_{i-1};
# the last stage is y_{n+1}.
MRI_ERK22B = {"name": "MRI-GARK-ERK22b", "order": 2, "c": [0.0, 0.5, 1.0],
              "G": [[[0.5], [-0.5, 1.0]]]}
# the Knoth-Wolke third-order multirate infinitesimal step (MIS) method, whose slow table is
# c = (0, 1/3, 3/4), a21 = 1/3, a31 = -3/16, a32 = 15/16, b = (1/6, 3/10, 8/15)
# (O. Knoth, R. Wolke, Appl. Numer. Math. 28 (1998) 327-341), in MRI-GARK form:
# G[0][i-1][j] = a_{i,j} - a_{i-1,j} with a_{s+1,j} = b_j
MRI_KW3 = {"name": "MIS-KW3", "order": 3, "c": [0.0, 1.0 / 3.0, 0.75, 1.0],
           "G": [[[1.0 / 3.0], [-25.0 / 48.0, 15.0 / 16.0],
                  [17.0 / 48.0, -51.0 / 80.0, 8.0 / 15.0]]]}
MRI_ERK33A = {"name": "MRI-GARK-ERK33a", "order": 3, "c": [0.0, 1.0 / 3.0, 2.0 / 3.0, 1.0],
              "G": [[[1.0 / 3.0], [-1.0 / 3.0, 2.0 / 3.0], [0.0, -2.0 / 3.0, 1.0]],
                    [[0.0], [0.0, 0.0], [0.5, 0.0, -0.5]]]}


def mri_gark_evolve(slow_rhs, fast_evolve, t0, tf, y, h, table=MRI_ERK22B):
    """Explicit MRI-GARK integration with a fixed slow step h (MRIStep's slow stepping):
    slow_rhs(t, y) -> list of slow tendencies; fast_evolve(ta, tb, y, forcing, tshift, tscale)
    advances y in place over [ta, tb] under ffast + sum_k ((t - tshift)/tscale)^k forcing[k].
    Array-library agnostic.  Returns an MRIResult."""
    res = MRIResult()
    c, G = table["c"], table["G"]
    ns = len(c)
    nsteps = int(round((tf - t0) / h))
    if nsteps < 1 or abs(nsteps * h - (tf - t0)) > 1e-12 * max(abs(tf), 1.0):
        raise ValueError("tf - t0 must be a whole number of slow steps")
    for n in range(nsteps):
        t = t0 + n * h
        F = [slow_rhs(t, y)]
        res.slow_rhs += 1
        for i in range(1, ns):
            dc = c[i] - c[i - 1]
            ta, tb = t + c[i - 1] * h, t + c[i] * h
            forcing = []
            for Gk in G:
                row = Gk[i - 1]
                terms = [(row[j] / dc, F[j]) for j in range(len(row)) if row[j] != 0.0]
                forcing.append(_combo(None, terms) if terms else [x * 0.0 for x in F[0]])
            while len(forcing) > 1 and all(v == 0.0 for v in G[len(forcing) - 1][i - 1]):
                forcing.pop()  # drop vanishing top powers for this stage
            res.fast_failed_cells += fast_evolve(ta, tb, y, forcing, ta, dc * h) or 0
            if i < ns - 1:
                F.append(slow_rhs(tb, y))
                res.slow_rhs += 1
        res.slow_steps += 1
    return res


FORCING_UNITS = ("reference", "scaled")


def mri_evolve(gbmv, hydro, chem, w, t0, tf, h, energy_units, time_units, table=MRI_KW3,
               precision=0, slow_rhs=None, forcing_units="reference", itable=112,
               **fast_opts):
    """Multirate chemistry-hydrodynamics integration (the MRIStep driver of
    src/multirate_chem_hydro_main.cpp) with a fixed slow step h and an explicit MRI-GARK
    coupling `table`, by default MIS-KW3, MRIStep's default third-order explicit coupling that
    the reference runs when its input leaves `mtable` negative
    (src/multirate_chem_hydro_main.cpp:18, :545-551; inputs/input_generic.txt:49): the slow RHS fs = fexpl (WENO hydro + glue, `precision`), each fast
    problem w' = ffast(t, w) + r(t) with the stage's forcing polynomial integrated by
    gbmv_mri_fast_evolve (persistent batched DIRK for the chemistry, exact forcing integral
    for the fluid).  `w` (six torch CUDA tensors) is advanced in place; returns an MRIResult.

    Units of the slow chemistry forcing: fexpl returns the chemistry tendency of the physical
    densities, with the total-energy tendency (code units) in the gas-energy slot, as the
    reference's fslow does (src/multirate_chem_hydro_main.cpp:1061-1074, TUnitScale = 1),
    while the fast variables are the scaled ones (chemistry / scale).  forcing_units
    "reference" (the default) adds the two as they are, as the reference does;
    "scaled" converts the forcing to the scaled variables first -- species tendencies divided
    by scale, the gas-energy slot EnergyUnits * etdot / scale (`scaled_forcing`) -- which makes
    the coupling dimensionally consistent, a departure from the reference to select
    explicitly.  itable: the inner DIRK's table (the inputs' itable: 112 ARK4(3)7L[2]SA or 102
    TR-BDF2); fast_opts: the other gbmv_dirk_opts fields of the inner DIRK."""
    import torch
    if forcing_units not in FORCING_UNITS:
        raise ValueError(f"forcing_units must be one of {FORCING_UNITS}")
    fs0 = slow_rhs or (lambda t, y, out: gbmv.fexpl(hydro, chem, t, y, out, energy_units,
                                                    precision))
    inv_scale = chem.state("inv_scale").view(-1, 10)

    def fs(t, y):
        out = [torch.empty_like(x) for x in y]
        if fs0(t, y, out) != 0:
            raise RuntimeError("slow RHS failed (illegal state)")
        if forcing_units == "scaled":
            scaled_forcing(out[5].view(-1, 10), inv_scale, energy_units)
        return out

    def fast(ta, tb, y, forcing, tshift, tscale):
        return gbmv.mri_fast_evolve(hydro, chem, ta, tb, y, time_units, forcing, tshift, tscale,
                                    precision=precision, table=itable, **fast_opts)

    return mri_gark_evolve(fs, fast, t0, tf, w, h, table)


class GraphMRI:
    """mri_evolve with every slow step one CUDA graph: the slow right-hand sides
    (gbmv_fexpl_async), the stage forcing polynomials (linear combinations into preallocated
    ManyVectors) and the fast evolves (gbmv_mri_fast_evolve_async, the persistent DIRK) of all
    stages are captured once and replayed per slow step; illegal states and failed cells land
    in device words read once per `evolve` call.  The chemistry network is autonomous, so each
    stage's inner problem runs on local time [0, dc h] with tshift 0 and tscale dc h (the same
    forcing polynomial as tau = (t - T_{i-1}) / (dc h)), which makes every slow step's graph
    the same.  Options as mri_evolve; fast_opts must allow the DIRK block size to be tuned
    by the eager first step (block 0) or fix it."""

    def __init__(self, gbmv, hydro, chem, w, h, energy_units, time_units, table=MRI_KW3,
                 precision=0, forcing_units="reference", itable=112, **fast_opts):
        import torch
        if forcing_units not in FORCING_UNITS:
            raise ValueError(f"forcing_units must be one of {FORCING_UNITS}")
        self.g, self.torch = gbmv, torch
        self.hydro, self.chem, self.w, self.h = hydro, chem, w, h
        self.eu, self.tu, self.table, self.precision = energy_units, time_units, table, precision
        self.units, self.fast_opts = forcing_units, dict(fast_opts, table=itable)
        dev = w[0].device
        sizes = [x.numel() for x in w]
        self.sizes = sizes
        ns = len(table["c"])

        def mv():
            flat = torch.empty(sum(sizes), dtype=torch.float64, device=dev)
            return flat, [v.view(x.shape) for v, x in zip(torch.split(flat, sizes), w)]
        self.F = [mv() for _ in range(ns - 1)]
        self.force = [[mv() for _ in table["G"]] for _ in range(ns)]
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.nfail = torch.zeros(1, dtype=torch.int32, device=dev)
        self.inv9 = chem.state("inv_scale").view(-1, 10)[:, :9]
        self.inv_ge = chem.state("inv_scale").view(-1, 10)[:, 9] * energy_units
        self.graph = None

    def _slow(self, j):
        flat, comps = self.F[j]
        self.g.fexpl_async(self.hydro, self.chem, 0.0, self.w, comps, self.eu, self.status,
                           self.precision)
        if self.units == "scaled":
            c5 = comps[5].view(-1, 10)
            c5[:, :9].mul_(self.inv9)
            c5[:, 9].mul_(self.inv_ge)

    def _body(self):
        c, G, h = self.table["c"], self.table["G"], self.h
        ns = len(c)
        self._slow(0)
        for i in range(1, ns):
            dc = c[i] - c[i - 1]
            forcing = []
            for q, Gk in enumerate(G):
                row = Gk[i - 1]
                flat, comps = self.force[i][q]
                flat.zero_()
                for j in range(len(row)):
                    if row[j] != 0.0:
                        flat.add_(self.F[j][0], alpha=row[j] / dc)
                forcing.append(comps)
            while len(forcing) > 1 and all(v == 0.0 for v in G[len(forcing) - 1][i - 1]):
                forcing.pop()  # drop vanishing top powers for this stage
            self.g.mri_fast_evolve_async(self.hydro, self.chem, 0.0, dc * h, self.w, self.tu,
                                         self.nfail, forcing, 0.0, dc * h,
                                         precision=self.precision, **self.fast_opts)
            if i < ns - 1:
                self._slow(i)

    def evolve(self, t0, tf):
        """Advance w by whole slow steps from t0 to tf; returns an MRIResult."""
        torch = self.torch
        nsteps = int(round((tf - t0) / self.h))
        if nsteps < 1 or abs(nsteps * self.h - (tf - t0)) > 1e-12 * max(abs(tf), 1.0):
            raise ValueError("tf - t0 must be a whole number of slow steps")
        res = MRIResult()
        ns = len(self.table["c"])
        start = 0
        if self.graph is None:
            # the first step eagerly: the DIRK block-size tuning and first-use allocations
            # happen outside the capture
            if not self.fast_opts.get("block"):  # tune on copies of the state
                keep = [self.chem.state(k).clone() for k in ("Ts", "dTs_ge")]
                self.g.mri_fast_evolve(self.hydro, self.chem, 0.0, self.h * 1e-6,
                                       [x.clone() for x in self.w], self.tu,
                                       precision=self.precision, **self.fast_opts)
                for k, v in zip(("Ts", "dTs_ge"), keep):
                    self.chem.state(k).copy_(v)
                self.fast_opts["block"] = self.chem.dirk_block(self.precision)
            self._body()
            torch.cuda.synchronize()
            start = 1
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=side):
                self._body()
            torch.cuda.synchronize()
        for _ in range(start, nsteps):
            self.graph.replay()
        st, nf = int(self.status.item()), int(self.nfail.item())
        if st:
            raise RuntimeError(f"slow RHS: illegal state (mask {st})")
        res.slow_steps = nsteps
        res.slow_rhs = nsteps * (ns - 1)
        res.fast_failed_cells = nf
        self.nfail.zero_()
        return res


def mri_erk22b_evolve(gbmv, hydro, chem, w, t0, tf, h, energy_units, time_units,
                      precision=0, slow_rhs=None, **kw):
    """mri_evolve with the second-order MRI-GARK-ERK22b coupling (explicit midpoint: forcings
    g1 = fs(Y1) on [t, t+h/2] and g2 = 2 fs(Y2) - fs(Y1) on [t+h/2, t+h])."""
    return mri_evolve(gbmv, hydro, chem, w, t0, tf, h, energy_units, time_units, MRI_ERK22B,
                      precision, slow_rhs, **kw)


# ---------------------------------------------------------------------------- ARK-IMEX


def ark_table(etable=2, itable=104):
    """The additive method ARKStepSetTableNum(itable, etable) selects (src/imex_chem_hydro_main.
    cpp:386): both >= 0 an IMEX pair (they must share c, b and bhat: ARK3(2)4L[2]SA = (2, 104),
    ARK4(3)7L[2]SA = (13, 112)), only itable >= 0 a DIRK on fi alone, only etable >= 0 an ERK
    on fe alone.  Returns a dict with name, q, p, c, b, bhat, ae (strictly lower rows), ai
    (rows with the diagonal), explicit, implicit."""
    if etable < 0 and itable < 0:
        raise ValueError("at least one of etable / itable must name a table")
    E = butcher(etable) if etable >= 0 else None
    Im = butcher(itable) if itable >= 0 else None
    for T, kind in ((E, "explicit"), (Im, "implicit")):
        if T is None:
            continue
        A = T["A"]
        diag = [A[i][i] for i in range(T["s"])]
        if kind == "explicit" and any(diag):
            raise ValueError(f"table {T['id']} is not explicit")
        if kind == "implicit" and not (diag[0] == 0.0 and all(d == diag[1] for d in diag[1:])
                                       and diag[1] > 0.0):
            raise ValueError(f"table {T['id']} is not an ESDIRK with one diagonal value")
    if E is not None and Im is not None and (E["c"] != Im["c"] or E["b"] != Im["b"] or
                                             E["bhat"] != Im["bhat"]):
        raise ValueError(f"tables {etable} and {itable} are not an additive pair")
    B = E if E is not None else Im
    s = B["s"]
    return {"name": "+".join(T["name"] for T in (E, Im) if T is not None),
            "q": B["q"], "p": B["p"], "c": B["c"], "b": B["b"], "bhat": B["bhat"],
            "ae": [list(E["A"][i][:i]) if E else [0.0] * i for i in range(s)],
            "ai": [list(Im["A"][i][:i + 1]) if Im else [0.0] * (i + 1) for i in range(s)],
            "explicit": E is not None, "implicit": Im is not None}


class ImexResult:
    def __init__(self):
        self.steps = 0       # accepted steps
        self.attempts = 0    # step attempts
        self.netf = 0        # error-test failures
        self.ncf = 0         # nonlinear (Newton) convergence failures
        self.nni = 0         # Newton iterations
        self.nsetups = 0     # Newton-matrix setups (Jacobian + factorisation)
        self.nfe = 0         # explicit RHS evaluations
        self.nfi = 0         # implicit RHS evaluations
        self.h_last = 0.0    # last accepted step
        self.h_next = 0.0    # the step the controller would attempt next (the restart h0)


def _combo(base, terms):
    """base + sum coef * vec over ManyVector component lists (None components are zero);
    base None: the sum alone."""
    out = []
    for k in range(len(terms[0][1]) if base is None else len(base)):
        acc = None if base is None else base[k]
        for coef, vec in terms:
            v = vec[k]
            if v is not None and coef != 0.0:
                acc = coef * v if acc is None else acc + coef * v
        out.append(acc)
    return out


def _fsum(fe_, fi_):
    """fe + fi over ManyVector component lists, either may be None (absent part)."""
    if fe_ is None:
        return fi_
    if fi_ is None:
        return fe_
    return _combo(fe_, [(1.0, fi_)])


class _PartProblem:
    """fe / fi of a problem with the absent part of the method's table returning None."""

    def __init__(self, prob, use_e, use_i):
        self.p, self.use_e, self.use_i = prob, use_e, use_i

    def fe(self, t, y):
        return self.p.fe(t, y) if self.use_e else [None] * len(y)

    def fi(self, t, y):
        return self.p.fi(t, y) if self.use_i else [None] * len(y)

    def norm(self, v, y):
        return self.p.norm(v, y)


def _clone(x):
    return x.clone() if hasattr(x, "clone") else x.copy()


def _initial_step(prob, t0, tf, y, f0, atol):
    """First step size when none is given, by the rule ARKODE (arkHin) and CVODE (CVHin) use:
    bounds hlb = 100 u max(|t0|, |tf|) and hub = min(0.1 |tf - t0|, 1 / max_i |f_i| /
    (0.1 |y_i| + atol)); starting from sqrt(hlb hub), up to four estimates
    h = sqrt(2 / ||y''||) with y'' ~ (f(t0 + h, y0 + h f0) - f0) / h, accepted when two agree
    within a factor 2; then half of it, clipped to [hlb, hub].  The trial evaluations use a
    copy of y."""
    tdist = abs(tf - t0)
    hlb = 100.0 * 2.220446049250313e-16 * max(abs(t0), abs(tf))
    inv = 0.0
    for yk, fk in zip(y, f0):
        if (fk.numel() if hasattr(fk, "numel") else fk.size) > 0:
            inv = max(inv, float((abs(fk) / (0.1 * abs(yk) + atol)).max()))
    hub = 0.1 * tdist
    if hub * inv > 1.0:
        hub = 1.0 / inv
    hg = math.sqrt(hlb * hub)
    if hub < hlb:
        return hg
    hnew = hg
    for count in range(1, 5):
        ytry = _combo(y, [(hg, f0)])
        ftry = _combo(prob.fe(t0 + hg, ytry), [(1.0, prob.fi(t0 + hg, ytry))])
        ydd = prob.norm(_combo(None, [(1.0 / hg, ftry), (-1.0 / hg, f0)]), y)
        hnew = math.sqrt(2.0 / ydd) if ydd * hub * hub > 2.0 else math.sqrt(hg * hub)
        if count == 4:
            break
        hrat = hnew / hg
        if 0.5 < hrat < 2.0:
            break
        if count >= 2 and hrat > 2.0:
            hnew = hg
            break
        hg = hnew
    return min(max(0.5 * hnew, hlb), hub)


def ark_imex_evolve(prob, t0, tf, y, rtol=1e-6, atol=1e-10, h0=0.0, hmax=math.inf,
                    fixed_h=0.0, etacf=0.25, maxnef=7, maxncf=10, maxcor=3, nlscoef=0.1,
                    crdown=0.3, rdiv=2.3, dgmax=0.2, msbp=20, max_steps=5000, table=None,
                    **adapt):
    """Adaptive additive Runge-Kutta (IMEX) integration of y' = fe(t, y) + fi(t, y) from t0 to
    tf, the ARKStep configuration of src/imex_chem_hydro_main.cpp:337-475 (fexpl explicit,
    fimpl implicit, the block-diagonal direct solver on the chemistry subvector, a
    PostprocessStep after every step).  `y` is a list of ManyVector components (numpy arrays
    or torch tensors) advanced in place; `prob` supplies

      fe(t, y) -> list               explicit RHS (may rewrite dependent fields of y, as the
                                     reference's fexpl rewrites et)
      fi(t, y) -> list               implicit RHS, None for components it does not touch
      setup(t, y, gamma) -> int      form and factor M = I - gamma dfi/dy at y (0 ok, > 0 a
                                     recoverable failure such as a singular block)
      solve(b) -> list               M^{-1} b (identity on the components fi does not touch)
      norm(v, y) -> float            WRMS norm of v with weights 1 / (rtol |y| + atol)
      postprocess(t, y)              optional, after every accepted step
      correction(t, z, a, gamma)     optional: one full Newton correction of the stage equation
                                     at z with the Newton matrix formed afresh (used instead of
                                     fi / setup / solve when prob.fused_newton is true)

    Each implicit stage z = a + gamma fi(t_i, z) is solved by modified Newton from the trivial
    predictor z = y_n with ARKODE's rules: matrix set up again when gamma moved by more than
    dgmax since the last setup, after msbp steps, or after a convergence failure with a matrix
    from an earlier step; correction scaled by 2 / (1 + gamma / gamma_p) against a lagged
    matrix; rate estimate crate = max(crdown crate, del / del_p); converged when
    min(1, crate) del / nlscoef <= 1; divergence when del > rdiv del_p; at most maxcor
    iterations; a failure with a current matrix cuts the step by etacf.  With
    prob.fused_newton the stage iterations are full Newton steps from prob.correction (the
    matrix current at every iterate, so no setups, lagging or gamma-ratio scaling) under the
    same convergence test.  Error control: WRMS norm dsm of the embedded difference with
    weights from y_n, accepted when dsm <= 1, the step factor from ARKODE's controller
    (`Controller`, adapt options adapt_method, k1-k3, pq, safety, bias, growth, etamx1,
    etamxf, small_nef); h <= hmax.  fixed_h > 0 takes fixed steps without error control.
    table: ark_table(...) (default ARK3(2)4L[2]SA, ARKStep's default IMEX method); with an
    explicit-only table fi, setup and solve are not used, with an implicit-only one fe is
    not.  Defaults are ARKODE's; the reference's IMEX inputs use safety 0.99, bias 2, growth
    2, maxcor 10, nlscoef 0.01 and the ARK4(3)7L[2]SA pair.  Returns an ImexResult; raises
    RuntimeError when a step cannot be completed."""
    st = ImexResult()
    table = table if table is not None else ark_table(2, 104)
    ae, ai, c = table["ae"], table["ai"], table["c"]
    b, bh = table["b"], table["bhat"]
    e = [x - xh for x, xh in zip(b, bh)]
    ns = len(c)
    use_e, use_i = table.get("explicit", True), table.get("implicit", True)
    ctl = Controller(table["p"], table.get("q"), **adapt)
    post = getattr(prob, "postprocess", None)
    fused = bool(getattr(prob, "fused_newton", False))
    t = t0
    gp, nst_lp, crate = 0.0, 0, 1.0
    force_setup, jcur = True, False
    F0 = None  # (Fe, Fi) at (t, y), kept across retries of a step
    h = fixed_h if fixed_h > 0.0 else h0
    first = True
    nef_s = ncf_s = 0
    while t < tf:
        if st.attempts >= max_steps:
            raise RuntimeError("ark_imex_evolve: max_steps attempts reached")
        if F0 is None:
            F0 = (prob.fe(t, y) if use_e else None, prob.fi(t, y) if use_i else None)
            st.nfe += int(use_e)
            st.nfi += int(use_i)
        if h <= 0.0:
            h = _initial_step(_PartProblem(prob, use_e, use_i), t, tf, y,
                              _fsum(F0[0], F0[1]), atol)
        h = min(h, hmax)
        last = tf - t <= h * (1.0 + 1e-8)  # stretch a step by a rounding sliver onto tf
        if last:
            h = tf - t
        st.attempts += 1
        Fe, Fi = [F0[0]], [F0[1]]
        conv_fail = False
        for i in range(1, ns):
            ti = t + c[i] * h
            gam = h * ai[i][i]
            a = _combo(y, [(h * ae[i][j], Fe[j]) for j in range(i) if Fe[j] is not None] +
                       [(h * ai[i][j], Fi[j]) for j in range(i) if Fi[j] is not None])
            if not use_i:  # explicit stage
                Fe.append(prob.fe(ti, a))
                Fi.append(None)
                st.nfe += 1
                continue
            z = [_clone(x) for x in y]  # trivial predictor
            m, delp = 0, 0.0
            if fused:
                jcur = True  # the rate estimate carries across stages, as between setups
            while True:
                if fused:
                    d = prob.correction(ti, z, a, gam)
                    st.nfi += 1
                    st.nsetups += 1
                    if d is None:  # a singular block
                        conv_fail = True
                        break
                else:
                    fiz = prob.fi(ti, z)
                    st.nfi += 1
                    if (force_setup or st.steps >= nst_lp + msbp or
                            not abs(gam / gp - 1.0) <= dgmax):
                        rc = prob.setup(ti, z, gam)
                        st.nsetups += 1
                        gp, nst_lp, crate = gam, st.steps, 1.0
                        jcur, force_setup = True, False
                        if rc != 0:
                            conv_fail = True
                            break
                    r = _combo(a, [(-1.0, z), (gam, fiz)])
                    d = prob.solve(r)
                    if gam != gp:
                        sc = 2.0 / (1.0 + gam / gp)
                        d = [x * sc for x in d]
                z = _combo(z, [(1.0, d)])
                dn = prob.norm(d, y)
                m += 1
                st.nni += 1
                if m > 1:
                    crate = max(crdown * crate, dn / delp)
                if min(crate, 1.0) * dn / nlscoef <= 1.0:
                    break
                if (m > 1 and dn > rdiv * delp) or m >= maxcor or not math.isfinite(dn):
                    conv_fail = True
                    break
                delp = dn
            if conv_fail:
                break
            Fe.append(prob.fe(ti, z) if use_e else None)
            Fi.append(prob.fi(ti, z))
            st.nfe += int(use_e)
            st.nfi += 1
        if conv_fail:
            st.ncf += 1
            ncf_s += 1
            if ncf_s >= maxncf:
                raise RuntimeError("ark_imex_evolve: too many Newton failures in one step")
            if fixed_h > 0.0:
                raise RuntimeError("ark_imex_evolve: Newton failure at a fixed step")
            if jcur:
                h *= etacf
            else:
                force_setup = True
            continue
        F = [_fsum(fe_, fi_) for fe_, fi_ in zip(Fe, Fi)]
        ynew = _combo(y, [(h * b[j], F[j]) for j in range(ns)])
        if fixed_h > 0.0:
            dsm = 0.0
        else:
            err = _combo(None, [(h * e[j], F[j]) for j in range(ns)])
            dsm = prob.norm(err, y)
            if not math.isfinite(dsm):
                dsm = 1e10
        if dsm <= 1.0:
            t = tf if last else t + h
            for k in range(len(y)):
                if hasattr(y[k], "copy_"):
                    y[k].copy_(ynew[k])
                else:
                    y[k][...] = ynew[k]
            st.steps += 1
            st.h_last = h
            if post is not None:
                post(t, y)
            F0 = None
            jcur = False
            if fixed_h > 0.0:
                h = fixed_h
            else:
                h = min(h * ctl.accepted(dsm, first, nef_s > 0 or ncf_s > 0), hmax)
            first = False
            nef_s = ncf_s = 0
        else:
            st.netf += 1
            nef_s += 1
            if nef_s >= maxnef:
                raise RuntimeError("ark_imex_evolve: too many error-test failures in one step")
            h *= ctl.rejected(dsm, nef_s)
    st.h_next = h
    return st


def batched_equilibrate(A, sweeps=10):
    """Row and column factors (r, c), each [ncell, k], that equilibrate every block of A
    ([ncell, k, k]): diag(r) A diag(c) has the maxima of its rows and columns near 1 (Ruiz's
    iteration: each sweep divides the rows, then the columns, by
    the square roots of their maxima; D. Ruiz, "A scaling algorithm to equilibrate both rows
    and columns norms in matrices", RAL-TR-2001-034).  Zero rows or columns keep factor 1.
    The scaling for batched_gmres (precond=r, right=c) on badly scaled blocks."""
    import torch
    B = A.abs()
    r = torch.ones(A.shape[:2], dtype=A.dtype, device=A.device)
    c = torch.ones_like(r)
    for _ in range(sweeps):
        mr = B.amax(dim=2)
        dr = torch.where(mr > 0, torch.rsqrt(mr), torch.ones_like(mr))
        B = B * dr[:, :, None]
        r = r * dr
        mc = B.amax(dim=1)
        dc = torch.where(mc > 0, torch.rsqrt(mc), torch.ones_like(mc))
        B = B * dc[:, None, :]
        c = c * dc
    return r, c


def batched_gmres(matvec, b, m=10, rtol=1e-13, precond=None, right=None, cycles=1):
    """Matrix-free GMRES on many independent small systems at once: b is [ncell, k] (one
    right-hand side of k entries per cell), matvec(v) applies every cell's operator to the
    rows of v ([ncell, k]).  Each cell builds its own Krylov basis (Arnoldi with modified
    Gram-Schmidt and one re-orthogonalisation, Givens rotations on its Hessenberg matrix), all
    cells advancing together, one matvec per iteration for all of them; at most m iterations
    (m = k solves each system exactly in exact arithmetic), fewer once every cell's residual
    is below rtol times its |b|.  A cell stops using its basis at its own convergence or at a
    breakdown of its Arnoldi process (a zero new vector: its Krylov space is invariant), so
    later iterations of the other cells leave its solution alone.  Scaling: precond, None or per-row factors dl [ncell, k] (left), and
    right, None or per-column factors dr (right): GMRES then runs on diag(dl) A diag(dr) u =
    diag(dl) b and returns x = diag(dr) u.  cycles > 1 restarts from the residual b - A x
    (restarted GMRES(m)).  Returns (x [ncell, k], total iterations)."""
    import torch
    if cycles > 1:
        x, its = batched_gmres(matvec, b, m, rtol, precond, right)
        for _ in range(cycles - 1):
            dx, it = batched_gmres(matvec, b - matvec(x), m, rtol, precond, right)
            x, its = x + dx, its + it
        return x, its
    if precond is not None or right is not None:
        dl = precond if precond is not None else torch.ones_like(b)
        dr = right if right is not None else torch.ones_like(b)
        u, it = batched_gmres(lambda v: dl * matvec(dr * v), dl * b, m, rtol)
        return dr * u, it
    n, k = b.shape
    m = min(m, k)
    dt = b.dtype
    beta = torch.linalg.vector_norm(b, dim=1)
    safe = torch.where(beta > 0, beta, torch.ones_like(beta))
    V = [b / safe[:, None]]
    H = torch.zeros(n, m + 1, m, dtype=dt, device=b.device)
    cs = torch.zeros(n, m, dtype=dt, device=b.device)
    sn = torch.zeros(n, m, dtype=dt, device=b.device)
    g = torch.zeros(n, m + 1, dtype=dt, device=b.device)
    g[:, 0] = beta
    # columns of the basis each cell uses: it stops at convergence or breakdown
    kc = torch.where(beta > 0, torch.full_like(beta, m, dtype=torch.long),
                     torch.zeros_like(beta, dtype=torch.long))
    it = 0
    for j in range(m):
        w = matvec(V[j])
        for _ in range(2):  # modified Gram-Schmidt, twice
            for i in range(j + 1):
                hij = (w * V[i]).sum(dim=1)
                H[:, i, j] += hij
                w = w - hij[:, None] * V[i]
        hn = torch.linalg.vector_norm(w, dim=1)
        H[:, j + 1, j] = hn
        V.append(w / torch.where(hn > 0, hn, torch.ones_like(hn))[:, None])
        for i in range(j):  # earlier rotations on the new column
            a, c = H[:, i, j].clone(), H[:, i + 1, j].clone()
            H[:, i, j] = cs[:, i] * a + sn[:, i] * c
            H[:, i + 1, j] = -sn[:, i] * a + cs[:, i] * c
        a, c = H[:, j, j], H[:, j + 1, j]
        r = torch.sqrt(a * a + c * c)
        rs = torch.where(r > 0, r, torch.ones_like(r))
        cs[:, j] = torch.where(r > 0, a / rs, torch.ones_like(r))
        sn[:, j] = torch.where(r > 0, c / rs, torch.zeros_like(r))
        H[:, j, j] = r
        H[:, j + 1, j] = 0.0
        g[:, j + 1] = -sn[:, j] * g[:, j]
        g[:, j] = cs[:, j] * g[:, j]
        it = j + 1
        done = (g[:, j + 1].abs() <= rtol * beta) | (hn == 0)
        kc = torch.where(done & (kc > j + 1), torch.full_like(kc, j + 1), kc)
        if bool((kc <= j + 1).all()):
            break
    R = H[:, :it, :it]
    cols = torch.arange(it, device=b.device)
    unused = cols[None, :] >= kc[:, None]  # basis columns past the cell's own stop
    diag = torch.diagonal(R, dim1=1, dim2=2)
    dead = unused | (diag == 0)
    R = torch.where(dead[:, None, :], torch.zeros_like(R), R) + torch.diag_embed(dead.to(dt))
    gy = torch.where(dead, torch.zeros_like(g[:, :it]), g[:, :it])
    y = torch.linalg.solve_triangular(R, gy[:, :, None], upper=True)[:, :, 0]
    x = torch.zeros_like(b)
    for i in range(it):
        x = x + y[:, i:i + 1] * V[i]
    return x, it


class ChemHydroImex:
    """The reference's IMEX splitting (src/imex_chem_hydro_main.cpp) over the drop-in entry
    points, all on the device: fe = fexpl (WENO flux divergence of every field and the
    gas-energy coupling, :910-1000; with forcing_units "reference" (the default) its
    chemistry tendency is added to the scaled chemistry unconverted, as the reference does,
    with "scaled" converted by `scaled_forcing` first), fi = fimpl (TimeUnits x the chemistry
    source on component 5, zero on the fluid, :811-848), the Newton matrix I - gamma Jimpl
    (:850-908) from gbmv_chem_jac + gbmv_block_form_newton, factored and solved by the
    block-diagonal LU (SUNLinSol_BDMPIMV, :1075-1194), PostprocessStep after every step
    (:1002-1051), WRMS norms by gbmv_wrms_norm.  `precision` selects the fexpl form;
    `fused_newton` replaces fi / setup / solve in the stage iterations by the fused per-cell
    kernel's full Newton corrections."""

    def __init__(self, gbmv, hydro, chem, energy_units, time_units, rtol, atol, precision=0,
                 fused_newton=False, lu_precision=1, refine=4, forcing_units="reference",
                 linear_solver="direct"):
        import torch
        if forcing_units not in FORCING_UNITS:
            raise ValueError(f"forcing_units must be one of {FORCING_UNITS}")
        if linear_solver not in ("direct", "gmres"):
            raise ValueError("linear_solver must be 'direct' or 'gmres'")
        # "gmres": matrix-free Newton-Krylov -- each stage correction solves
        # (I - gamma J(z)) x = b per cell by batched GMRES whose Jacobian actions are
        # gbmv_chem_jvp at the current iterate (the temperature state of the fi call that
        # precedes every solve), no Jacobian formed or factored
        self.linear_solver = linear_solver
        self.krylov_iters = 0
        self.forcing_units = forcing_units
        self.g, self.hydro, self.chem = gbmv, hydro, chem
        # fused_newton: stage corrections from gbmv_chem_newton_stage (source, Jacobian and
        # factor per cell and per iterate, no Jacobian in HBM), by default with the FP32 factor
        # and up to four FP64-residual refinements; blocks whose refinement does not converge
        # take the FP64 factor inside the kernel (measured at 64^3: 99 steps, 1.59 s, against
        # 96 steps, 1.76 s with the FP64 factor throughout)
        self.fused_newton = fused_newton
        self.lu_precision, self.refine = lu_precision, refine
        self.eu, self.tu = energy_units, time_units
        self.rtol, self.atol = rtol, atol
        self.precision = precision
        n = chem.n
        self.J = torch.empty(100 * n, dtype=torch.float64, device="cuda")
        self.ls = gbmv.BlockLinearSolver(n)
        self.inv_scale = chem.state("inv_scale").view(-1, 10)

    def fe(self, t, y):
        import torch
        out = [torch.empty_like(x) for x in y]
        if self.g.fexpl(self.hydro, self.chem, t, y, out, self.eu, self.precision) != 0:
            raise RuntimeError("fexpl: illegal state")
        if self.forcing_units == "scaled":
            scaled_forcing(out[5].view(-1, 10), self.inv_scale, self.eu)
        return out

    def fi(self, t, y):
        import torch
        f = torch.empty_like(y[5])
        self.chem.calculate_rhs_cvklu(t, y[5].view(-1), f.view(-1), self.tu)
        self._z5 = y[5].reshape(-1)  # the iterate whose temperature state J v uses (GMRES)
        return [None] * 5 + [f]

    def setup(self, t, y, gamma):
        if self.linear_solver == "gmres":
            # two-sided diagonal scaling at the setup state: ten Jacobian actions along the
            # species unit vectors give the columns e_k - gamma J e_k of every block, which are
            # equilibrated (batched_equilibrate) and then dropped; the Krylov iterations apply
            # J only through gbmv_chem_jvp.  The blocks' columns and rows span many decades
            # (2-norm condition numbers up to 1e32 on the chem-hydro state, a few 1e9 once
            # equilibrated): row (Jacobi) scaling alone, or one row and column sweep, leaves
            # GMRES's residual norm blind to the small components.
            import torch
            self.gamma, self.t_lin = gamma, t
            y5 = y[5].reshape(-1)
            n = y5.numel() // 10
            e = torch.zeros_like(y5)
            jv = torch.empty_like(y5)
            A = torch.empty(n, 10, 10, dtype=y5.dtype, device=y5.device)
            for sp in range(10):
                e.zero_()
                e.view(n, 10)[:, sp] = 1.0
                self.chem.jvp(t, y5, e, jv, self.tu)
                A[:, :, sp] = e.view(n, 10) - gamma * jv.view(n, 10)
            self.precond, self.right = batched_equilibrate(A)
            return 0
        self.chem.calculate_jacobian_cvklu(t, y[5].view(-1), self.J, self.tu)
        self.g.form_newton_matrix(self.J, gamma)
        return self.ls.setup(self.J)

    def solve(self, b, z=None):
        import torch
        if self.linear_solver == "gmres":
            y = self._z5
            jv = torch.empty(y.numel(), dtype=torch.float64, device=y.device)

            def matvec(v):
                self.chem.jvp(self.t_lin, y, v.reshape(-1), jv, self.tu)
                return v - self.gamma * jv.view(-1, 10)
            x, it = batched_gmres(matvec, b[5].reshape(-1, 10), precond=self.precond,
                                  right=self.right, cycles=2)
            self.krylov_iters += it
            return list(b[:5]) + [x.view(b[5].shape)]
        x = torch.empty_like(b[5])
        self.ls.solve(self.J, x.view(-1), b[5].view(-1))
        return list(b[:5]) + [x]

    def correction(self, t, z, a, gamma):
        import torch
        b = a[5] - z[5]
        f, x = torch.empty_like(z[5]), torch.empty_like(z[5])
        if self.chem.newton_stage(t, z[5].view(-1), b.view(-1), f.view(-1), x.view(-1), gamma,
                                  self.tu, self.lu_precision, self.refine) != 0:
            return None
        return [ai - zi for ai, zi in zip(a[:5], z[:5])] + [x]

    def norm(self, v, y):
        return self.hydro.wrms_norm(v, y, self.rtol, self.atol)

    def postprocess(self, t, y):
        self.g.PostprocessStep(self.hydro, self.chem, y, self.eu)
