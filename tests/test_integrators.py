"""Host integrator layer (integrate.py) on the CPU: the Butcher tables' order conditions, the
ARK-IMEX driver's convergence order and error control on a manufactured split problem, its
recovery from a failed Newton-matrix setup, and the Dormand-Prince driver's error control.
numpy backends stand in for the device problem; the drivers are array-library agnostic."""
import math

import numpy as np
import pytest

import integrate as I


def _tables(etable=2, itable=104):
    t = I.ark_table(etable, itable)
    n = len(t["c"])
    AE = np.zeros((n, n))
    AI = np.zeros((n, n))
    for i in range(n):
        AE[i, :len(t["ae"][i])] = t["ae"][i]
        AI[i, :len(t["ai"][i])] = t["ai"][i]
    return AE, AI, np.array(t["b"]), np.array(t["bhat"]), np.array(t["c"])


def test_ark324_order_conditions():
    AE, AI, b, bh, c = _tables()
    tol = 1e-14
    for A in (AE, AI):
        assert np.allclose(A.sum(axis=1), c, atol=tol, rtol=0)  # row sums = abscissae
        assert abs(b.sum() - 1) < tol
        assert abs(b @ c - 1 / 2) < tol
        assert abs(b @ c ** 2 - 1 / 3) < tol
        assert abs(b @ (A @ c) - 1 / 6) < tol
    # the embedding is second order and not third
    assert abs(bh.sum() - 1) < tol and abs(bh @ c - 1 / 2) < tol
    assert abs(bh @ c ** 2 - 1 / 3) > 1e-3 or abs(bh @ (AE @ c) - 1 / 6) > 1e-3
    # explicit part strictly lower triangular; implicit part ESDIRK, stiffly accurate
    assert np.all(np.triu(AE) == 0)
    assert AI[0, 0] == 0 and np.allclose(np.diag(AI)[1:], AI[1, 1])
    assert np.array_equal(AI[-1], b)
    # L-stability of the implicit part: R(z) = det(I - zA + z 1 b^T) / det(I - zA) decays
    # like 1/z as z -> -inf
    e = np.ones(len(c))
    for z in (-1e4, -1e6):
        R = (np.linalg.det(np.eye(len(c)) - z * AI + z * np.outer(e, b)) /
             np.linalg.det(np.eye(len(c)) - z * AI))
        assert abs(R) < 5.0 / abs(z)


def test_ark_table_selection_rules():
    """ARKStepSetTableNum's rules: both numbers an IMEX pair, one of them a pure method,
    neither refused; mismatched pairs and wrong kinds refused."""
    t = I.ark_table(13, 112)
    assert t["explicit"] and t["implicit"] and t["q"] == 4 and t["p"] == 3
    assert not I.ark_table(-1, 112)["explicit"] and not I.ark_table(13, -1)["implicit"]
    for bad in ((-1, -1), (13, 104), (112, -1), (-1, 13)):
        with pytest.raises((ValueError, Exception)):
            I.ark_table(*bad)


class SplitProblem:
    """x' = y (explicit only), y' = -x (explicit) + lam (y - cos t) (implicit): exact
    x = sin t, y = cos t for x(0) = 0, y(0) = 1; the implicit part touches component 1 only."""

    def __init__(self, lam, rtol=1e-6, atol=1e-10, fail_setups=0):
        self.lam, self.rtol, self.atol = lam, rtol, atol
        self.fail_setups = fail_setups
        self.g = None
        self.post = 0

    def fe(self, t, y):
        return [y[1].copy(), -y[0]]

    def fi(self, t, y):
        return [None, self.lam * (y[1] - math.cos(t))]

    def setup(self, t, y, gamma):
        if self.fail_setups > 0:  # a singular block, recoverable
            self.fail_setups -= 1
            return 1
        self.g = gamma
        return 0

    def solve(self, b):
        return [b[0], b[1] / (1.0 - self.g * self.lam)]

    def norm(self, v, y):
        s = sum(float(((a / (self.rtol * np.abs(w) + self.atol)) ** 2).sum()) for a, w in zip(v, y))
        return math.sqrt(s / 2.0)

    def postprocess(self, t, y):
        self.post += 1


def _run(prob, T, **kw):
    y = [np.zeros(1), np.ones(1)]
    st = I.ark_imex_evolve(prob, 0.0, T, y, rtol=prob.rtol, atol=prob.atol, **kw)
    return y, st


@pytest.mark.parametrize("lam,order", [(-2.0, 2.85), (-1e4, 1.9)])
def test_imex_fixed_step_order(lam, order):
    """Third order on the nonstiff problem; in the stiff limit the classical reduction to the
    stage order (2) of the ESDIRK."""
    T = 2.0
    errs = []
    for h in (0.1, 0.05, 0.025, 0.0125):
        y, st = _run(SplitProblem(lam), T, fixed_h=h, maxcor=10, nlscoef=1e-3)
        errs.append(max(abs(y[0][0] - math.sin(T)), abs(y[1][0] - math.cos(T))))
        assert st.steps == round(T / h) and st.netf == 0
    orders = [math.log2(errs[i] / errs[i + 1]) for i in range(3)]
    assert min(orders[1:]) > order, (errs, orders)


def test_imex_adaptive_error_tracks_tolerance():
    T = 3.0
    errs, steps = [], []
    for rtol in (1e-4, 1e-6, 1e-8):
        p = SplitProblem(-1e4, rtol=rtol, atol=rtol * 1e-3)
        y, st = _run(p, T, max_steps=20000)
        errs.append(max(abs(y[0][0] - math.sin(T)), abs(y[1][0] - math.cos(T))))
        steps.append(st.steps)
        assert p.post == st.steps  # PostprocessStep after every accepted step
        assert st.nni >= 3 * st.steps and st.nsetups >= 1 and st.nfe == st.nfi - st.nni
    assert errs[0] > errs[1] > errs[2] and errs[2] < 1e-6
    assert steps[0] < steps[1] < steps[2]
    # the stiff implicit part does not limit the step: far fewer steps than |lam| T
    assert steps[1] < 1e4 * T / 50


class FusedSplitProblem(SplitProblem):
    """The same problem with full Newton corrections (the fused-kernel protocol)."""
    fused_newton = True

    def correction(self, t, z, a, gamma):
        r = [a[0] - z[0], (a[1] - z[1]) + gamma * self.lam * (z[1] - math.cos(t))]
        return [r[0], r[1] / (1.0 - gamma * self.lam)]


def test_imex_fused_newton_matches_modified():
    T = 2.0
    p1 = SplitProblem(-1e3, rtol=1e-8, atol=1e-11)
    p2 = FusedSplitProblem(-1e3, rtol=1e-8, atol=1e-11)
    y1, s1 = _run(p1, T)
    y2, s2 = _run(p2, T)
    for y in (y1, y2):
        assert abs(y[0][0] - math.sin(T)) < 1e-6 and abs(y[1][0] - math.cos(T)) < 1e-6
    assert abs(y1[1][0] - y2[1][0]) < 1e-7
    # a linear implicit part: the full Newton step is exact, so each stage converges at once
    assert s2.ncf == 0 and s2.nni <= s1.nni


def test_imex_recovers_from_failed_setup():
    _, base = _run(SplitProblem(-50.0), 1.0)
    p = SplitProblem(-50.0, fail_setups=2)
    y, st = _run(p, 1.0)
    assert st.ncf == base.ncf + 2 and st.nsetups >= base.nsetups + 2 and st.steps > 0
    assert abs(y[0][0] - math.sin(1.0)) < 1e-4 and abs(y[1][0] - math.cos(1.0)) < 1e-4


def test_imex_gives_up_on_persistent_failure():
    p = SplitProblem(-50.0, fail_setups=10 ** 6)
    with pytest.raises(RuntimeError, match="Newton failures"):
        _run(p, 1.0)


def test_erk_error_control():
    def rhs(t, y):
        return np.array([y[1], -y[0]])
    for rtol in (1e-6, 1e-9):
        y, st = I.erk_evolve(rhs, 0.0, 5.0, np.array([0.0, 1.0]), rtol, rtol * 1e-3)
        err = max(abs(y[0] - math.sin(5.0)), abs(y[1] - math.cos(5.0)))
        assert err < 100 * rtol and st.steps > 5


def test_scaled_forcing_units():
    torch = pytest.importorskip("torch")
    g = torch.arange(1.0, 21.0, dtype=torch.float64).view(2, 10)
    inv = torch.full((2, 10), 0.5, dtype=torch.float64)
    ref = g.clone()
    I.scaled_forcing(g, inv, 4.0)
    assert torch.equal(g[:, :9], ref[:, :9] * 0.5)
    assert torch.equal(g[:, 9], ref[:, 9] * 2.0)


def _mri_linear(table, h, T=1.0):
    """y' = Lf y + Ls y (non-commuting 2x2 parts), exact y = expm((Lf + Ls) t) y0; the fast
    problems v' = Lf v + r(tau) solved by fine RK4 substeps (far below the method error)."""
    import scipy.linalg as sl
    Lf = np.array([[-20.0, 5.0], [3.0, -12.0]])
    Ls = np.array([[-0.5, 1.0], [-1.0, -0.3]])
    y0 = np.array([1.0, 0.5])

    def slow(t, y):
        return [Ls @ y[0]]

    def fast(ta, tb, y, forcing, tshift, tscale):
        nsub = 200
        dt = (tb - ta) / nsub

        def f(t, v):
            tau = (t - tshift) / tscale
            r = sum((tau ** k) * fk[0] for k, fk in enumerate(forcing))
            return Lf @ v + r
        v, t = y[0].copy(), ta
        for _ in range(nsub):
            k1 = f(t, v)
            k2 = f(t + dt / 2, v + dt / 2 * k1)
            k3 = f(t + dt / 2, v + dt / 2 * k2)
            k4 = f(t + dt, v + dt * k3)
            v = v + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
            t += dt
        y[0][...] = v
        return 0
    y = [y0.copy()]
    I.mri_gark_evolve(slow, fast, 0.0, T, y, h, table)
    return np.max(np.abs(y[0] - sl.expm((Lf + Ls) * T) @ y0))


@pytest.mark.parametrize("table", [I.MRI_ERK22B, I.MRI_KW3, I.MRI_ERK33A],
                         ids=lambda t: t["name"])
def test_mri_gark_tables_order(table):
    """Each coupling table reaches its order on a linear multirate problem, and its rows are
    consistent (the constant-term rows sum to the stage length, higher powers to zero)."""
    c, G = table["c"], table["G"]
    for i in range(1, len(c)):
        assert abs(sum(G[0][i - 1]) - (c[i] - c[i - 1])) < 1e-15
        for Gk in G[1:]:
            assert abs(sum(Gk[i - 1])) < 1e-15
    errs = [_mri_linear(table, h) for h in (0.1, 0.05, 0.025)]
    orders = [math.log2(errs[k] / errs[k + 1]) for k in range(2)]
    assert min(orders) > table["order"] - 0.25, (errs, orders)


@pytest.mark.parametrize("table,order", [(3, 4), (13, 4), (8, 5), (6, 5), (1, 3)])
def test_erk_tables_fixed_step_order(table, order):
    """The explicit tables the inputs select (order 4 -> Zonneveld, etable 13, the
    Dormand-Prince and Cash-Karp pairs, Bogacki-Shampine) converge at their order."""
    def rhs(t, y):
        return np.array([y[1], -y[0] + 0.1 * math.sin(t) * y[0] ** 2])
    ref, _ = I.erk_evolve(rhs, 0.0, 2.0, np.array([0.2, 1.0]), table=8, fixed_h=1e-3)
    errs = []
    for h in (0.2, 0.1, 0.05):
        y, st = I.erk_evolve(rhs, 0.0, 2.0, np.array([0.2, 1.0]), table=table, fixed_h=h)
        errs.append(np.max(np.abs(y - ref)))
    orders = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(orders) > order - 0.4, (errs, orders)


@pytest.mark.parametrize("am", [0, 1, 2])
def test_erk_adaptivity_controllers(am):
    def rhs(t, y):
        return np.array([y[1], -y[0]])
    for rtol in (1e-6, 1e-9):
        y, st = I.erk_evolve(rhs, 0.0, 5.0, np.array([0.0, 1.0]), rtol, rtol * 1e-3, table=3,
                             adapt_method=am)
        err = max(abs(y[0] - math.sin(5.0)), abs(y[1] - math.cos(5.0)))
        assert err < 100 * rtol and st.steps > 5
    with pytest.raises(ValueError):
        I.erk_evolve(rhs, 0.0, 1.0, np.array([0.0, 1.0]), adapt_method=4)


def test_imex_ark437_fixed_step_order():
    """ARK4(3)7L[2]SA (etable 13, itable 112): fourth order on the nonstiff split problem."""
    T = 2.0
    errs = []
    for h in (0.2, 0.1, 0.05):
        y, st = _run(SplitProblem(-2.0), T, fixed_h=h, maxcor=10, nlscoef=1e-4,
                     table=I.ark_table(13, 112))
        errs.append(max(abs(y[0][0] - math.sin(T)), abs(y[1][0] - math.cos(T))))
    orders = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(orders) > 3.6, (errs, orders)


class StiffOnly:
    """y' = lam (y - cos t) - sin t (implicit part only): y = cos t."""

    def __init__(self, lam):
        self.lam, self.rtol, self.atol, self.g = lam, 1e-8, 1e-12, None

    def fe(self, t, y):
        raise AssertionError("an implicit-only table evaluates no explicit part")

    def fi(self, t, y):
        return [self.lam * (y[0] - math.cos(t)) - math.sin(t)]

    def setup(self, t, y, gamma):
        self.g = gamma
        return 0

    def solve(self, b):
        return [b[0] / (1.0 - self.g * self.lam)]

    def norm(self, v, y):
        return float(abs(v[0][0]) / (self.rtol * abs(y[0][0]) + self.atol))


def test_imex_implicit_only_and_explicit_only_tables():
    p = StiffOnly(-1e5)
    y = [np.ones(1)]
    st = I.ark_imex_evolve(p, 0.0, 1.0, y, rtol=p.rtol, atol=p.atol, maxcor=10,
                           table=I.ark_table(-1, 112))
    assert abs(y[0][0] - math.cos(1.0)) < 1e-7 and st.nfe == 0 and st.steps < 200
    y = [np.zeros(1), np.ones(1)]
    prob = SplitProblem(0.0)
    st = I.ark_imex_evolve(prob, 0.0, 2.0, y, rtol=1e-8, atol=1e-12,
                           table=I.ark_table(13, -1))
    assert abs(y[0][0] - math.sin(2.0)) < 1e-6 and st.nni == 0 and st.nsetups == 0
