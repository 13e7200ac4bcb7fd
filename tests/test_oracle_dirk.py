"""The oracle's per-cell DIRK integrator (orc_chem_dirk_evolve, CPU): convergence of the
ESDIRK tables (ARK4(3)7L[2]SA, the reference inputs' itable 112, and TR-BDF2, itable 102) and
its bookkeeping, on the static-chemistry inputs."""
import numpy as np
import pytest

import oracle_py as O
import workloads as W

TU = 1.0e11


def _run(tables, scale, tout, **kw):
    oc = O.Chem(tables, scale)
    n = scale.size // 10
    z, st, nf = oc.dirk_evolve(np.ones(10 * n), 0.0, tout, TU, **kw)
    return z.reshape(n, 10), st, nf, oc


@pytest.mark.parametrize("table", [112, 102])
def test_dirk_global_error_shrinks_with_tolerance(tables, table):
    y, _ = W.primordial(24, seed=W.SEED_BASE + 510)
    scale = y.reshape(-1)
    zt, _, nf, _ = _run(tables, scale, 2e-4, rtol=1e-11, atol=1e-15, maxcor=10, nlscoef=0.01,
                        max_steps=500000, table=table)
    assert nf == 0
    errs = []
    for rtol in (1e-5, 1e-7):
        z, st, nf, _ = _run(tables, scale, 2e-4, rtol=rtol, atol=rtol * 1e-4, maxcor=10,
                            nlscoef=0.01, table=table)
        assert nf == 0
        errs.append(np.median(np.abs(z - zt) / (np.abs(zt) + 1e-4)))
    # ~100x tighter tolerance gives a clearly smaller global error
    assert errs[1] < errs[0] / 5.0, errs
    assert errs[0] < 1e-3, errs


@pytest.mark.parametrize("table,stages", [(112, 7), (102, 3)])
def test_dirk_stats_bookkeeping(tables, table, stages):
    y, _ = W.primordial(16, seed=W.SEED_BASE + 511)
    z, st, nf, oc = _run(tables, y.reshape(-1), 1e-4, maxcor=10, nlscoef=0.01, table=table)
    assert nf == 0 and np.all(st[:, 7] == 0)
    steps, nni, netf, ncf, nsetup, nje, nfe = (st[:, k] for k in range(7))
    assert np.all(nni >= (stages - 1) * steps)
    # F evaluations: the first-stage derivative, one per Newton iteration and one per
    # converged implicit stage (stages - 1 per attempted step)
    assert np.all(nfe >= 1 + nni + (stages - 1) * steps)
    assert np.all(nje >= 1) and np.all(nsetup >= nje)
    assert np.all(np.isfinite(z)) and np.all(np.isfinite(oc.Ts))


def test_dirk_max_steps_reports_failure(tables):
    y, _ = W.primordial(8, seed=W.SEED_BASE + 512)
    z, st, nf, _ = _run(tables, y.reshape(-1), 1e-3, max_steps=2)
    assert nf == int(st[:, 7].sum()) and nf > 0
    assert np.all(st[st[:, 7] == 1, 0] == 2)


@pytest.mark.parametrize("table", [112, 102])
def test_dirk_deduced_stage_derivatives(tables, table):
    """deduce = 1: the intermediate stages' derivatives come from the stage equations, so the
    only F evaluations besides Newton's are the first stage's and one per attempt that reaches
    the last stage; the global error against a tight-tolerance solution stays that of the
    evaluated form."""
    y, _ = W.primordial(24, seed=W.SEED_BASE + 513)
    scale = y.reshape(-1)
    opts = dict(rtol=1e-6, atol=1e-10, maxcor=10, nlscoef=0.01, table=table)
    zt, _, nf, _ = _run(tables, scale, 2e-4, rtol=1e-11, atol=1e-15, maxcor=10, nlscoef=0.01,
                        max_steps=500000, table=table)
    assert nf == 0
    z0, s0, nf0, _ = _run(tables, scale, 2e-4, **opts)
    z1, s1, nf1, _ = _run(tables, scale, 2e-4, deduce=1, **opts)
    assert nf0 == nf1 == 0
    steps, nni, netf, ncf, nfe = s1[:, 0], s1[:, 1], s1[:, 2], s1[:, 3], s1[:, 6]
    assert np.all(nfe == 1 + nni + steps + netf)
    assert s1[:, 6].sum() < 0.9 * s0[:, 6].sum()      # ~16 % fewer F evaluations
    assert s1[:, 1].sum() <= 1.03 * s0[:, 1].sum()    # Newton iterations about unchanged
    # per-cell error (largest over the species) against the tight solution
    e0 = (np.abs(z0 - zt) / (np.abs(zt) + 1e-4)).max(axis=1)
    e1 = (np.abs(z1 - zt) / (np.abs(zt) + 1e-4)).max(axis=1)
    assert np.median(e1) <= 1.25 * np.median(e0), (np.median(e1), np.median(e0))
    assert np.max(e1) <= 1.25 * np.max(e0), (np.max(e1), np.max(e0))
