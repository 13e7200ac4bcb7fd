"""Persistent batched DIRK chemistry integrator (gbmv_chem_dirk_evolve) on the GPU against the
oracle's restatement of the same algorithm (orc_chem_dirk_evolve), on the static-chemistry
inputs: uniform density 1e2 m_H, log-uniform mass fractions in [1e-10, 1], log-uniform
temperature in [10, 1e4] K (src/primordial_static.cpp:86-160), scaled variables z = y / y0.

Tolerances.  The GPU FP64 form runs the oracle's algorithm with the same operation order up to
libm-versus-CUDA rounding of log/exp/pow/cbrt, so most cells take the identical step sequence
and agree to ~1e-12; a cell whose accept/converge decision flips on such a rounding difference
follows another step sequence and agrees only to the integration tolerance.  The mixed form
(equilibrated FP32 LU, optionally refined against FP64 residuals; FP32 temperature iterations)
solves the same FP64 residual equations, so its error against a tight-tolerance reference
solution must match the FP64 form's.
"""
import numpy as np
import pytest

import oracle_py as O
import workloads as W

pytestmark = pytest.mark.gpu

TU = 1.0e11  # TimeUnits of the chemistry inputs (seconds per time unit)
OPTS = dict(rtol=1e-6, atol=1e-10, maxcor=10, nlscoef=0.01)  # Newton settings of the inputs


def _cells(n, seed):
    y, _ = W.primordial(n, seed=seed)
    return y.reshape(-1)


def _gpu_run(torch, tables, scale, tout, **opts):
    import gbmv
    n = scale.size // 10
    c = gbmv.Chem(n, tables)
    c.set_scale(torch.from_numpy(scale.copy()).cuda())
    z = torch.ones(10 * n, dtype=torch.float64, device="cuda")
    st = torch.zeros(8 * n, dtype=torch.int32, device="cuda")
    nf = c.dirk_evolve(0.0, tout, z, TU, stats=st, **opts)
    torch.cuda.synchronize()
    return z.cpu().numpy().reshape(n, 10), st.cpu().numpy().reshape(n, 8), nf, c


def _relerr(a, b, floor):
    return np.abs(a - b) / (np.abs(b) + floor)


@pytest.mark.parametrize("table,deduce", [(112, 0), (102, 0), (112, 1)])
def test_dirk_fp64_matches_oracle(cuda, tables, table, deduce):
    """Both ESDIRK tables (112 = ARK4(3)7L[2]SA, the inputs' itable; 102 = TR-BDF2), and the
    intermediate stage derivatives evaluated (ARKODE's default) or deduced."""
    n, tout = 256, 1e-3
    scale = _cells(n, W.SEED_BASE + 500)
    zg, sg, nfg, _ = _gpu_run(cuda, tables, scale, tout, precision=0, block=64, table=table,
                              deduce=deduce, **OPTS)
    oc = O.Chem(tables, scale)
    zo, so, nfo = oc.dirk_evolve(np.ones(10 * n), 0.0, tout, TU, table=table, deduce=deduce,
                                 **OPTS)
    zo = zo.reshape(n, 10)
    assert nfg == nfo == 0
    same = np.all(sg[:, :7] == so[:, :7], axis=1)
    err = _relerr(zg, zo, OPTS["atol"] / OPTS["rtol"]).max(axis=1)
    got = (same.mean(), np.median(err[same]), np.max(err[same]), np.max(err))
    assert same.mean() >= 0.7, got  # identical step/iteration/setup counts
    # identical decisions: rounding-level agreement (a few stiff cells amplify libm-versus-CUDA
    # rounding of the rates over hundreds of steps to ~1e-8).  Equal totals do not mean equal
    # per-stage iteration counts, and a deduced stage derivative carries its stage's Newton
    # error (up to nlscoef x the tolerance) into the next stage's base, so with deduce = 1 a
    # cell whose iterations split differently between its stages parts at that level (median
    # 1.1e-11, largest 4.3e-6 measured)
    assert np.median(err[same]) <= (3e-11 if deduce else 1e-11), got
    assert np.max(err[same]) <= (1e-5 if deduce else 1e-6), got
    assert np.max(err) <= 1e-3, got  # decision flips: within the integration error


def test_dirk_mixed_accuracy_matches_fp64(cuda, tables):
    """Both forms against a tight-tolerance oracle solution: same global error."""
    n, tout = 256, 1e-3
    scale = _cells(n, W.SEED_BASE + 501)
    z64, s64, nf64, _ = _gpu_run(cuda, tables, scale, tout, precision=0, block=64, **OPTS)
    zmx, smx, nfmx, _ = _gpu_run(cuda, tables, scale, tout, precision=1, block=64, **OPTS)
    assert nf64 == nfmx == 0
    oc = O.Chem(tables, scale)
    zt, _, nft = oc.dirk_evolve(np.ones(10 * n), 0.0, tout, TU, rtol=1e-10, atol=1e-14,
                                maxcor=10, nlscoef=0.01, max_steps=200000)
    assert nft == 0
    zt = zt.reshape(n, 10)
    floor = OPTS["atol"] / OPTS["rtol"]
    e64 = _relerr(z64, zt, floor)
    emx = _relerr(zmx, zt, floor)
    assert np.median(emx) <= 2.0 * np.median(e64) + 1e-9, (np.median(emx), np.median(e64))
    assert np.max(emx) <= 2.0 * np.max(e64) + 1e-6, (np.max(emx), np.max(e64))
    # both forms differ from each other by far less than their error against the truth
    assert np.median(_relerr(zmx, z64, floor)) <= 1e-6
    # the mixed form does not need more Newton iterations than FP64 on average (+10 %)
    assert smx[:, 1].mean() <= 1.1 * s64[:, 1].mean()
    # FP32 LU with one FP64-residual refinement per linear solve: same accuracy
    zrf, srf, nfrf, _ = _gpu_run(cuda, tables, scale, tout, precision=1, refine=1, block=64,
                                 **OPTS)
    assert nfrf == 0
    erf = _relerr(zrf, zt, floor)
    assert np.median(erf) <= 2.0 * np.median(e64) + 1e-9
    assert srf[:, 1].mean() <= 1.1 * s64[:, 1].mean()
    # intermediate stage derivatives deduced from the stage equations: same accuracy, fewer F
    zdd, sdd, nfdd, _ = _gpu_run(cuda, tables, scale, tout, precision=1, deduce=1, block=64,
                                 **OPTS)
    assert nfdd == 0
    edd = _relerr(zdd, zt, floor)
    assert np.median(edd) <= 2.0 * np.median(e64) + 1e-9, (np.median(edd), np.median(e64))
    assert np.max(edd) <= 2.0 * np.max(e64) + 1e-6, (np.max(edd), np.max(e64))
    assert sdd[:, 6].sum() < 0.9 * smx[:, 6].sum()
    assert sdd[:, 1].mean() <= 1.1 * s64[:, 1].mean()


def test_dirk_block_sizes_bitwise_equal_and_autotune(cuda, tables):
    """Per-cell work is independent of scheduling: every block size gives identical bits;
    the autotuner picks one of them and leaves the temperature state untouched."""
    import gbmv
    torch = cuda
    n, tout = 3000, 2e-4
    scale = _cells(n, W.SEED_BASE + 502)
    ref = None
    for b in (32, 64, 128):
        z, st, nf, _ = _gpu_run(torch, tables, scale, tout, precision=1, block=b, **OPTS)
        assert nf == 0
        if ref is None:
            ref = (z, st)
        else:
            assert np.array_equal(z, ref[0]) and np.array_equal(st, ref[1]), b
    z, st, nf, c = _gpu_run(torch, tables, scale, tout, precision=1, block=0, **OPTS)
    assert c.dirk_block(gbmv.MIXED) in (32, 64)
    assert c.dirk_block(gbmv.FP64) == 0
    assert np.array_equal(z, ref[0]) and np.array_equal(st, ref[1])


@pytest.mark.parametrize("precision", [0, 1])
def test_dirk_setup_batching_bitwise_equal(cuda, tables, precision):
    """Gathering a warp's Newton-matrix setups (setup_batch lanes wait, skipping their F
    evaluations, until they set up together) changes only the interleaving of the lanes'
    work: every cell's state, temperature and counters are identical for any setup_batch."""
    torch = cuda
    n, tout = 6000, 2e-4   # more cells than resident lanes at 32 threads per block
    scale = _cells(n, W.SEED_BASE + 505)
    ref = None
    for sb in (1, 6, 32):
        z, st, nf, c = _gpu_run(torch, tables, scale, tout, precision=precision, block=32,
                                setup_batch=sb, **OPTS)
        Ts = c.state("Ts").cpu().numpy()
        assert nf == 0
        if ref is None:
            ref = (z, st, Ts)
        else:
            assert np.array_equal(z, ref[0]) and np.array_equal(st, ref[1]), sb
            assert np.array_equal(Ts, ref[2]), sb


@pytest.mark.parametrize("precision", [0, 1])
def test_dirk_cost_order_bitwise_equal(cuda, tables, precision):
    """Taking the cells largest initial derivative first (order 1, the default) instead of by
    index changes only which lane integrates which cell when: every cell's state, temperature
    and counters are identical."""
    torch = cuda
    n, tout = 6000, 2e-4
    scale = _cells(n, W.SEED_BASE + 506)
    ref = None
    for order in (0, 1):
        z, st, nf, c = _gpu_run(torch, tables, scale, tout, precision=precision, block=64,
                                order=order, **OPTS)
        Ts = c.state("Ts").cpu().numpy()
        assert nf == 0
        if ref is None:
            ref = (z, st, Ts)
        else:
            assert np.array_equal(z, ref[0]) and np.array_equal(st, ref[1])
            assert np.array_equal(Ts, ref[2])


def test_dirk_every_cell_retired_once_and_histogram(cuda, tables):
    torch = cuda
    import gbmv
    n, tout = 20000, 1e-4   # more cells than resident lanes: cells are pulled repeatedly
    scale = _cells(n, W.SEED_BASE + 503)
    z, st, nf, c = _gpu_run(torch, tables, scale, tout, precision=1, block=64, **OPTS)
    assert nf == 0
    assert np.all(st[:, 0] >= 1) and np.all(st[:, 7] == 0)
    assert np.all(st[:, 1] >= 6 * st[:, 0])     # six implicit stages per accepted step
    assert np.all(st[:, 6] >= st[:, 1])         # an F evaluation per Newton iteration
    assert np.all(np.isfinite(z)) and not np.any(np.all(z == 1.0, axis=1))
    hist = np.bincount(st[:, 1])
    assert hist.sum() == n and len(hist) > 2    # uneven per-cell iteration counts
    # the temperature state was carried: every cell's Ts moved off the 1000 K start
    Ts = c.state("Ts").cpu().numpy()
    assert np.all(np.isfinite(Ts)) and np.all(Ts > 0)


def test_dirk_failure_counted_not_faulted(cuda, tables):
    """A cell that cannot finish within max_steps is reported as failed with its last
    accepted state, and the other cells are unaffected."""
    n, tout = 512, 1e-3
    scale = _cells(n, W.SEED_BASE + 504)
    zf, sf, nf, _ = _gpu_run(cuda, tables, scale, tout, precision=0, block=64, max_steps=3,
                             **OPTS)
    assert nf == int(sf[:, 7].sum()) and nf > 0
    assert np.all(sf[sf[:, 7] == 1, 0] == 3)
    assert np.all(np.isfinite(zf))


def test_dirk_options_rejected(cuda, tables):
    import gbmv
    torch = cuda
    c = gbmv.Chem(16, tables)
    z = torch.ones(160, dtype=torch.float64, device="cuda")
    for bad in (dict(rtol=0.0), dict(block=48), dict(refine=9), dict(precision=3),
                dict(maxcor=0), dict(table=13), dict(table=104 + 1000), dict(table=8),
                dict(setup_batch=0), dict(setup_batch=33), dict(order=2), dict(deduce=2)):
        with pytest.raises(gbmv.GbmvError):
            c.dirk_evolve(0.0, 1e-3, z, TU, **bad)
    with pytest.raises(gbmv.GbmvError):
        c.dirk_evolve(1.0, 0.5, z, TU)   # tout must exceed t0


@pytest.mark.parametrize("deduce", [0, 1])
def test_mri_fast_evolve_with_forcing(cuda, tables, deduce):
    """RankLocalStepper_Evolve counterpart: chemistry by the DIRK with the forcing's chemistry
    component in its right-hand side (against the oracle's forced integration), fluid
    components by the forcing polynomial's exact integral; intermediate stage derivatives
    evaluated or deduced (a deduced one includes the forcing through the stage equation)."""
    torch = cuda
    import gbmv
    wl = W.chem_hydro(shape=(8, 6, 5))
    nz, ny, nx = wl["fields"][0].shape
    n = nx * ny * nz
    h = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(n, tables)
    c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    rng = np.random.default_rng(11)
    fh = [[1e-2 * rng.standard_normal(f.shape) for f in wl["fields"]] for _ in range(2)]
    forcing = [[torch.from_numpy(a).cuda() for a in fv] for fv in fh]
    t0, tout, tshift, tscale = 0.2, 0.2 + 1e-4, 0.15, 1e-3
    st = torch.zeros(8 * n, dtype=torch.int32, device="cuda")
    nf = gbmv.mri_fast_evolve(h, c, t0, tout, w, TU, forcing, tshift, tscale, stats=st,
                              precision=0, block=64, deduce=deduce, **OPTS)
    torch.cuda.synchronize()
    assert nf == 0
    tau0, tau1 = (t0 - tshift) / tscale, (tout - tshift) / tscale
    for k in range(5):
        ref = wl["fields"][k] + sum(fh[i][k] * tscale * (tau1 ** (i + 1) - tau0 ** (i + 1)) / (i + 1)
                                    for i in range(2))
        assert np.max(np.abs(w[k].cpu().numpy() - ref)) <= 1e-14 * max(1.0, np.max(np.abs(ref)))
    oc = O.Chem(tables, wl["scale"].reshape(-1))
    zo, so, nfo = oc.dirk_evolve(wl["fields"][5].reshape(-1), t0, tout, TU,
                                 forcing=[fv[5] for fv in fh], tshift=tshift, tscale=tscale,
                                 deduce=deduce, **OPTS)
    assert nfo == 0
    zg = w[5].cpu().numpy().reshape(n, 10)
    zo = zo.reshape(n, 10)
    sg = st.cpu().numpy().reshape(n, 8)
    same = np.all(sg[:, :7] == so[:, :7], axis=1)
    assert same.mean() >= 0.75
    err = _relerr(zg, zo, OPTS["atol"] / OPTS["rtol"]).max(axis=1)
    assert np.median(err[same]) <= (3e-11 if deduce else 1e-11) and np.max(err) <= 1e-3
    # the forcing changed the chemistry: an unforced run lands elsewhere
    oc2 = O.Chem(tables, wl["scale"].reshape(-1))
    zu, _, _ = oc2.dirk_evolve(wl["fields"][5].reshape(-1), t0, tout, TU, **OPTS)
    assert np.max(np.abs(zu.reshape(n, 10) - zo)) > 1e-8


def test_mixed_dirk_second_pass_mechanism(cuda, tables):
    """The FP32-LU DIRK sends the cells it cannot finish to a second pass with the FP64 factor,
    from their start state.  With the per-step error-test failure limit at 1 (maxnef), every
    cell whose first try of some step is rejected fails its FP32 pass: those cells are listed
    (gbmv_chem_dirk_retried), integrated again, and the failures counted are those of the
    second pass, which fails them (nearly always) where the FP64 form does; the other cells
    keep their FP32-pass result."""
    torch = cuda
    n, tout = 4096, 1e-3
    y, _ = W.primordial(n, seed=W.SEED_BASE + 2)
    scale = y.reshape(-1)
    strict = dict(OPTS, maxnef=1)
    zm, sm, nfm, cm = _gpu_run(torch, tables, scale, tout, precision=1, block=64, **strict)
    retried = cm.dirk_retried()
    z64, s64, nf64, _ = _gpu_run(torch, tables, scale, tout, precision=0, block=64, **strict)
    assert len(retried) >= 1 and len(retried) < n
    assert nfm == int(sm[retried, 7].sum())  # failures counted are those of the second pass
    # the second pass fails where the FP64 form fails, but for the few cells whose first-try
    # rejection its (mixed) temperature solve moves across the threshold
    assert np.mean(sm[retried, 7] == s64[retried, 7]) >= 0.95
    kept = np.setdiff1d(np.arange(n), retried)
    assert np.all(sm[kept, 7] == 0) and np.all(np.isfinite(zm))


def test_mixed_dirk_second_pass_accuracy(cuda, tables):
    """On the 64^3 static-chemistry inputs a few cells' Newton iterations keep failing on their
    FP32 factor: the second pass (FP64 factor, the mixed temperature solve) finishes them, and
    they end within the integration tolerance of the FP64 form."""
    torch = cuda
    n, tout = 64 ** 3, 1e-3
    y, _ = W.primordial(n, seed=W.SEED_BASE + 2)
    scale = y.reshape(-1)
    zm, sm, nfm, cm = _gpu_run(torch, tables, scale, tout, precision=1, block=64, **OPTS)
    retried = cm.dirk_retried()
    if len(retried) == 0:
        pytest.skip("no cell of these inputs needed the second pass")
    z64, s64, nf64, _ = _gpu_run(torch, tables, scale, tout, precision=0, block=64, **OPTS)
    assert nfm == 0 and nf64 == 0
    assert np.all(sm[retried, 7] == 0)
    floor = OPTS["atol"] / OPTS["rtol"]
    err = np.abs(zm[retried] - z64[retried]) / (np.abs(z64[retried]) + floor)
    assert err.max() <= 1e-3, err.max()