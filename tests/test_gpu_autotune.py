"""The launch-shape autotuners (gbmv_hydro_autotune: the face sweeps' threads per block per
precision; gbmv_chem_newton_autotune: the fused Newton's resident blocks per SM; the DIRK's
block size is tuned inside gbmv_chem_dirk_evolve and tested with it): each picks one of its
candidates, and the results after tuning equal the untuned results bit for bit (one face or
cell per thread, independent of the launch shape)."""
import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu


def test_sweep_autotune_keeps_results(cuda):
    torch = cuda
    import gbmv
    wl = W.rayleigh_taylor(shape=(40, 36, 32), nchem=10, seed=W.SEED_BASE + 800)
    nz, ny, nx = wl["fields"][0].shape
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    for prec in (gbmv.FP64, gbmv.MIXED, gbmv.MIXED_FAST):
        h = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"], wl["force"])
        a = [torch.empty_like(x) for x in w]
        b = [torch.empty_like(x) for x in w]
        assert h.fEuler(0.0, w, a, prec) == 0
        t = h.autotune(w, prec)
        assert t in (32, 64, 128)
        assert h.fEuler(0.0, w, b, prec) == 0
        torch.cuda.synchronize()
        assert all(torch.equal(x, y) for x, y in zip(a, b)), prec


def test_sweep_budget_keeps_results(cuda):
    """The shared register budget (sweeps sized to run beside the Newton) computes the same
    tendencies bit for bit, every tracer count, every precision (FP64 and GBMV_MIXED ignore it)."""
    torch = cuda
    import gbmv
    for nchem in (0, 4, 10):
        wl = W.rayleigh_taylor(shape=(24, 20, 18), nchem=nchem, seed=W.SEED_BASE + 801 + nchem)
        nz, ny, nx = wl["fields"][0].shape
        w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
        h = gbmv.Hydro((nx, ny, nz), nchem, wl["bc"], wl["gamma"], wl["force"])
        for prec in (gbmv.FP64, gbmv.MIXED, gbmv.MIXED_FAST):
            a = [torch.empty_like(x) for x in w]
            b = [torch.empty_like(x) for x in w]
            h.set_sweep_budget(False)
            assert h.fEuler(0.0, w, a, prec) == 0
            h.set_sweep_budget(True)
            assert h.fEuler(0.0, w, b, prec) == 0
            torch.cuda.synchronize()
            assert all(torch.equal(x, y) for x, y in zip(a, b)), (nchem, prec)
            for threads in (32, 64):  # the caller-set launch shape, likewise
                h.set_sweep_threads(prec, threads)
                assert h.fEuler(0.0, w, b, prec) == 0
                torch.cuda.synchronize()
                assert all(torch.equal(x, y) for x, y in zip(a, b)), (nchem, prec, threads)
            h.set_sweep_threads(prec, 0)
    assert gbmv.load().gbmv_hydro_set_sweep_budget(h.h, 2) == -101  # GBMV_EINVAL
    assert gbmv.load().gbmv_hydro_set_sweep_threads(h.h, gbmv.MIXED_FAST, 96) == -101


def test_newton_autotune_keeps_results_and_state(cuda, tables):
    torch = cuda
    import gbmv
    n = 20000
    y, _ = W.primordial(n, seed=W.SEED_BASE + 801)
    c = gbmv.Chem(n, tables)
    c.set_scale(torch.from_numpy(y.reshape(-1).copy()).cuda())
    z = torch.ones(10 * n, dtype=torch.float64, device="cuda")
    f1, x1 = torch.empty_like(z), torch.empty_like(z)
    f2, x2 = torch.empty_like(z), torch.empty_like(z)
    ts0 = c.state("Ts").clone()
    bps = c.newton_autotune(z, 1e-4, 1e11, gbmv.MIXED, 2)
    assert bps in (0, 2, 3, 4, 5, 6, 8)
    assert torch.equal(c.state("Ts"), ts0)  # the temperature state restored
    assert c.newton_iteration(0.0, z, f1, x1, 1e-4, 1e11, lu_precision=gbmv.MIXED) == 0
    c.state("Ts").copy_(ts0)
    c.set_newton_occupancy(0)
    assert c.newton_iteration(0.0, z, f2, x2, 1e-4, 1e11, lu_precision=gbmv.MIXED) == 0
    torch.cuda.synchronize()
    assert torch.equal(f1, f2) and torch.equal(x1, x2)


@pytest.mark.parametrize("lu", ["fp64", "mixed"])
def test_newton_queue_launches_share_one_pass(cuda, tables, lu):
    """gbmv_chem_newton_queue_async: a narrow launch on a second stream and a full-width one on
    the first, sharing one chunk counter, compute every cell exactly as one plain launch does
    (f, x and the carried temperature), on a cell count that leaves a partial last chunk."""
    torch = cuda
    import gbmv
    n = 20000 + 13
    prec = gbmv.MIXED if lu == "mixed" else gbmv.FP64
    y, _ = W.primordial(n, seed=W.SEED_BASE + 802)
    c = gbmv.Chem(n, tables)
    c.set_scale(torch.from_numpy(y.reshape(-1).copy()).cuda())
    z = torch.ones(10 * n, dtype=torch.float64, device="cuda")
    ts0 = c.state("Ts").clone()
    f1, x1 = torch.empty_like(z), torch.empty_like(z)
    assert c.newton_iteration(0.0, z, f1, x1, 1e-4, 1e11, lu_precision=prec) == 0
    ts1 = c.state("Ts").clone()
    c.state("Ts").copy_(ts0)
    f2, x2 = torch.full_like(z, np.nan), torch.full_like(z, np.nan)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    queue = torch.zeros(1, dtype=torch.int64, device="cuda")
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    gbmv.chem_newton_queue_async(c, 0.0, z, f2, x2, 1e-4, 1e11, info, queue, 2,
                                 lu_precision=prec, refine=2, stream=side)
    gbmv.chem_newton_queue_async(c, 0.0, z, f2, x2, 1e-4, 1e11, info, queue, 0,
                                 lu_precision=prec, refine=2)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    assert int(queue.item()) >= n
    assert torch.equal(f1, f2) and torch.equal(x1, x2)
    assert torch.equal(c.state("Ts"), ts1)
