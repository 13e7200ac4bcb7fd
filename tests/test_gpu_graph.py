"""The mixed-precision chemistry-hydrodynamics stage captured in a CUDA graph: replay must
reproduce the eager launches bit for bit (the asynchronous entry points report the legal-state
mask and singular blocks through device words instead of host syncs)."""
import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu


def _make(torch, gbmv, wl, tables):
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(nx * ny * nz, tables)
    c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    wdot = [torch.empty_like(f) for f in w]
    n = nx * ny * nz
    f = torch.empty(10 * n, dtype=torch.float64, device="cuda")
    x = torch.empty_like(f)
    return h, c, w, wdot, f, x


def test_stage_graph_replay_matches_eager(cuda, tables):
    torch = cuda
    import gbmv
    wl = W.chem_hydro(shape=(24, 20, 16))
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    A = _make(torch, gbmv, wl, tables)
    B = _make(torch, gbmv, wl, tables)
    status = torch.zeros(2, dtype=torch.int32, device="cuda")

    def stage(h, c, w, wdot, f, x):
        status.zero_()
        gbmv.fexpl_async(h, c, 0.0, w, wdot, eu, status[0:1], gbmv.MIXED)
        gbmv.chem_newton_async(c, 0.0, w[5].view(-1), f, x, 1e-4, tu, status[1:2],
                               lu_precision=gbmv.MIXED, refine=4)

    for _ in range(3):  # eager
        stage(*A)
    stage(*B)  # first mixed call on a handle allocates its buffers: outside the capture
    torch.cuda.synchronize()
    assert int(status.sum()) == 0
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        stage(*B)
    # capture records without executing: two replays reproduce eager stages 2 and 3
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert int(status.sum()) == 0
    for a, b in zip(A[2] + A[3] + [A[4], A[5]], B[2] + B[3] + [B[4], B[5]]):
        assert torch.equal(a, b)
    assert torch.equal(A[1].state("Ts"), B[1].state("Ts"))


@pytest.mark.parametrize("form,bps", [("MIXED", 2), ("MIXED_FAST", 4)])
def test_concurrent_branch_graph_matches_serial_eager(cuda, tables, form, bps):
    """The stage as two graph branches -- chemistry Newton on its own stream with a persistent
    grid of `bps` blocks per SM, WENO sweep on the capture stream -- gives the serial eager
    bits: the mixed fexpl never writes w[5], so the branches share no written data."""
    torch = cuda
    import gbmv
    prec = getattr(gbmv, form)
    wl = W.chem_hydro(shape=(24, 20, 16))
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    A = _make(torch, gbmv, wl, tables)
    B = _make(torch, gbmv, wl, tables)
    B[1].set_newton_occupancy(bps)
    status = torch.zeros(2, dtype=torch.int32, device="cuda")
    chem_stream = torch.cuda.Stream()

    def serial(h, c, w, wdot, f, x):
        status.zero_()
        gbmv.fexpl_async(h, c, 0.0, w, wdot, eu, status[0:1], prec)
        gbmv.chem_newton_async(c, 0.0, w[5].view(-1), f, x, 1e-4, tu, status[1:2],
                               lu_precision=gbmv.MIXED, refine=4)

    def branches(h, c, w, wdot, f, x):
        status.zero_()
        main = torch.cuda.current_stream()
        fork = torch.cuda.Event()
        fork.record(main)
        chem_stream.wait_event(fork)
        gbmv.chem_newton_async(c, 0.0, w[5].view(-1), f, x, 1e-4, tu, status[1:2],
                               lu_precision=gbmv.MIXED, refine=4, stream=chem_stream)
        gbmv.fexpl_async(h, c, 0.0, w, wdot, eu, status[0:1], prec)
        join = torch.cuda.Event()
        join.record(chem_stream)
        main.wait_event(join)

    for _ in range(3):
        serial(*A)
    serial(*B)  # allocations outside the capture
    torch.cuda.synchronize()
    w5 = B[2][5].clone()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        branches(*B)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert int(status.sum()) == 0
    assert torch.equal(B[2][5], w5)  # the chemistry component was never rewritten
    for a, b in zip(A[2] + A[3] + [A[4], A[5]], B[2] + B[3] + [B[4], B[5]]):
        assert torch.equal(a, b)
    assert torch.equal(A[1].state("Ts"), B[1].state("Ts"))
