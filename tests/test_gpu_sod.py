"""Whole run of the Sod configuration (128x3x3, reflecting x, periodic y/z, gamma 1.4) to
t_f = 0.2 with an adaptive ERK at rtol 1e-6, atol 1e-11: the GPU flux divergence against the
same integration driven by the oracle (the reference's fEuler restated), and both against the
exact Riemann solution."""
import numpy as np
import pytest

import integrate as I
import oracle_py as O
import workloads as W

pytestmark = pytest.mark.gpu


def test_sod_whole_run(cuda):
    torch = cuda
    import gbmv
    nx = 128
    wl = W.sod(nx, 3, 3)
    shape = wl["fields"][0].shape
    n = int(np.prod(shape))

    def rhs_cpu(t, y):
        st, out = O.feuler([y[i].reshape(shape) for i in range(5)], 0, wl["bc"], wl["gamma"], None)
        assert st == 0
        return np.stack([o.reshape(-1) for o in out])

    h = gbmv.Hydro((nx, 3, 3), 0, wl["bc"], wl["gamma"])
    wdot = torch.empty((5, n), dtype=torch.float64, device="cuda")

    def rhs_gpu(t, y):
        w = [y[i].view(shape) for i in range(5)]
        d = [wdot[i].view(shape) for i in range(5)]
        assert h.fEuler(t, w, d) == 0
        return wdot.clone()

    y0 = np.stack([f.reshape(-1) for f in wl["fields"]])
    yc, stc = I.erk_evolve(rhs_cpu, 0.0, 0.2, y0, 1e-6, 1e-11)
    yg, stg = I.erk_evolve(rhs_gpu, 0.0, 0.2, torch.from_numpy(y0).cuda(), 1e-6, 1e-11)
    yg = yg.cpu().numpy()
    # same RHS to 1e-12 -> same step sequence -> same solution far inside the tolerance
    for v in range(5):
        scale = max(np.max(np.abs(yc[v])), 1e-300)
        assert np.max(np.abs(yg[v] - yc[v])) / scale <= 1e-8, v
    x = (np.arange(nx) + 0.5) / nx
    r, u, p = I.sod_exact(x, 0.2)
    for y in (yc, yg):
        rho = y[0].reshape(shape)[1, 1]
        mx = y[1].reshape(shape)[1, 1]
        assert np.mean(np.abs(rho - r)) < 7e-3      # WENO5 at 128 cells, shock-smeared (5.3e-3)
        assert np.mean(np.abs(mx / rho - u)) < 2e-2
        # the solution is uniform across the periodic y/z directions
        assert np.allclose(y[0].reshape(shape), y[0].reshape(shape)[:1, :1], rtol=0, atol=1e-12)
