"""Whole-grid parity of the headline stage and of the Rayleigh-Taylor RHS against the oracle.

The other GPU tests pin every kernel on small grids; these run the benchmark's own
compositions on grids large enough for every launch to wrap its grid-stride loops many times
and for the per-direction face scratch to span many blocks, and compare every output with the
oracle evaluated on all host cores (z-slabs / cell ranges on threads):

* the fused chemistry-hydrodynamics stage (fexpl WENO RHS of all 15 fields + glue, chemistry
  source, Jacobian, I - gamma J factor and solve), FP64 form through the separate drop-in
  entries, two stages in a row (the temperature state carried from the first into the second);
* the same stage in the mixed forms, captured once as a CUDA graph and replayed twice;
* the Rayleigh-Taylor WENO RHS in the FP64 and both mixed forms.

Tolerances (per field, max|gpu - oracle| / max|oracle|; chemistry per species): FP64 forms
1e-12 for the tendencies and the chemistry source, 1e-10 for the Newton update (a 10x10
solve with partial pivoting: the GPU's elimination rounds differently from the oracle's and
the blocks' condition numbers reach ~1e4); mixed forms 1e-6, the metric's bar.
"""
import numpy as np
import pytest

import oracle_py as O
import workloads as W
from conftest import TABLES, maxnorm_err

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12
TOL_X_FP64 = 1e-10
TOL_MIXED = 1e-6
NEWTON_GAMMA = 1e-4
N = 48
NAMES = ["rho", "mx", "my", "mz", "et", "chem", "fimpl", "newton_x"]


def _errs(outs, refs):
    e = {}
    for nm, a, b in zip(NAMES, outs, refs):
        if nm in ("chem", "fimpl", "newton_x"):
            a2, b2 = np.asarray(a).reshape(-1, 10), np.asarray(b).reshape(-1, 10)
            e[nm] = max(maxnorm_err(a2[:, s], b2[:, s]) for s in range(10))
        else:
            e[nm] = maxnorm_err(a, b)
    return e


class _Stage:
    def __init__(self, torch, wl, precision):
        import gbmv
        import h5tables
        self.torch, self.g, self.wl, self.precision = torch, gbmv, wl, precision
        n = wl["fields"][0].shape[0]
        self.ncell = n ** 3
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        self.w = [dev(f) for f in wl["fields"]]
        self.wdot = [torch.empty_like(f) for f in self.w]
        self.f = torch.empty(10 * self.ncell, dtype=torch.float64, device="cuda")
        self.x = torch.empty_like(self.f)
        self.hydro = gbmv.Hydro((n, n, n), 10, wl["bc"], wl["gamma"])
        self.chem = gbmv.Chem(self.ncell, h5tables.load_table_block(TABLES))
        self.chem.set_scale(dev(wl["scale"].reshape(-1)))
        self.EU, self.TU = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
        self.status = torch.zeros(2, dtype=torch.int32, device="cuda")

    def fp64_step(self):
        g = self.g
        assert g.fexpl(self.hydro, self.chem, 0.0, self.w, self.wdot, self.EU, g.FP64) == 0
        y = self.w[5].view(-1)
        J = self.torch.empty(100 * self.ncell, dtype=self.torch.float64, device="cuda")
        self.chem.calculate_rhs_cvklu(0.0, y, self.f, self.TU)
        self.chem.calculate_jacobian_cvklu(0.0, y, J, self.TU)
        g.form_newton_matrix(J, NEWTON_GAMMA)
        ls = g.BlockLinearSolver(self.ncell)
        assert ls.setup(J) == 0
        ls.solve(J, self.x, self.f)

    def capture_mixed(self):
        g, torch = self.g, self.torch

        def stage():
            self.status.zero_()
            g.fexpl_async(self.hydro, self.chem, 0.0, self.w, self.wdot, self.EU,
                          self.status[0:1], self.precision)
            g.chem_newton_async(self.chem, 0.0, self.w[5].view(-1), self.f, self.x,
                                NEWTON_GAMMA, self.TU, self.status[1:2], lu_precision=g.MIXED,
                                refine=2)
        # first calls outside the capture (they allocate the handle's float-float buffers)
        stage()
        torch.cuda.synchronize()
        self.chem.state("Ts").fill_(1000.0)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=side):
            stage()
        torch.cuda.synchronize()
        for d, h in zip(self.w, self.wl["fields"]):  # back to the initial state
            d.copy_(torch.from_numpy(np.ascontiguousarray(h)))
        self.chem.state("Ts").fill_(1000.0)
        torch.cuda.synchronize()
        return graph

    def outputs(self):
        self.torch.cuda.synchronize()
        assert self.status.cpu().tolist() == [0, 0]
        return [t.cpu().numpy() for t in self.wdot] + [self.f.cpu().numpy(),
                                                       self.x.cpu().numpy()]


def _oracle_steps(wl, tables, nsteps):
    fields = [np.array(f, copy=True) for f in wl["fields"]]
    oc = O.Chem(tables, wl["scale"].reshape(-1))
    outs = []
    for _ in range(nsteps):
        st, out = O.fused_chem_hydro_step(fields, wl["scale"], oc, wl["bc"], wl["gamma"],
                                          wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"],
                                          NEWTON_GAMMA, threads=0)
        assert st == 0
        outs.append(out)
    return outs


@pytest.fixture(scope="module")
def chem_hydro_case(tables):
    wl = W.chem_hydro(n=N)
    return wl, _oracle_steps(wl, tables, 2)


def test_fused_stage_fp64_matches_oracle_two_stages(cuda, chem_hydro_case):
    torch = cuda
    import gbmv
    wl, refs = chem_hydro_case
    s = _Stage(torch, wl, gbmv.FP64)
    for k in range(2):  # the second stage starts from the temperature the first one left
        s.fp64_step()
        e = _errs(s.outputs(), refs[k])
        for nm, v in e.items():
            assert v <= (TOL_X_FP64 if nm == "newton_x" else TOL_FP64), (k, nm, v)


@pytest.mark.parametrize("form", ["mixed", "mixed_fast"])
def test_fused_stage_mixed_graph_matches_oracle(cuda, chem_hydro_case, form):
    torch = cuda
    import gbmv
    wl, refs = chem_hydro_case
    s = _Stage(torch, wl, {"mixed": gbmv.MIXED, "mixed_fast": gbmv.MIXED_FAST}[form])
    graph = s.capture_mixed()
    for k in range(2):  # replays carry the temperature state like the eager stages
        graph.replay()
        e = _errs(s.outputs(), refs[k])
        assert max(e.values()) <= TOL_MIXED, (form, k, e)


def test_rayleigh_taylor_rhs_all_forms_match_oracle(cuda):
    torch = cuda
    import gbmv
    n = 64
    wl = W.rayleigh_taylor(n=n, nchem=10)
    st, ref = O.feuler(wl["fields"], 10, wl["bc"], wl["gamma"], wl["force"], threads=0)
    assert st == 0
    h = gbmv.Hydro((n, n, n), 10, wl["bc"], wl["gamma"], wl["force"])
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    for prec, tol in ((gbmv.FP64, TOL_FP64), (gbmv.MIXED, TOL_MIXED),
                      (gbmv.MIXED_FAST, TOL_MIXED)):
        wdot = [torch.full_like(f, np.nan) for f in w]
        assert h.fEuler(0.0, w, wdot, prec) == 0
        torch.cuda.synchronize()
        for i, (a, b) in enumerate(zip(wdot, ref)):
            e = maxnorm_err(a.cpu().numpy(), b)
            assert e <= tol, (prec, i, e)
