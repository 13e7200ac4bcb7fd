"""Checkpoint / restart of a chemistry-hydrodynamics run in the reference's formats: an ARK-IMEX
run stopped at t1 is written as output-%07i.hdf5 (from the device state) with its
restart_parameters.txt, read back into fresh handles as read_restart does (fluid fields
through the CGS units and back, the next step size from the parameter file, the temperature
history re-initialised as a restarted reference run re-initialises it) and continued to t2;
the result matches the run that continued in place to well inside the integration
tolerance."""
import numpy as np
import pytest

import h5io
import workloads as W
from conftest import maxnorm_err

pytestmark = pytest.mark.gpu
# the primordial inputs' controller (adapt_method 2, no error history, so the continued and the
# restarted run take the same steps) and method pair
OPTS = dict(rtol=1e-6, atol=1e-10, maxcor=10, nlscoef=0.01, safety=0.99, bias=2.0, growth=2.0,
            adapt_method=2)
DOMAIN = (0.0, 1.0, 0.0, 1.0, 0.0, 1.0)


def _problem(torch, wl, tables, fields):
    import gbmv
    import integrate
    nz, ny, nx = wl["fields"][0].shape
    hy = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(nx * ny * nz, tables)
    c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in fields]
    u = wl["units"]
    prob = integrate.ChemHydroImex(gbmv, hy, c, u["EnergyUnits"], u["TimeUnits"],
                                   OPTS["rtol"], OPTS["atol"], 0)
    return prob, w


def test_restart_continues_the_run(cuda, tables, tmp_path):
    torch = cuda
    import integrate
    wl = W.chem_hydro(shape=(12, 10, 8))
    u = wl["units"]
    field_units = h5io.units(u["MassUnits"], u["LengthUnits"], u["TimeUnits"])
    t1, t2 = 2e-6, 4e-6
    # the run to t1, then continued in place
    prob, w = _problem(torch, wl, tables, wl["fields"])
    st1 = integrate.ark_imex_evolve(prob, 0.0, t1, w, **OPTS)
    assert st1.steps > 3 and st1.h_next > 0.0
    path = h5io.write_solution(str(tmp_path), 1, t1, w, DOMAIN, field_units)
    params = {k: (0 if kind == "i" else 0.0) for k, kind in h5io.PARAMETERS}
    nz, ny, nx = wl["fields"][0].shape
    params.update(nx=nx, ny=ny, nz=nz, nout=2, tf=t2, rtol=OPTS["rtol"], atol=OPTS["atol"],
                  MassUnits=u["MassUnits"], LengthUnits=u["LengthUnits"],
                  TimeUnits=u["TimeUnits"], gamma=wl["gamma"], xr=1.0, yr=1.0, zr=1.0)
    h5io.write_parameters(str(tmp_path), params, tcur=t1, hcur=st1.h_next, iout=1)
    integrate.ark_imex_evolve(prob, t1, t2, w, h0=st1.h_next, **OPTS)
    cont = [x.cpu().numpy() for x in w]
    # the restarted run: state and step size from the files, fresh handles
    p = h5io.read_parameters(str(tmp_path / "restart_parameters.txt"))
    assert p["restart"] == 1 and p["t0"] == t1 and p["nout"] == 1
    t, fields = h5io.read_restart(str(tmp_path), p["restart"], 10, DOMAIN,
                                  wl["fields"][0].shape, field_units)
    assert t == t1 and path.endswith("output-0000001.hdf5")
    prob2, w2 = _problem(torch, wl, tables, fields)
    integrate.ark_imex_evolve(prob2, t, t2, w2, h0=p["h0"], **OPTS)
    rest = [x.cpu().numpy() for x in w2]
    for k in range(5):
        assert maxnorm_err(rest[k], cont[k]) <= 1e-9, k
    n = rest[5].size // 10
    for s in range(10):
        assert maxnorm_err(rest[5].reshape(n, 10)[:, s], cont[5].reshape(n, 10)[:, s]) <= 1e-7, s
