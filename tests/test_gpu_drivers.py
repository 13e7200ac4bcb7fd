"""The input-file drivers on the GPU: the ERK hydrodynamics driver on the Sod configuration
(against the exact Riemann solution; conservation totals; a run restarted from its
output-0000002.hdf5 and restart_parameters.txt reproduces the uninterrupted run bit for bit,
since the state and the step size round-trip exactly), and the ARK-IMEX and multirate
chemistry drivers on a small chemistry-hydrodynamics grid (outputs, restart continuation
within the integration tolerance, the multirate run equal to one mri_evolve call)."""
import os

import numpy as np
import pytest

import drivers as D
import h5io
import integrate as I
import workloads as W

pytestmark = pytest.mark.gpu

# order 4 -> Zonneveld 5-3-4 (input_sod.txt's method); the I controller (adapt_method 2) keeps
# no error history, so a restart from the saved step size continues the step sequence exactly
# (the PID default would restart its history, as a restarted reference run does)
SOD = dict(nx=128, ny=3, nz=3, xlbc=3, xrbc=3, gamma=1.4, tf=0.2, nout=4, rtol=1e-6,
           atol=1e-11, showstats=1, order=4, adapt_method=2)


def _sod_problem(inp):
    return W.sod(inp.u["nx"], inp.u["ny"], inp.u["nz"], inp.u["gamma"])


def _fields(path, nchem, inp):
    return h5io.read_restart(os.path.dirname(path), int(path[-12:-5]), nchem, inp.domain,
                             inp.shape, inp.field_units())


def test_euler_driver_sod_and_restart(cuda, tmp_path):
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    inp = D.load_inputs(**SOD)
    ra = D.run_euler(inp, _sod_problem, str(a), log=lambda s: None)
    assert len(ra.outputs) == 5 and abs(ra.t - 0.2) < 1e-15
    assert [os.path.basename(p) for p in ra.outputs] == [h5io.output_name(i) for i in range(5)]
    t, f = _fields(ra.outputs[-1], 0, inp)
    assert t == ra.t
    x = (np.arange(128) + 0.5) / 128
    r, u, p = I.sod_exact(x, 0.2)
    assert np.mean(np.abs(f[0][1, 1] - r)) < 7e-3
    # reflecting x, periodic y/z: mass and energy conserved to rounding
    m0, e0 = ra.conservation[0][1:]
    for _, m, e in ra.conservation[1:]:
        assert abs(m - m0) / m0 < 1e-12 and abs(e - e0) / e0 < 1e-12
    assert len(ra.field_rms) == 5 and all(len(v) == 5 for _, v in ra.field_rms)
    # the same run stopped at t = 0.1 (outputs 0-2), then restarted from its files
    D.run_euler(D.load_inputs(**{**SOD, "tf": 0.1, "nout": 2}), _sod_problem, str(b),
                log=lambda s: None)
    rin = D.load_inputs(str(b / "restart_parameters.txt"), tf=0.2, nout=2)
    assert rin.restart == 2 and rin.u["t0"] == 0.1
    rb = D.run_euler(rin, _sod_problem, str(b), log=lambda s: None)
    assert [os.path.basename(p) for p in rb.outputs] == [h5io.output_name(i) for i in (2, 3, 4)]
    _, g = _fields(rb.outputs[-1], 0, inp)
    for k in range(5):
        assert np.array_equal(f[k], g[k]), k


def _chem_inputs(wl, **kw):
    nz, ny, nx = wl["fields"][0].shape
    u = wl["units"]
    # the method and controller settings of the reference's primordial inputs
    # (input_primordial_blast_imex.txt / _mr.txt): ARK4(3)7L[2]SA, I controller
    base = dict(nx=nx, ny=ny, nz=nz, xlbc=3, xrbc=3, gamma=wl["gamma"], tf=4e-6, nout=2,
                rtol=1e-6, atol=1e-10, MassUnits=u["MassUnits"], LengthUnits=u["LengthUnits"],
                TimeUnits=u["TimeUnits"], maxniters=10, nlconvcoef=0.01, safety=0.99, bias=2.0,
                growth=2.0, showstats=1, order=0, etable=13, itable=112, adapt_method=2)
    base.update(kw)
    return D.load_inputs(**base)


def _chem_problem(wl):
    return lambda inp: dict(fields=wl["fields"], scale=wl["scale"], force=None)


def test_imex_driver_outputs_and_restart(cuda, tables, tmp_path):
    wl = W.chem_hydro(shape=(12, 10, 8))
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    inp = _chem_inputs(wl)
    ra = D.run_imex(inp, _chem_problem(wl), tables, str(a), log=lambda s: None)
    assert len(ra.outputs) == 3 and ra.steps > 3 and ra.h > 0.0
    _, f = _fields(ra.outputs[-1], 10, inp)
    D.run_imex(_chem_inputs(wl, tf=2e-6, nout=1), _chem_problem(wl), tables, str(b),
               log=lambda s: None)
    rin = D.load_inputs(str(b / "restart_parameters.txt"), tf=4e-6, nout=1)
    assert rin.restart == 1 and rin.u["t0"] == 2e-6
    rb = D.run_imex(rin, _chem_problem(wl), tables, str(b), log=lambda s: None)
    _, g = _fields(rb.outputs[-1], 10, inp)
    # the restarted run re-initialises the temperature history, as the reference's does
    for k in range(5):
        scale = max(np.max(np.abs(f[k])), 1e-300)
        assert np.max(np.abs(g[k] - f[k])) / scale <= 1e-9, k
    for s in range(10):
        scale = max(np.max(np.abs(f[5][..., s])), 1e-300)
        assert np.max(np.abs(g[5][..., s] - f[5][..., s])) / scale <= 1e-6, s


def test_multirate_driver_matches_direct_run(cuda, tables, tmp_path):
    import torch
    import gbmv
    wl = W.chem_hydro(shape=(8, 6, 5))
    inp = _chem_inputs(wl, h0=1e-6, showstats=0)
    fast = dict(rtol=1e-6, atol=1e-10, maxcor=10, nlscoef=0.01, safety=0.99, growth=2.0,
                max_steps=5000, itable=112)
    r = D.run_multirate(inp, _chem_problem(wl), tables, str(tmp_path), log=lambda s: None)
    assert len(r.outputs) == 3 and r.steps == 4
    _, f = _fields(r.outputs[-1], 10, inp)
    # one call over (0, 4e-6] with the same slow step
    nz, ny, nx = inp.shape
    hy = gbmv.Hydro((nx, ny, nz), 10, inp.bc, inp.u["gamma"], domain=inp.domain)
    c = gbmv.Chem(nx * ny * nz, tables)
    c.set_scale(torch.from_numpy(np.ascontiguousarray(wl["scale"]).reshape(-1)).cuda())
    w = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in wl["fields"]]
    eu = inp.field_units()[2]
    I.mri_evolve(gbmv, hy, c, w, 0.0, 4e-6, 1e-6, eu, inp.u["TimeUnits"], I.MRI_KW3, 0, **fast)
    g = [x.cpu().numpy() for x in w]
    for k in range(5):
        scale = max(np.max(np.abs(g[k])), 1e-300)
        assert np.max(np.abs(f[k] - g[k])) / scale <= 1e-9, k
    for s in range(10):
        scale = max(np.max(np.abs(g[5][..., s])), 1e-300)
        assert np.max(np.abs(f[5][..., s] - g[5][..., s])) / scale <= 1e-7, s
