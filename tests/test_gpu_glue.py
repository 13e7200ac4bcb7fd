"""Chemistry-hydrodynamics glue on the GPU: fexpl / fslow, PostprocessStep and the CFL
stability function, against the oracle composition of the reference's steps
(src/multirate_chem_hydro_main.cpp:996-1083, src/imex_chem_hydro_main.cpp:910-1051,
src/utilities.cpp:483-528)."""
import numpy as np
import pytest

import oracle_py as O
import workloads as W
from conftest import maxnorm_err

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _oracle_fexpl(wl, energy_units):
    f = [x.copy() for x in wl["fields"]]
    scale = wl["scale"]
    phys = f[5] * scale                                      # apply_Dengo_scaling
    f[4] = phys[..., 9] * (1.0 / energy_units) + 0.5 / f[0] * (f[1] * f[1] + f[2] * f[2] + f[3] * f[3])
    st, out = O.feuler(f[:5] + [phys], 10, wl["bc"], wl["gamma"], None)
    out[5][..., 9] = out[4]                                  # chemdot[ge] = etdot
    out[4][:] = 0.0
    f[5] = phys / scale                                      # unapply_Dengo_scaling
    return st, out, f


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_fexpl_matches_oracle_composition(cuda, tables, precision):
    torch = cuda
    import gbmv
    wl = W.chem_hydro(shape=(16, 12, 10))
    eu = wl["units"]["EnergyUnits"]
    st0, ref, wref = _oracle_fexpl(wl, eu)
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(nx * ny * nz, tables)
    c.set_scale(_dev(torch, wl["scale"].reshape(-1)))
    w = [_dev(torch, f) for f in wl["fields"]]
    wdot = [torch.full_like(f, np.nan) for f in w]
    st = gbmv.fexpl(h, c, 0.0, w, wdot, eu, precision)
    torch.cuda.synchronize()
    assert st == st0 == 0
    tol = 1e-12 if precision == 0 else 1e-6
    for i, (a, b) in enumerate(zip(wdot, ref)):
        if i == 5:
            a2, b2 = a.cpu().numpy().reshape(-1, 10), b.reshape(-1, 10)
            for s in range(10):
                assert maxnorm_err(a2[:, s], b2[:, s]) <= tol, (i, s)
        else:
            assert maxnorm_err(a.cpu().numpy(), b) <= tol, i
    # the state is updated as the reference updates it: et from ge, chem*scale/scale
    assert maxnorm_err(w[4].cpu().numpy(), wref[4]) <= 1e-15
    assert maxnorm_err(w[5].cpu().numpy(), wref[5]) <= 1e-15


def test_postprocess_step(cuda, tables):
    torch = cuda
    import gbmv
    wl = W.chem_hydro(shape=(8, 6, 5))
    eu = wl["units"]["EnergyUnits"]
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(nx * ny * nz, tables)
    c.set_scale(_dev(torch, wl["scale"].reshape(-1)))
    w = [_dev(torch, f) for f in wl["fields"]]
    gbmv.PostprocessStep(h, c, w, eu)
    torch.cuda.synchronize()
    f = wl["fields"]
    phys = f[5] * wl["scale"]
    et = phys[..., 9] * (1.0 / eu) + 0.5 / f[0] * (f[1] ** 2 + f[2] ** 2 + f[3] ** 2)
    assert maxnorm_err(w[4].cpu().numpy(), et) <= 1e-15


def test_stability_cfl(cuda):
    torch = cuda
    import gbmv
    wl = W.rayleigh_taylor(shape=(20, 18, 16), nchem=0)
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), 0, wl["bc"], wl["gamma"])
    w = [_dev(torch, f) for f in wl["fields"]]
    dt = h.stability(w, 0.5)
    rho, mx, my, mz, et = wl["fields"]
    p = (wl["gamma"] - 1.0) * (et - (mx * mx + my * my + mz * mz) * 0.5 / rho)
    alpha = np.max(np.abs(mx / rho) + np.sqrt(wl["gamma"] * p / rho))  # |mx/rho| for all axes
    ref = 0.5 * min(1.0 / nx, 1.0 / ny, 1.0 / nz) / alpha
    assert abs(dt - ref) <= 1e-14 * ref


@pytest.mark.parametrize("nforcing", [0, 2])
def test_ffast_matches_oracle_composition(cuda, tables, nforcing):
    """ffast = TimeUnits * f_chem on the chemistry component, zero fluid tendencies, plus
    the MRI forcing sum_i tau^i r_i on all six components."""
    torch = cuda
    import gbmv
    wl = W.chem_hydro(shape=(10, 8, 6))
    TU = wl["units"]["TimeUnits"]
    nz, ny, nx = wl["fields"][0].shape
    n = nx * ny * nz
    h = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(n, tables)
    c.set_scale(_dev(torch, wl["scale"].reshape(-1)))
    w = [_dev(torch, f) for f in wl["fields"]]
    wdot = [torch.full_like(f, np.nan) for f in w]
    rng = np.random.default_rng(7)
    forcing_h = [[rng.standard_normal(f.shape) for f in wl["fields"]] for _ in range(nforcing)]
    forcing = [[_dev(torch, a) for a in fv] for fv in forcing_h]
    t, tshift, tscale = 0.37, 0.1, 0.5
    gbmv.ffast(h, c, t, w, wdot, TU, forcing, tshift, tscale)
    torch.cuda.synchronize()
    oc = O.Chem(tables, wl["scale"].reshape(-1))
    ref = [np.zeros_like(f) for f in wl["fields"]]
    ref[5] = (oc.rhs(wl["fields"][5].reshape(-1)) * TU).reshape(wl["fields"][5].shape)
    tau = (t - tshift) / tscale
    for i, fv in enumerate(forcing_h):
        for k in range(6):
            ref[k] = ref[k] + tau ** i * fv[k]
    for k in range(6):
        a, b = wdot[k].cpu().numpy(), ref[k]
        if k == 5:
            for s in range(10):
                assert maxnorm_err(a[..., s], b[..., s]) <= 1e-12, (k, s)
        else:
            assert maxnorm_err(a, b) <= 1e-15, k


def test_check_conservation_sums(cuda):
    """check_conservation (src/io.cpp:503-542): FP64 totals of rho and et, deterministic, equal
    to exactly rounded sums to 1e-15; and on a periodic grid an explicit RHS step conserves
    them to rounding."""
    torch = cuda
    import math
    import gbmv
    wl = W.rayleigh_taylor(shape=(40, 36, 30), nchem=2)
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), 2, wl["bc"], wl["gamma"])
    w = [_dev(torch, f) for f in wl["fields"]]
    m, e = h.check_conservation(w, 2.0, 3.0)
    assert abs(m - 2.0 * math.fsum(wl["fields"][0].ravel())) <= 1e-15 * abs(m)
    assert abs(e - 3.0 * math.fsum(wl["fields"][4].ravel())) <= 1e-15 * abs(e)
    assert h.check_conservation(w, 2.0, 3.0) == (m, e)  # bitwise repeatable
    ws = W.smooth_periodic(shape=(24, 20, 16), nchem=0)
    hp = gbmv.Hydro((24, 20, 16), 0, ws["bc"], ws["gamma"])
    wp = [_dev(torch, f) for f in ws["fields"]]
    wd = [torch.empty_like(f) for f in wp]
    assert hp.fEuler(0.0, wp, wd, 0) == 0
    m0, e0 = hp.check_conservation(wp)
    w1 = [a + 1e-3 * b for a, b in zip(wp, wd)]
    m1, e1 = hp.check_conservation(w1)
    assert abs(m1 - m0) <= 1e-13 * abs(m0) and abs(e1 - e0) <= 1e-13 * abs(e0)


@pytest.mark.parametrize("nchem", [0, 10])
def test_print_stats_rms(cuda, nchem):
    """print_stats (src/io.cpp:552-640): per-field RMS over the grid, fluid fields through the
    CGS units when asked, chemistry as stored; against exactly rounded sums to 1e-14,
    bitwise repeatable."""
    torch = cuda
    import math
    import gbmv
    wl = W.rayleigh_taylor(shape=(20, 18, 14), nchem=nchem)
    nz, ny, nx = wl["fields"][0].shape
    h = gbmv.Hydro((nx, ny, nz), nchem, wl["bc"], wl["gamma"])
    w = [_dev(torch, f) for f in wl["fields"]]
    n = nx * ny * nz
    for units in ((1.0, 1.0, 1.0), (1.0210809016257265e-21, 0.031507493381465045, 9.7e17)):
        rms = h.print_stats(w, units)
        assert len(rms) == 5 + nchem
        u = (units[0], units[1], units[1], units[1], units[2])
        for v in range(5):
            ref = math.sqrt(math.fsum(((wl["fields"][v] * u[v]) ** 2).ravel()) / n)
            assert abs(rms[v] - ref) <= 1e-14 * ref, v
        for v in range(nchem):
            ref = math.sqrt(math.fsum((wl["fields"][5][..., v] ** 2).ravel()) / n)
            assert abs(rms[5 + v] - ref) <= 1e-14 * ref, v
        assert h.print_stats(w, units) == rms


def test_glue_matches_the_reference_program(cuda, tables):
    """gbmv_fexpl (FP64), gbmv_postprocess_step and the Dengo scaling entries against the
    reference's own IMEX-program fexpl / PostprocessStep and the static problem's
    prepare / apply / unapply_Dengo_scaling compiled from its source
    (tests/golden/glue_cases.npz): fexpl <= 1e-12 per field over two calls in a row (the state
    it rewrites included), the others bit for bit."""
    import os
    torch = cuda
    import gbmv
    from conftest import GOLDEN
    g = np.load(os.path.join(GOLDEN, "glue_cases.npz"))
    for name in [str(c) for c in g["cases"]]:
        w0 = g[f"{name}/w0"]
        nz, ny, nx = w0.shape
        n = nx * ny * nz
        bc = tuple(int(b) for b in g[f"{name}/bc"])
        eu = float(g[f"{name}/EnergyUnits"])
        h = gbmv.Hydro((nx, ny, nz), 10, bc, float(g[f"{name}/gamma"]))
        c = gbmv.Chem(n, tables)
        phys = torch.from_numpy(g[f"{name}/scale"].reshape(-1).copy()).cuda()
        c.prepare_Dengo_structures(phys)  # scale = chem, chem = 1 (prepare_Dengo_structures)
        torch.cuda.synchronize()
        assert torch.equal(phys, torch.ones_like(phys))
        w = [torch.from_numpy(g[f"{name}/w{i}"].copy()).cuda() for i in range(6)]
        for call in range(2):
            out = [torch.empty_like(x) for x in w]
            assert gbmv.fexpl(h, c, 0.0, w, out, eu, gbmv.FP64) == 0
            for i in range(6):
                e = maxnorm_err(out[i].cpu().numpy(), g[f"{name}/fexpl{call}_wdot{i}"])
                assert e <= 1e-12, (name, call, i, e)
                assert np.array_equal(w[i].cpu().numpy(), g[f"{name}/fexpl{call}_w{i}"]), \
                    (name, call, "state", i)
        q = [torch.from_numpy(g[f"{name}/post_in{i}"].copy()).cuda() for i in range(6)]
        assert gbmv.PostprocessStep(h, c, q, eu) == 0
        for i in range(6):
            assert np.array_equal(q[i].cpu().numpy(), g[f"{name}/post_out{i}"]), (name, i)
        s5 = torch.from_numpy(g[f"{name}/w5"].copy()).cuda()
        c.apply_Dengo_scaling(s5.view(-1))
        torch.cuda.synchronize()
        assert np.array_equal(s5.cpu().numpy(), g[f"{name}/applied_chem"])
        c.unapply_Dengo_scaling(s5.view(-1))
        torch.cuda.synchronize()
        assert np.array_equal(s5.cpu().numpy(), g[f"{name}/unapplied_chem"])
