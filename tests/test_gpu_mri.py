"""Multirate chemistry-hydrodynamics integration on the GPU (integrate.mri_evolve with the
MRI-GARK-ERK22b, MIS-KW3 and MRI-GARK-ERK33a couplings: the slow WENO stages through
gbmv_fexpl, the fast stages through gbmv_mri_fast_evolve) against the same scheme driven by
the oracle (fexpl composition of the oracle's fEuler and scaling glue,
the oracle's forced per-cell DIRK, the exact fluid forcing integral)."""
import numpy as np
import pytest

import oracle_py as O
import workloads as W
from conftest import maxnorm_err

pytestmark = pytest.mark.gpu
FAST = dict(rtol=1e-8, atol=1e-12, maxcor=10, nlscoef=0.01)


def _oracle_fexpl(wl_state, wl, eu, units):
    f = [x.copy() for x in wl_state]
    scale = wl["scale"]
    phys = f[5] * scale
    f[4] = phys[..., 9] * (1.0 / eu) + 0.5 / f[0] * (f[1] * f[1] + f[2] * f[2] + f[3] * f[3])
    st, out = O.feuler(f[:5] + [phys], 10, wl["bc"], wl["gamma"], None)
    assert st == 0
    out[5][..., 9] = out[4]
    out[4][:] = 0.0
    f[5] = phys / scale
    if units == "scaled":  # slow chemistry forcing in the scaled fast variables
        out[5][..., :9] = out[5][..., :9] * (1.0 / scale[..., :9])
        out[5][..., 9] = out[5][..., 9] * ((1.0 / scale[..., 9]) * eu)
    return out, f


def _oracle_mri(wl, tables, t0, h, nsteps, eu, tu, table, units):
    """The explicit MRI-GARK step written out over the oracle: stage i's forcing polynomial
    r(tau) = sum_k tau^k sum_j G[k][i-1][j] / dc F_j, tau = (t - ta) / (dc h)."""
    y = [x.copy() for x in wl["fields"]]
    oc = O.Chem(tables, wl["scale"].reshape(-1))
    n = y[0].size
    c, G = table["c"], table["G"]

    def fast(y, ta, tb, g):
        for k in range(5):  # polynomial forcing: exact integral over tau in [0, 1]
            y[k] = y[k] + sum((tb - ta) / (q + 1) * gq[k] for q, gq in enumerate(g))
        z, _, nf = oc.dirk_evolve(y[5].reshape(-1), ta, tb, tu,
                                  forcing=[gq[5].reshape(-1) for gq in g],
                                  tshift=ta, tscale=tb - ta, **FAST)
        assert nf == 0
        y[5] = z.reshape(y[5].shape)
        return y

    for s in range(nsteps):
        t = t0 + s * h
        Fs = []
        for i in range(1, len(c)):
            f, y = _oracle_fexpl(y, wl, eu, units)
            Fs.append(f)
            dc = c[i] - c[i - 1]
            g = [[sum(Gk[i - 1][j] / dc * Fs[j][k] for j in range(i)) for k in range(6)]
                 for Gk in G]
            y = fast(y, t + c[i - 1] * h, t + c[i] * h, g)
    return y, n


def _gpu_mri(torch, wl, tables, t0, h, nsteps, eu, tu, precision, table=None,
             units="reference"):
    import gbmv
    import integrate
    nz, ny, nx = wl["fields"][0].shape
    hy = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(nx * ny * nz, tables)
    c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    if table is None:
        r = integrate.mri_erk22b_evolve(gbmv, hy, c, w, t0, t0 + nsteps * h, h, eu, tu,
                                        precision=precision, forcing_units=units, block=64,
                                        **FAST)
    else:
        r = integrate.mri_evolve(gbmv, hy, c, w, t0, t0 + nsteps * h, h, eu, tu, table,
                                 precision=precision, forcing_units=units, block=64, **FAST)
    torch.cuda.synchronize()
    assert r.fast_failed_cells == 0 and r.slow_steps == nsteps
    return [x.cpu().numpy() for x in w]


def _tables():
    import integrate
    return [None, integrate.MRI_KW3, integrate.MRI_ERK33A]


@pytest.mark.parametrize("which,units", [(0, "scaled"), (1, "scaled"), (2, "scaled"),
                                         (1, "reference")],
                         ids=["erk22b", "kw3", "erk33a", "kw3-reference-units"])
def test_mri_fp64_matches_oracle_driven_scheme(cuda, tables, which, units):
    """Both forcing units: "reference" adds fexpl's chemistry tendency unconverted (the
    reference's fslow), "scaled" converts it to the scaled fast variables first."""
    import integrate
    table = _tables()[which]
    wl = W.chem_hydro(shape=(8, 6, 5))
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    t0, h, ns = 0.0, 2e-6, 2
    ref, n = _oracle_mri(wl, tables, t0, h, ns, eu, tu, table or integrate.MRI_ERK22B, units)
    got = _gpu_mri(cuda, wl, tables, t0, h, ns, eu, tu, 0, table, units)
    for k in range(5):
        assert maxnorm_err(got[k], ref[k]) <= 1e-10, k
    a, b = got[5].reshape(n, 10), ref[5].reshape(n, 10)
    for s in range(10):
        assert maxnorm_err(a[:, s], b[:, s]) <= 1e-6, s
    # the run moved every field (slow and fast parts both active)
    for k in range(6):
        assert not np.array_equal(got[k], wl["fields"][k]) or k == 4


def test_mri_mixed_matches_fp64(cuda, tables):
    wl = W.chem_hydro(shape=(12, 10, 8))
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    a = _gpu_mri(cuda, wl, tables, 0.0, 2e-6, 3, eu, tu, 0)
    b = _gpu_mri(cuda, wl, tables, 0.0, 2e-6, 3, eu, tu, 1)
    for k in range(5):
        assert maxnorm_err(b[k], a[k]) <= 1e-6, k
    n = a[5].size // 10
    for s in range(10):
        assert maxnorm_err(b[5].reshape(n, 10)[:, s], a[5].reshape(n, 10)[:, s]) <= 1e-6, s


@pytest.mark.parametrize("units", ["reference", "scaled"])
def test_mri_graph_replay_matches_host_loop(cuda, tables, units):
    """GraphMRI (each slow step one CUDA graph: fexpl, forcing combinations and the
    persistent-DIRK fast evolves of all stages) against the host loop mri_evolve: the inner
    problems run in local time, so the DIRK's step sequences agree up to the rounding of the
    stage times and the results to well inside the inner tolerance."""
    torch = cuda
    import gbmv
    import integrate
    wl = W.chem_hydro(shape=(8, 6, 5))
    eu, tu = wl["units"]["EnergyUnits"], wl["units"]["TimeUnits"]
    h, ns = 2e-6, 3
    ref = _gpu_mri(torch, wl, tables, 0.0, h, ns, eu, tu, 0, integrate.MRI_KW3, units)
    nz, ny, nx = wl["fields"][0].shape
    hy = gbmv.Hydro((nx, ny, nz), 10, wl["bc"], wl["gamma"])
    c = gbmv.Chem(nx * ny * nz, tables)
    c.set_scale(torch.from_numpy(wl["scale"].reshape(-1).copy()).cuda())
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in wl["fields"]]
    gm = integrate.GraphMRI(gbmv, hy, c, w, h, eu, tu, integrate.MRI_KW3, 0,
                            forcing_units=units, block=64, **FAST)
    r1 = gm.evolve(0.0, h)           # eager first step, then the capture
    r2 = gm.evolve(h, ns * h)        # replays
    assert r1.fast_failed_cells == 0 and r2.fast_failed_cells == 0 and r2.slow_steps == ns - 1
    got = [x.cpu().numpy() for x in w]
    for k in range(5):
        assert maxnorm_err(got[k], ref[k]) <= 1e-9, k
    n = got[5].size // 10
    for s in range(10):
        assert maxnorm_err(got[5].reshape(n, 10)[:, s], ref[5].reshape(n, 10)[:, s]) <= 1e-6, s
