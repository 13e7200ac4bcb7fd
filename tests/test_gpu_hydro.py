"""WENO flux divergence on the GPU (part a) against the reference's outputs and the oracle.

Tolerance: the FP64 form must match the reference's fEuler to 1e-12 relative, measured per
field as max|gpu - ref| / max|ref| over the grid (pointwise relative error is meaningless
where flux differences cancel); NaN positions (homogeneous Dirichlet ghosts of the density)
must coincide.
"""
import numpy as np
import pytest

import oracle_py as O
import workloads as W
from conftest import case_fields, feuler_case_names, maxnorm_err

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12


def to_dev(torch, fields):
    return [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in fields]


def run_gpu(torch, fields, nchem, bc, gamma, force, precision=0):
    import gbmv
    nz, ny, nx = fields[0].shape
    h = gbmv.Hydro((nx, ny, nz), nchem, bc, gamma, force)
    w = to_dev(torch, fields)
    wdot = [torch.full_like(f, np.nan) for f in w]
    st = h.fEuler(0.0, w, wdot, precision)
    torch.cuda.synchronize()
    return st, [x.cpu().numpy() for x in wdot]


def test_feuler_matches_reference_fixtures(cuda, golden_feuler):
    g = golden_feuler
    for name in feuler_case_names(g):
        w, nchem, bc, gamma, force = case_fields(g, name)
        st, out = run_gpu(cuda, w, nchem, bc, gamma, force)
        assert st == int(g[f"{name}/status"]), name
        if st:
            continue
        for i, o in enumerate(out):
            e = maxnorm_err(o, g[f"{name}/wdot{i}"])
            assert e <= TOL_FP64, (name, i, e)


@pytest.mark.parametrize("nchem", [0, 2, 4, 6, 10])
def test_feuler_matches_oracle_random(cuda, nchem):
    wl = W.rayleigh_taylor(shape=(24, 20, 17), nchem=nchem, seed=W.SEED_BASE + 90 + nchem)
    wl["bc"] = (3, 3, 0, 0, 1, 2) if nchem % 4 == 0 else (0, 0, 3, 1, 3, 3)
    st0, ref = O.feuler(wl["fields"], nchem, wl["bc"], wl["gamma"], wl["force"])
    st1, out = run_gpu(cuda, wl["fields"], nchem, wl["bc"], wl["gamma"], wl["force"])
    assert st0 == st1 == 0
    for i, (a, b) in enumerate(zip(out, ref)):
        assert maxnorm_err(a, b) <= TOL_FP64, (i, maxnorm_err(a, b))


def test_constant_state_is_steady(cuda):
    """compile_test.cpp's invariant: a uniform state has zero flux divergence."""
    shape = (9, 7, 5)
    sh = (shape[2], shape[1], shape[0])
    f = [np.full(sh, 4.0), np.full(sh, 0.5), np.full(sh, 0.3), np.full(sh, 0.1), np.full(sh, 2.0)]
    f.append(np.broadcast_to((np.arange(4) + 1.0) / 4, sh + (4,)).copy())
    for bc in [(0,) * 6, (1,) * 6]:
        st, out = run_gpu(cuda, f, 4, bc, 1.4, None)
        assert st == 0
        for o in out:
            assert np.all(o == 0.0)


def test_periodic_conservation_full_size(cuda):
    """At 128^3 x 15 (periodic in x/y/z, no forcing) the flux divergence telescopes: the
    grid sum of every field's tendency vanishes to rounding."""
    torch = cuda
    wl = W.rayleigh_taylor(n=128, nchem=10)
    wl["bc"] = (0,) * 6
    st, out = run_gpu(torch, wl["fields"], 10, wl["bc"], wl["gamma"], None)
    assert st == 0
    for i, o in enumerate(out):
        o = o.reshape(-1, 10) if i == 5 else o.reshape(-1, 1)
        tot = np.abs(o.sum(axis=0))
        scale = np.abs(o).sum(axis=0) + 1e-300
        assert np.all(tot / scale < 1e-11), (i, tot / scale)


def test_illegal_state_returns_minus_one(cuda):
    wl = W.rayleigh_taylor(shape=(6, 5, 4), nchem=0)
    wl["fields"][0][1, 1, 1] = -1.0
    st, _ = run_gpu(cuda, wl["fields"], 0, wl["bc"], wl["gamma"], None)
    assert st == -1


def test_invalid_grid_rejected(cuda):
    import gbmv
    with pytest.raises(gbmv.GbmvError):
        gbmv.Hydro((2, 5, 5), 0, (0,) * 6)
    with pytest.raises(gbmv.GbmvError):
        gbmv.Hydro((5, 5, 5), 0, (0, 1, 0, 0, 0, 0))
    with pytest.raises(gbmv.GbmvError):
        gbmv.Hydro((5, 5, 5), 3, (0,) * 6)
