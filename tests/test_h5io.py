"""Solution output / restart in the reference's formats (h5io): the HDF5 writer against the
conventions of the libhdf5-written table file the reference ships, round trips through the
reader, read_restart's compatibility checks, and restart_parameters.txt."""
import os
import struct

import numpy as np
import pytest

import h5io
import h5tables
from conftest import GOLDEN


def _state(shape=(4, 5, 6), nchem=10, seed=3):
    rng = np.random.default_rng(seed)
    w = [rng.uniform(0.5, 2.0, shape)] + [rng.standard_normal(shape) for _ in range(3)]
    w.append(rng.uniform(1.0, 3.0, shape))
    w.append(rng.uniform(0.0, 1.0, shape + (nchem,)))
    return w


UNITS = h5io.units(3.0e70, 3.0857e30, 1.0e11)
DOMAIN = (0.0, 1.0, -0.5, 0.5, 0.0, 2.0)


def test_units_as_reference():
    m, l, t = 3.0e70, 3.0857e30, 1.0e11
    du, mu, eu = h5io.units(m, l, t)
    assert du == m / l / l / l and mu == m / l / l / t and eu == m / l / t / t


def test_solution_round_trip(tmp_path):
    w = _state()
    path = h5io.write_solution(str(tmp_path), 12, 0.375, w, DOMAIN, UNITS)
    assert os.path.basename(path) == "output-0000012.hdf5"
    ds = h5io.read_h5(path)
    names = {"time", "nchem", "domain", *h5io.FLUID_NAMES,
             *["Chemical-%03d" % v for v in range(10)]}
    assert set(ds) == names
    assert ds["time"].shape == () and float(ds["time"]) == 0.375
    assert ds["nchem"].dtype == np.int32 and int(ds["nchem"]) == 10
    assert np.array_equal(ds["domain"], [[0.0, 2.0], [-0.5, 0.5], [0.0, 1.0]])
    du, mu, eu = UNITS
    assert np.array_equal(ds["Density"], w[0] * du)  # CGS on disk
    assert np.array_equal(ds["TotalEnergy"], w[4] * eu)
    assert np.array_equal(ds["Chemical-007"], w[5][..., 7])  # chemistry as stored
    t, r = h5io.read_restart(str(tmp_path), 12, 10, DOMAIN, w[0].shape, UNITS)
    assert t == 0.375
    for k, u in zip(range(5), (du, mu, mu, mu, eu)):
        assert np.array_equal(r[k], (w[k] * u) * (1.0 / u))  # the reference's scalings
        np.testing.assert_allclose(r[k], w[k], rtol=1e-15, atol=0)
    assert np.array_equal(r[5], w[5])


def test_writer_follows_libhdf5_layout(tmp_path):
    """Superblock fields, root-group B-tree keys, symbol-table node order and heap free list
    follow the conventions of the table file libhdf5 wrote."""
    ref = open(os.path.join(GOLDEN, "primordial_tables.h5"), "rb").read()
    w = _state(nchem=30)  # 38 links: five symbol-table nodes
    path = h5io.write_solution(str(tmp_path), 0, 1.0, w, DOMAIN, UNITS)
    d = open(path, "rb").read()
    assert d[:24] == ref[:24]  # signature, versions, sizes, K values, flags
    f = h5tables._File(d)
    assert struct.unpack_from("<Q", d, 40)[0] == len(d)  # end-of-file address
    bt = f.root_btree
    ntype, level, nused = struct.unpack_from("<BBH", d, bt + 4)
    assert (d[bt:bt + 4], ntype, level, nused) == (b"TREE", 0, 0, 5)
    hd = f.heap_data(f.root_heap)
    size, free, _ = struct.unpack_from("<QQQ", d, f.root_heap + 8)
    assert struct.unpack_from("<QQ", d, hd + free) == (1, 16) and free + 16 == size
    assert d[hd:hd + 8] == bytes(8)
    p = bt + 24
    keys, kids = [], []
    for _ in range(nused):
        keys.append(f.name_at(hd, struct.unpack_from("<Q", d, p)[0]))
        kids.append(struct.unpack_from("<Q", d, p + 8)[0])
        p += 16
    keys.append(f.name_at(hd, struct.unpack_from("<Q", d, p)[0]))
    all_names = []
    for i, k in enumerate(kids):
        ents = [n for n, _ in f.snod_entries(k, hd)]
        assert 1 <= len(ents) <= 8 and ents == sorted(ents, key=str.encode)
        assert keys[i] < ents[0] and keys[i + 1] == ents[-1]
        all_names += ents
    assert keys[0] == "" and len(all_names) == 38
    assert all_names == sorted(all_names, key=str.encode)
    ds = h5io.read_h5(path)
    assert np.array_equal(ds["Chemical-029"], w[5][..., 29])


def test_read_restart_rejects_incompatible_files(tmp_path):
    w = _state()
    h5io.write_solution(str(tmp_path), 3, 0.5, w, DOMAIN, UNITS)
    d = str(tmp_path)
    shape = w[0].shape
    with pytest.raises(ValueError, match="chemical"):
        h5io.read_restart(d, 3, 9, DOMAIN, shape, UNITS)
    with pytest.raises(ValueError, match="domain"):
        h5io.read_restart(d, 3, 10, (0.0, 1.0, -0.5, 0.5, 0.0, 2.1), shape, UNITS)
    with pytest.raises(ValueError, match="field size"):
        h5io.read_restart(d, 3, 10, DOMAIN, (4, 5, 7), UNITS)
    with pytest.raises(FileNotFoundError):
        h5io.read_restart(d, 4, 10, DOMAIN, shape, UNITS)
    with pytest.raises(ValueError):
        h5io.write_h5(os.path.join(d, "bad.h5"), {"x": np.zeros(3, dtype=np.float32)})


def test_hydro_only_output(tmp_path):
    w = _state(nchem=0)[:5] + [None]
    h5io.write_solution(str(tmp_path), 1, 0.0, w, DOMAIN, UNITS)
    t, r = h5io.read_restart(str(tmp_path), 1, 0, DOMAIN, w[0].shape, UNITS)
    assert r[5].shape == w[0].shape + (0,)


def test_restart_parameters(tmp_path):
    params = {k: (1 if kind == "i" else 0.5) for k, kind in h5io.PARAMETERS}
    params.update(nout=10, nx=128, TimeUnits=1.0e11, rtol=1e-6)
    path = h5io.write_parameters(str(tmp_path), params, tcur=0.25, hcur=3.0e-5, iout=4)
    lines = open(path).read().splitlines()
    assert lines[0] == "# Euler3D restart file"
    assert [ln.split(" = ")[0] for ln in lines[1:]] == [k for k, _ in h5io.PARAMETERS]
    assert "t0 = 2.5000000000000000e-01" in lines and "nout = 6" in lines
    assert "TimeUnits = 1.0000000000000000e+11" in lines and "restart = 4" in lines
    back = h5io.read_parameters(path)
    assert back["t0"] == 0.25 and back["h0"] == 3.0e-5 and back["nx"] == 128
    assert isinstance(back["nx"], int) and back["rtol"] == 1e-6
