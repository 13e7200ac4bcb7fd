"""The superblock-v0 table reader against the file shipped with the reference (CPU)."""
import numpy as np
import pytest

import h5tables
from conftest import TABLES


def test_reads_all_datasets():
    t = h5tables.read_tables(TABLES)
    assert len(t) == 55
    for name in h5tables.TABLE_NAMES:
        assert t[name].shape == (1024,)
        assert np.all(np.isfinite(t[name]))


def test_table_block_order():
    blk = h5tables.load_table_block(TABLES)
    t = h5tables.read_tables(TABLES)
    assert blk.shape == (50, 1024)
    for i, name in enumerate(h5tables.TABLE_NAMES):
        assert np.array_equal(blk[i], t[name])
    # the H2 adiabatic index tables are physical (gamma between 1 and ~5/3)
    g1 = t["gammaH2_1"]
    assert np.all((g1 > 1.0) & (g1 < 1.7))


def test_rejects_non_hdf5(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not an hdf5 file at all" * 10)
    with pytest.raises(ValueError):
        h5tables.read_tables(str(p))
