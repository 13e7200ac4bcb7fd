"""Reader for the primordial-chemistry rate-table file (``primordial_tables.h5``).

The reference reads these tables with ``H5LTread_dataset_double`` (src/raja_primordial_network.cpp:432-904),
which needs libhdf5.  The file shipped with the reference is an HDF5 file with superblock version 0, a
symbol-table root group and unfiltered, contiguous, little-endian float64 one-dimensional datasets, so a
small reader of exactly that subset of the format suffices and keeps libhdf5 out of the dependency list.
Anything outside that subset (chunked or filtered layouts, other datatypes, newer superblocks) raises
``ValueError`` instead of returning wrong numbers.

Format facts used (HDF5 File Format Specification, version 0 superblock / version 1 B-tree / symbol table
node / local heap / version 1 object header):
  * superblock: signature, versions, size-of-offsets, size-of-lengths, addresses, root symbol-table entry
    whose scratch pad holds the root group's B-tree and local-heap addresses;
  * group B-tree nodes ``TREE`` (type 0) whose leaves point at ``SNOD`` symbol-table nodes;
  * ``SNOD`` entries: link-name offset into the local heap + object-header address;
  * object header v1 messages: 0x0001 dataspace, 0x0003 datatype, 0x0008 data layout, 0x0010 continuation.
"""
from __future__ import annotations

import struct

import numpy as np

# The 50 tables the network uses, in the order the device-side table block stores them.
# Rate coefficients k01..k22 (k20 absent), cooling terms, then the H2 adiabatic-index tables
# (src/raja_primordial_network.hpp:115-166).
RATE_NAMES = ["k01", "k02", "k03", "k04", "k05", "k06", "k07", "k08", "k09", "k10", "k11",
              "k12", "k13", "k14", "k15", "k16", "k17", "k18", "k19", "k21", "k22"]
COOLING_NAMES = ["brem_brem", "ceHeI_ceHeI", "ceHeII_ceHeII", "ceHI_ceHI", "cie_cooling_cieco",
                 "ciHeI_ciHeI", "ciHeII_ciHeII", "ciHeIS_ciHeIS", "ciHI_ciHI", "compton_comp_",
                 "gloverabel08_gael", "gloverabel08_gaH2", "gloverabel08_gaHe", "gloverabel08_gaHI",
                 "gloverabel08_gaHp", "gloverabel08_h2lte", "h2formation_h2mcool",
                 "h2formation_h2mheat", "h2formation_ncrd1", "h2formation_ncrd2", "h2formation_ncrn",
                 "reHeII1_reHeII1", "reHeII2_reHeII2", "reHeIII_reHeIII", "reHII_reHII"]
GAMMA_NAMES = ["gammaH2_1", "dgammaH2_1_dT", "gammaH2_2", "dgammaH2_2_dT"]
TABLE_NAMES = RATE_NAMES + COOLING_NAMES + GAMMA_NAMES
TABLE_LEN = 1024

_SIG = b"\x89HDF\r\n\x1a\n"


class _File:
    def __init__(self, data: bytes):
        self.d = data
        if data[:8] != _SIG:
            raise ValueError("not an HDF5 file")
        if data[8] != 0:
            raise ValueError(f"superblock version {data[8]} not supported (need 0)")
        self.so = data[13]  # size of offsets
        self.sl = data[14]  # size of lengths
        if self.so != 8 or self.sl != 8:
            raise ValueError("only 8-byte offsets/lengths supported")
        p = 24
        self.base, _free, _eof, _drv = struct.unpack_from("<4Q", data, p)
        p += 32
        # root group symbol table entry: name off, obj header addr, cache type, reserved, scratch(16)
        _name, self.root_ohdr, cache_type, _res = struct.unpack_from("<QQII", data, p)
        if cache_type != 1:
            raise ValueError("root symbol-table entry does not cache a B-tree/heap address")
        self.root_btree, self.root_heap = struct.unpack_from("<QQ", data, p + 24)

    def u64(self, p):
        return struct.unpack_from("<Q", self.d, p)[0]

    def heap_data(self, heap_addr):
        if self.d[heap_addr:heap_addr + 4] != b"HEAP":
            raise ValueError("bad local heap")
        _size, _free, data_addr = struct.unpack_from("<QQQ", self.d, heap_addr + 8)
        return data_addr

    def name_at(self, heap_data_addr, off):
        p = heap_data_addr + off
        e = self.d.index(b"\0", p)
        return self.d[p:e].decode()

    def group_entries(self):
        """Yield (name, object-header address) for every link in the root group."""
        heap = self.heap_data(self.root_heap)
        stack = [self.root_btree]
        while stack:
            node = stack.pop()
            if self.d[node:node + 4] != b"TREE":
                raise ValueError("bad B-tree node")
            ntype, level, nused = struct.unpack_from("<BBH", self.d, node + 4)
            if ntype != 0:
                raise ValueError("not a group B-tree")
            p = node + 8 + 16  # skip signature/type/level/entries + left/right sibling
            p += self.sl       # key 0
            for _ in range(nused):
                child = self.u64(p)
                p += self.so + self.sl
                if level > 0:
                    stack.append(child)
                else:
                    yield from self.snod_entries(child, heap)

    def snod_entries(self, addr, heap):
        if self.d[addr:addr + 4] != b"SNOD":
            raise ValueError("bad symbol table node")
        nsym = struct.unpack_from("<H", self.d, addr + 6)[0]
        p = addr + 8
        for _ in range(nsym):
            name_off, ohdr = struct.unpack_from("<QQ", self.d, p)
            yield self.name_at(heap, name_off), ohdr
            p += 40

    def messages(self, ohdr):
        d = self.d
        if d[ohdr] != 1:
            raise ValueError("object header version != 1")
        nmsg = struct.unpack_from("<H", d, ohdr + 2)[0]
        hsize = struct.unpack_from("<I", d, ohdr + 8)[0]
        blocks = [(ohdr + 16, hsize)]
        out = []
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            p = start
            while p + 8 <= start + size and len(out) < nmsg:
                mtype, msize, _flags = struct.unpack_from("<HHB", d, p)
                body = p + 8
                if mtype == 0x10:
                    coff, clen = struct.unpack_from("<QQ", d, body)
                    blocks.append((coff, clen))
                out.append((mtype, body, msize))
                p = body + msize
        return out

    def read_f64(self, ohdr):
        dims = None
        layout = None
        for mtype, body, _size in self.messages(ohdr):
            d = self.d
            if mtype == 0x0001:  # dataspace
                ver, ndim = d[body], d[body + 1]
                off = body + (8 if ver == 1 else 4)
                dims = struct.unpack_from(f"<{ndim}Q", d, off)
            elif mtype == 0x0003:  # datatype
                cls_ver = d[body]
                dclass = cls_ver & 0x0F
                bits0 = d[body + 1]
                esize = struct.unpack_from("<I", d, body + 4)[0]
                if dclass != 1 or esize != 8 or (bits0 & 1):
                    raise ValueError("dataset is not little-endian float64")
            elif mtype == 0x0008:  # data layout
                ver = d[body]
                if ver == 3:
                    lclass = d[body + 1]
                    if lclass != 1:
                        raise ValueError("only contiguous layout supported")
                    addr, nbytes = struct.unpack_from("<QQ", d, body + 2)
                    layout = (addr, nbytes)
                elif ver in (1, 2):
                    ndim, lclass = d[body + 1], d[body + 2]
                    if lclass != 1:
                        raise ValueError("only contiguous layout supported")
                    addr = struct.unpack_from("<Q", d, body + 8)[0]
                    shp = struct.unpack_from(f"<{ndim}I", d, body + 16)
                    layout = (addr, int(np.prod(shp)))
                else:
                    raise ValueError(f"layout message version {ver} not supported")
            elif mtype == 0x000B:
                raise ValueError("filtered datasets not supported")
        if dims is None or layout is None:
            raise ValueError("dataset header lacks dataspace or layout")
        n = int(np.prod(dims))
        addr = layout[0] + self.base
        return np.frombuffer(self.d, dtype="<f8", count=n, offset=addr).copy().reshape(dims)

    def read_array(self, ohdr):
        """A contiguous dataset of little-endian float64, or of signed 32/64-bit integers, of
        any rank (a rank-0 version-1 dataspace is a scalar)."""
        d = self.d
        dtype = None
        for mtype, body, _size in self.messages(ohdr):
            if mtype == 0x0003:
                dclass, bits0 = d[body] & 0x0F, d[body + 1]
                esize = struct.unpack_from("<I", d, body + 4)[0]
                if bits0 & 1:
                    raise ValueError("big-endian datasets not supported")
                if dclass == 1 and esize == 8:
                    dtype = "<f8"
                elif dclass == 0 and esize in (4, 8) and (bits0 & 0x08):
                    dtype = "<i4" if esize == 4 else "<i8"
                else:
                    raise ValueError(f"datatype class {dclass} size {esize} not supported")
        if dtype is None:
            raise ValueError("dataset header lacks a datatype")
        if dtype == "<f8":
            return self.read_f64(ohdr)
        dims = layout = None
        for mtype, body, _size in self.messages(ohdr):
            if mtype == 0x0001:
                ver, ndim = d[body], d[body + 1]
                dims = struct.unpack_from(f"<{ndim}Q", d, body + (8 if ver == 1 else 4))
            elif mtype == 0x0008 and d[body] == 3 and d[body + 1] == 1:
                layout = struct.unpack_from("<Q", d, body + 2)[0]
        if dims is None or layout is None:
            raise ValueError("integer dataset lacks a dataspace or a contiguous layout")
        n = int(np.prod(dims))
        return np.frombuffer(d, dtype=dtype, count=n, offset=layout + self.base).copy().reshape(dims)


def read_datasets(path: str) -> dict[str, np.ndarray]:
    """Every root-group dataset of a file in the supported subset (float64 or integer)."""
    with open(path, "rb") as f:
        hf = _File(f.read())
    return {name: hf.read_array(oh) for name, oh in hf.group_entries()}


def read_tables(path: str) -> dict[str, np.ndarray]:
    """Read every dataset of the root group into a dict name -> float64 array."""
    with open(path, "rb") as f:
        hf = _File(f.read())
    return {name: hf.read_f64(oh) for name, oh in hf.group_entries()}


def load_table_block(path: str) -> np.ndarray:
    """Return the (50, 1024) float64 table block in ``TABLE_NAMES`` order."""
    t = read_tables(path)
    missing = [n for n in TABLE_NAMES if n not in t]
    if missing:
        raise ValueError(f"table file lacks datasets: {missing}")
    blk = np.stack([np.asarray(t[n], dtype=np.float64).reshape(-1) for n in TABLE_NAMES])
    if blk.shape != (len(TABLE_NAMES), TABLE_LEN):
        raise ValueError(f"unexpected table shape {blk.shape}")
    return np.ascontiguousarray(blk)
