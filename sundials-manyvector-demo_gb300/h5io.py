"""Solution output and restart in the reference's file formats (src/io.cpp), without libhdf5.

* ``write_solution`` -- output_solution (src/io.cpp:723-940): ``output-%07i.hdf5`` holding the
  scalar datasets ``time`` (float64) and ``nchem`` (int32), ``domain`` (3 x 2 float64: z, y, x
  bounds), the fluid fields ``Density``, ``x-Momentum``, ``y-Momentum``, ``z-Momentum``,
  ``TotalEnergy`` in CGS units (code value x DensityUnits / MomentumUnits / EnergyUnits) and one
  ``Chemical-%03d`` dataset per species as stored, each [nz][ny][nx] float64.  The reference
  scales the state in place and back around the write (a rounding round trip of the state);
  here the state is left untouched.
* ``read_restart`` -- read_restart (src/io.cpp:955-1158): the same checks (float64 time, equal
  nchem, a 3 x 2 domain within 1e-14, [nz][ny][nx] fields) and the fluid fields multiplied
  back by 1 / units.
* ``write_parameters`` / ``read_parameters`` -- write_parameters (src/io.cpp:641-721): the
  ``restart_parameters.txt`` ``key = value`` file, floats as ``%.16e``.

The HDF5 files are written in the layout libhdf5 uses for such a file by default, the same
subset ``h5tables`` reads: version-0 superblock (8-byte offsets and lengths, group leaf K 4,
internal K 16), a root group with a symbol table (one version-1 B-tree node over symbol-table
nodes of at most 8 entries sorted by name, keys = the largest name in each child, a local heap
with an 8-byte empty name at offset 0 and a trailing free block), and per dataset a version-1
object header with dataspace (v1), datatype, fill-value (v2) and contiguous-layout (v3)
messages.  (HDF5 File Format Specification, superblock v0, B-tree v1, symbol table node, local
heap, object header v1 and the messages named.)
"""
from __future__ import annotations

import math
import os
import struct

import numpy as np

from h5tables import _File

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF
_LEAF_K, _NODE_K = 4, 16  # libhdf5's defaults
_SNOD_CAP = 2 * _LEAF_K
_MAX_LINKS = _SNOD_CAP * 2 * _NODE_K  # one B-tree node of symbol-table nodes
# datatype messages, version 1: IEEE little-endian float64; signed little-endian int32
_T_F64 = bytes.fromhex("11203f00" "08000000" "0000" "4000" "34" "0b" "00" "34" "ff030000")
_T_I32 = bytes.fromhex("10080000" "04000000" "0000" "2000")
_FILL = bytes.fromhex("0202020100000000")  # fill value v2: late allocation, default fill

FLUID_NAMES = ["Density", "x-Momentum", "y-Momentum", "z-Momentum", "TotalEnergy"]


def _pad8(n: int) -> int:
    return (n + 7) & ~7


def _msg(mtype: int, body: bytes) -> bytes:
    body = body + bytes(_pad8(len(body)) - len(body))
    return struct.pack("<HHB3x", mtype, len(body), 0) + body


def _dataspace(shape) -> bytes:
    return struct.pack("<BBB5x", 1, len(shape), 0) + b"".join(struct.pack("<Q", int(d))
                                                               for d in shape)


class _Buffer:
    def __init__(self):
        self.b = bytearray()

    def alloc(self, n: int) -> int:
        a = _pad8(len(self.b))
        self.b.extend(bytes(a - len(self.b) + n))
        return a

    def put(self, addr: int, data: bytes):
        self.b[addr:addr + len(data)] = data


def write_h5(path: str, datasets) -> None:
    """Write a file whose root group holds `datasets` (name -> numpy array of float64 or int32,
    any rank; rank 0 is a scalar)."""
    items = []
    for name, arr in datasets.items():
        a = np.asarray(arr)
        if a.dtype == np.float64:
            a, dt = np.array(a, dtype="<f8", order="C"), _T_F64
        elif a.dtype == np.int32:
            a, dt = np.array(a, dtype="<i4", order="C"), _T_I32
        else:
            raise ValueError(f"{name}: dtype {a.dtype} not supported (float64, int32)")
        items.append((name.encode(), a, dt))
    items.sort(key=lambda it: it[0])  # symbol-table nodes are sorted by name (byte order)
    names = [it[0] for it in items]
    if len(set(names)) != len(names) or any(not n or b"\0" in n for n in names):
        raise ValueError("dataset names must be unique, non-empty, without NUL")
    if len(items) > _MAX_LINKS:
        raise ValueError(f"at most {_MAX_LINKS} datasets")
    f = _Buffer()
    sb = f.alloc(96)
    root = f.alloc(16 + 8 + 16)
    nsnod = max(1, math.ceil(len(items) / _SNOD_CAP))
    btree = f.alloc(24 + (2 * _NODE_K + 1) * 8 + 2 * _NODE_K * 8)
    heap = bytearray(8)  # the empty name at offset 0
    name_off = []
    for n in names:
        name_off.append(len(heap))
        heap += n + b"\0"
        heap += bytes(_pad8(len(heap)) - len(heap))
    free_off = len(heap)
    heap += struct.pack("<QQ", 1, 16)  # one free block: no next block (1), 16 bytes
    heap_hdr = f.alloc(32)
    heap_data = f.alloc(len(heap))
    snods = [f.alloc(8 + _SNOD_CAP * 40) for _ in range(nsnod)]
    ohdrs = []
    for _name, a, dt in items:
        nbytes = a.nbytes
        msgs_len = sum(8 + _pad8(len(x)) for x in (_dataspace(a.shape), dt, _FILL, bytes(18)))
        oh = f.alloc(16 + msgs_len)
        data = f.alloc(nbytes)
        body = (_msg(0x0001, _dataspace(a.shape)) + _msg(0x0003, dt) + _msg(0x0005, _FILL) +
                _msg(0x0008, struct.pack("<BBQQ", 3, 1, data, nbytes)))
        f.put(oh, struct.pack("<BBHII4x", 1, 0, 4, 1, len(body)) + body)
        f.put(data, a.tobytes())
        ohdrs.append(oh)
    eof = len(f.b)
    f.put(sb, _SIG + struct.pack("<8BHHI", 0, 0, 0, 0, 0, 8, 8, 0, _LEAF_K, _NODE_K, 0) +
          struct.pack("<4Q", 0, _UNDEF, eof, _UNDEF) +
          struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", btree, heap_hdr))
    f.put(root, struct.pack("<BBHII4x", 1, 0, 1, 1, 24) +
          _msg(0x0011, struct.pack("<QQ", btree, heap_hdr)))
    f.put(heap_hdr, b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), free_off, heap_data))
    f.put(heap_data, bytes(heap))
    node = bytearray(b"TREE" + struct.pack("<BBH", 0, 0, nsnod) +
                     struct.pack("<QQ", _UNDEF, _UNDEF))
    node += struct.pack("<Q", 0)  # key 0: the empty name
    for s in range(nsnod):
        lo, hi = s * _SNOD_CAP, min(len(items), (s + 1) * _SNOD_CAP)
        ent = b"".join(struct.pack("<QQII16x", name_off[k], ohdrs[k], 0, 0)
                       for k in range(lo, hi))
        f.put(snods[s], b"SNOD" + struct.pack("<BBH", 1, 0, hi - lo) + ent)
        node += struct.pack("<QQ", snods[s], name_off[hi - 1])  # child, then its largest name
    f.put(btree, bytes(node))
    with open(path, "wb") as fh:
        fh.write(bytes(f.b))


def read_h5(path: str) -> dict:
    """name -> numpy array for every dataset of a file in the supported subset."""
    with open(path, "rb") as fh:
        hf = _File(fh.read())
    return {name: hf.read_array(oh) for name, oh in hf.group_entries()}


# ------------------------------------------------------------------ the reference's layout

def units(mass_units: float, length_units: float, time_units: float):
    """(DensityUnits, MomentumUnits, EnergyUnits) as src/euler3D.hpp:389-391 forms them."""
    m, l, t = mass_units, length_units, time_units
    return m / l / l / l, m / l / l / t, m / l / t / t


def output_name(iout: int) -> str:
    return "output-%07i.hdf5" % iout


def _host(x) -> np.ndarray:
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    return np.asarray(x, dtype=np.float64)


def write_solution(directory: str, iout: int, t: float, w, domain, field_units) -> str:
    """output_solution: w = the six ManyVector components (host or device arrays; fluid
    [nz][ny][nx], chemistry [nz][ny][nx][nchem] or empty), domain = (xl, xr, yl, yr, zl, zr),
    field_units = (DensityUnits, MomentumUnits, EnergyUnits).  Returns the file path."""
    fl = [_host(x) for x in w[:5]]
    shape = fl[0].shape
    if len(shape) != 3 or any(x.shape != shape for x in fl):
        raise ValueError("fluid fields must share one [nz][ny][nx] shape")
    chem = _host(w[5]) if len(w) > 5 and w[5] is not None else np.zeros(shape + (0,))
    chem = chem.reshape(shape + (-1,))
    xl, xr, yl, yr, zl, zr = domain
    du, mu, eu = field_units
    ds = {"time": np.float64(t), "nchem": np.int32(chem.shape[3]),
          "domain": np.array([[zl, zr], [yl, yr], [xl, xr]], dtype=np.float64)}
    for name, x, u in zip(FLUID_NAMES, fl, (du, mu, mu, mu, eu)):
        ds[name] = x * u
    for v in range(chem.shape[3]):
        ds["Chemical-%03d" % v] = np.ascontiguousarray(chem[..., v])
    path = os.path.join(directory, output_name(iout))
    write_h5(path, ds)
    return path


def read_restart(directory: str, restart: int, nchem: int, domain, shape, field_units):
    """read_restart: (t, [rho, mx, my, mz, et, chem]) in code units from output-%07i.hdf5;
    shape = (nz, ny, nx); chem is [nz][ny][nx][nchem].  Raises ValueError where the reference
    reports an incompatible file."""
    path = os.path.join(directory, output_name(restart))
    with open(path, "rb") as fh:
        hf = _File(fh.read())
    links = dict(hf.group_entries())

    def get(name):
        if name not in links:
            raise ValueError(f"read_restart: {name} missing")
        return hf.read_array(links[name])
    t = get("time")
    if t.dtype != np.float64 or t.shape != ():
        raise ValueError("read_restart: file type does not match 'realtype' type")
    if int(get("nchem")) != nchem:
        raise ValueError("read_restart: incompatible number of chemical/tracer fields")
    dom = get("domain")
    xl, xr, yl, yr, zl, zr = domain
    if dom.shape != (3, 2) or np.any(np.abs(dom.reshape(-1) -
                                            np.array([zl, zr, yl, yr, xl, xr])) > 1e-14):
        raise ValueError("read_restart: incompatible domain")
    du, mu, eu = field_units
    out = []
    for name, u in zip(FLUID_NAMES, (du, mu, mu, mu, eu)):
        x = get(name)
        if x.ndim != 3:
            raise ValueError("read_restart: incompatible field dimensions")
        if tuple(x.shape) != tuple(shape):
            raise ValueError("read_restart: incompatible field size")
        out.append(x * (1.0 / u))
    chem = np.empty(tuple(shape) + (nchem,))
    for v in range(nchem):
        x = get("Chemical-%03d" % v)
        if tuple(x.shape) != tuple(shape):
            raise ValueError("read_restart: incompatible field size")
        chem[..., v] = x
    out.append(chem)
    return float(t), out


# restart_parameters.txt keys in the order write_parameters prints them; "e" = %.16e
PARAMETERS = [("xl", "e"), ("xr", "e"), ("yl", "e"), ("yr", "e"), ("zl", "e"), ("zr", "e"),
              ("t0", "e"), ("tf", "e"), ("gamma", "e"), ("MassUnits", "e"),
              ("LengthUnits", "e"), ("TimeUnits", "e"), ("nx", "i"), ("ny", "i"), ("nz", "i"),
              ("xlbc", "i"), ("xrbc", "i"), ("ylbc", "i"), ("yrbc", "i"), ("zlbc", "i"),
              ("zrbc", "i"), ("cfl", "e"), ("nout", "i"), ("showstats", "i"), ("order", "i"),
              ("dense_order", "i"), ("etable", "i"), ("itable", "i"), ("mtable", "i"),
              ("adapt_method", "i"), ("maxnef", "i"), ("mxhnil", "i"), ("mxsteps", "i"),
              ("safety", "e"), ("bias", "e"), ("growth", "e"), ("pq", "i"), ("k1", "e"),
              ("k2", "e"), ("k3", "e"), ("etamx1", "e"), ("etamxf", "e"), ("h0", "e"),
              ("hmin", "e"), ("hmax", "e"), ("fixedstep", "i"), ("htrans", "e"), ("rtol", "e"),
              ("atol", "e"), ("fusedkernels", "i"), ("localreduce", "i"), ("restart", "i")]


def write_parameters(directory: str, params: dict, tcur: float, hcur: float, iout: int) -> str:
    """restart_parameters.txt as write_parameters writes it: the run's parameters with t0 = tcur,
    h0 = hcur, nout = nout - iout and restart = iout.  Returns the path."""
    p = dict(params)
    p.update(t0=tcur, h0=hcur, nout=int(params["nout"]) - iout, restart=iout)
    lines = ["# Euler3D restart file"]
    for key, kind in PARAMETERS:
        val = "%.16e" % float(p[key]) if kind == "e" else "%i" % int(p[key])
        lines.append(f"{key} = {val}")
    path = os.path.join(directory, "restart_parameters.txt")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return path


def read_parameters(path: str) -> dict:
    """`key = value` lines (comments after '#', blank lines skipped), as the reference's input
    files are written; integers for the integer keys, floats otherwise."""
    kinds = dict(PARAMETERS)
    out = {}
    with open(path) as fh:
        for line in fh:
            line = line.split("#", 1)[0].strip()
            if not line:
                continue
            key, _, val = line.partition("=")
            key, val = key.strip(), val.strip()
            out[key] = int(val) if kinds.get(key) == "i" else float(val)
    return out
