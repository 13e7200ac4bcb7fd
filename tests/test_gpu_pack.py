"""The reference's halo / pack known-answer test (src/communication_test_main.cpp:133-595) on
the GPU stencil gather (gbmv_pack1d, the pack1D_x/y/z(_bdry) counterpart): every field holds
the digit code 0.TTsXXXyyyZZZ of its rank (0 here), field index and global x/y/z index, and
every stencil value each face reads must equal the code of the cell it should come from, to the
reference's 1e-12.  The reference's case is periodic on 12^3 with NVAR 5 and 9; the boundary
ghost rules (lower faces mirror, upper faces shifted copy, Dirichlet negates all fields,
reflecting negates the normal momentum) are checked the same way."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _code(v, i, j, k):
    return 0.001 * v + 0.000001 * i + 0.000000001 * j + 0.000000000001 * k


def _src(p, n, lo, hi):
    """(source index, negate-all, negate-normal) of stencil position p along an axis."""
    if p < 0:
        if lo == 0:
            return p + n, False, False
        return -1 - p, lo == 2, lo == 3
    if p >= n:
        if hi == 0:
            return p - n, False, False
        return p - 3, hi == 2, hi == 3
    return p, False, False


@pytest.mark.parametrize("nchem,bc", [
    (0, (0, 0, 0, 0, 0, 0)),
    (4, (0, 0, 0, 0, 0, 0)),
    (4, (1, 3, 2, 1, 3, 2)),
    (2, (3, 2, 0, 0, 1, 1)),
])
def test_pack_digits_kat(cuda, nchem, bc):
    torch = cuda
    import gbmv
    nx, ny, nz = 12, 12, 12
    nv = 5 + nchem
    kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    fields = [_code(v, ii, jj, kk) for v in range(5)]
    if nchem:
        fields.append(np.stack([_code(5 + v, ii, jj, kk) for v in range(nchem)], axis=-1))
    h = gbmv.Hydro((nx, ny, nz), nchem, bc, 1.4)
    w = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in fields]
    n = (nx, ny, nz)
    for d in range(3):
        ext = [nx, ny, nz]
        ext[d] += 1
        nfaces = ext[0] * ext[1] * ext[2]
        out = torch.empty(6 * nv * nfaces, dtype=torch.float64, device="cuda")
        h.pack1D(w, d, out)
        got = out.cpu().numpy().reshape(6, nv, ext[2], ext[1], ext[0])
        errs = 0
        for fk in range(ext[2]):
            for fj in range(ext[1]):
                for fi in range(ext[0]):
                    pos = [fi, fj, fk]
                    for l in range(6):
                        p, nall, nnorm = _src(pos[d] - 3 + l, n[d], bc[2 * d], bc[2 * d + 1])
                        q = list(pos)
                        q[d] = p
                        for v in range(nv):
                            t = _code(v, q[0], q[1], q[2])
                            if nall or (nnorm and v == 1 + d):
                                t = -t
                            if abs(got[l, v, fk, fj, fi] - t) > 1e-12:
                                errs += 1
        assert errs == 0, (d, errs)
