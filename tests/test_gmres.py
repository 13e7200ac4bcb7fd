"""Batched GMRES (integrate.batched_gmres) with Ruiz equilibration (integrate.
batched_equilibrate) on the chemistry's real Newton blocks (CPU: torch CPU tensors, the
oracle's analytic Jacobian): I - gamma J of the chem-hydro state for step sizes from the
IMEX driver's first steps up to 1e-2, solved per cell against LAPACK on the equilibrated
blocks.  The blocks' 2-norm condition numbers reach 1e32 (1e9 equilibrated), where Jacobi
scaling alone loses every digit; with equilibration and two restart cycles GMRES(10) agrees
with the direct solve to the equilibrated conditioning's rounding."""
import numpy as np
import pytest

import oracle_py as O
import workloads as W

torch = pytest.importorskip("torch")


def _blocks(tables, shape, gamma):
    wl = W.chem_hydro(shape=shape)
    oc = O.Chem(tables, wl["scale"].reshape(-1))
    y5 = wl["fields"][5].reshape(-1)
    oc.rhs(y5)  # the temperature state the Jacobian uses
    J = oc.jac(y5).reshape(-1, 10, 10).transpose(0, 2, 1) * wl["units"]["TimeUnits"]
    return np.eye(10)[None] - gamma * J


@pytest.mark.parametrize("gamma", [2.47e-7, 1e-5, 1e-4, 1e-2])
def test_gmres_equilibrated_matches_direct_on_chemistry_blocks(tables, gamma):
    import integrate as I
    A = _blocks(tables, (8, 6, 5), gamma)
    b = np.random.default_rng(8).standard_normal((A.shape[0], 10))
    At = torch.from_numpy(A)
    r, c = I.batched_equilibrate(At)
    B = A * r.numpy()[:, :, None] * c.numpy()[:, None, :]
    assert 0.99 <= np.abs(B).max() <= 1.01
    xe = np.linalg.solve(B, (r.numpy() * b)[:, :, None])[:, :, 0] * c.numpy()
    x, it = I.batched_gmres(lambda v: torch.einsum("nij,nj->ni", At, v), torch.from_numpy(b),
                            precond=r, right=c, cycles=2)
    x = x.numpy()
    assert it <= 20
    for s in range(10):
        assert np.max(np.abs(x[:, s] - xe[:, s])) <= 1e-9 * np.max(np.abs(xe[:, s])), s


def test_gmres_jacobi_alone_fails_on_these_blocks(tables):
    """The reason for the column scaling: row scaling by the diagonal alone leaves errors of
    order one on the same blocks."""
    import integrate as I
    A = _blocks(tables, (8, 6, 5), 1e-4)
    b = np.random.default_rng(8).standard_normal((A.shape[0], 10))
    At = torch.from_numpy(A)
    d = 1.0 / torch.diagonal(At, dim1=1, dim2=2)
    x, _ = I.batched_gmres(lambda v: torch.einsum("nij,nj->ni", At, v), torch.from_numpy(b),
                           precond=d, cycles=2)
    xd = np.linalg.solve(A, b[:, :, None])[:, :, 0]
    err = max(np.max(np.abs(x.numpy()[:, s] - xd[:, s])) / np.max(np.abs(xd[:, s]))
              for s in range(10))
    assert err > 1e-3


def test_gmres_stops_per_cell_and_handles_zero_rhs():
    """Cells whose right-hand side is zero, or whose Krylov space closes early (a diagonal
    block: one iteration), keep their exact solution while the other cells iterate."""
    import integrate as I
    rng = np.random.default_rng(3)
    n = 6
    A = rng.standard_normal((n, 10, 10)) + 10 * np.eye(10)[None]
    A[1] = np.diag(np.arange(1.0, 11.0))  # b below is an eigenvector: one iteration
    b = rng.standard_normal((n, 10))
    b[0] = 0.0
    b[1] = 0.0
    b[1, 3] = 2.0
    At = torch.from_numpy(A)
    x, _ = I.batched_gmres(lambda v: torch.einsum("nij,nj->ni", At, v), torch.from_numpy(b))
    x = x.numpy()
    assert np.all(x[0] == 0.0)
    assert np.allclose(x[1], np.linalg.solve(A[1], b[1]), rtol=0, atol=1e-15)
    xd = np.linalg.solve(A, b[:, :, None])[:, :, 0]
    assert np.allclose(x, xd, rtol=1e-12, atol=1e-14)
