"""The DCPSE_scheme solver's BiCGSTAB (openfpm_numerics_gb300/scheme.py) on
the CPU: convergence to the requested residual on a nonsymmetric 2D system,
an immediate return for a zero right-hand side, and a finite stop (no NaN)
on a breakdown, which solve() then reports."""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300.scheme import bicgstab

scipy_sparse = pytest.importorskip("scipy.sparse")


def _csr(A):
    return torch.sparse_csr_tensor(torch.tensor(A.indptr, dtype=torch.int64), torch.tensor(A.indices, dtype=torch.int64),
                                   torch.tensor(A.data, dtype=torch.float64), size=A.shape)


def _convection_diffusion(n):
    T = scipy_sparse.diags([-1.0, 2.2, -1.1], [-1, 0, 1], shape=(n, n))
    I = scipy_sparse.eye(n)
    return (scipy_sparse.kron(I, T) + scipy_sparse.kron(T, I)).tocsr()


@pytest.mark.parametrize("n", [20, 50])
def test_converges(n):
    A = _convection_diffusion(n)
    xt = np.random.default_rng(n).standard_normal(A.shape[0])
    x, it, res = bicgstab(_csr(A), torch.tensor(A @ xt), tol=1e-10)
    assert res <= 1e-10 and 0 < it < 2000
    assert np.abs(x.numpy() - xt).max() <= 1e-8 * np.abs(xt).max()
    # the residual it reports is the true one
    r = A @ x.numpy() - A @ xt
    assert np.linalg.norm(r) <= 2e-10 * np.linalg.norm(A @ xt)


def test_zero_rhs_returns_at_once():
    A = _convection_diffusion(8)
    x, it, res = bicgstab(_csr(A), torch.zeros(A.shape[0], dtype=torch.float64))
    assert it == 0 and res == 0.0 and torch.count_nonzero(x) == 0


def test_breakdown_stops_finite():
    S = scipy_sparse.csr_matrix(np.array([[1.0, 0.0], [0.0, 0.0]]))
    x, it, res = bicgstab(_csr(S), torch.tensor([1.0, 1.0], dtype=torch.float64), maxiter=500)
    assert it < 500 and res > 1e-3 and torch.isfinite(x).all()
