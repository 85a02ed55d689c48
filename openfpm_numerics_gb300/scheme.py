"""Implicit DC-PSE systems on one GPU: the role of DCPSE_scheme
(src/DCPSE/DCPSE_op/DCPSE_Solver.hpp:42-1040).

    S = DCPSE_scheme(parts)
    S.impose(Lap, bulk, rhs)            # rows of Lap(v) = rhs on the bulk particles
    S.impose(IDENTITY, boundary, g)     # v = g on the boundary
    x = S.solve()                       # BiCGSTAB on the device

Every operator row comes from the plan's CSR export (dcpse_operator_csr), the
same non-zeros value_nz hands to impose_git; rows of several imposed terms
on one equation are summed.  The reference hands the assembled system to
PETSc or Eigen; here the solve is a Jacobi-preconditioned BiCGSTAB with the
sparse products of torch (cuSPARSE), since the matrix already lives on the
device.
"""
from __future__ import annotations

import torch

IDENTITY = "identity"  # the unknown itself (impose(v, subset, rhs) in the reference)


def _as_index(subset):
    if isinstance(subset, torch.Tensor):
        return subset.to(device="cuda", dtype=torch.int64).contiguous()
    return torch.as_tensor(list(subset), dtype=torch.int64, device="cuda")


class DCPSE_scheme:
    """Linear system A x = b over the particles of ``parts`` with ``nvar``
    unknowns per particle (Sys_eqs::nvar); row and column of unknown v at
    particle p are p * nvar + v."""

    def __init__(self, parts, nvar=1):
        self.n = parts.size_local()
        self.nvar = int(nvar)
        self.N = self.n * self.nvar
        self.reset()

    def reset(self):
        self._rows, self._cols, self._vals = [], [], []
        self.b = torch.zeros(self.N, dtype=torch.float64, device="cuda")
        self.x_ig = None
        self._A = None

    def impose(self, op, subset, rhs, id=0):
        """Rows of ``op`` at the particles of ``subset`` with right-hand side
        ``rhs`` (a number, or a per-particle tensor read at the subset) as
        equation ``id`` (impose, DCPSE_Solver.hpp:600-790).  ``op`` is an
        operator with one output, IDENTITY, or a list of (coeff, op, var)
        terms summed into the same rows (value_nz of a sum expression)."""
        rows = _as_index(subset)
        terms = op if isinstance(op, list) else [(1.0, op, 0)]
        for coeff, o, var in terms:
            if o is IDENTITY or (isinstance(o, str) and o == IDENTITY):
                r = rows * self.nvar + id
                self._rows.append(r)
                self._cols.append(rows * self.nvar + var)
                self._vals.append(torch.full((rows.numel(),), float(coeff), dtype=torch.float64, device="cuda"))
                continue
            if o.plan.n_outputs != 1:
                raise ValueError("impose takes operators with one output (a component of a vector operator: "
                                 "pass a single-output operator)")
            rp, cols, vals = o.plan.operator_csr(0, coeff, rows=rows, nvar=self.nvar, var=var)
            counts = rp[1:] - rp[:-1]
            self._rows.append(torch.repeat_interleave(rows * self.nvar + id, counts))
            self._cols.append(cols)
            self._vals.append(vals)
        if isinstance(rhs, torch.Tensor):
            self.b[rows * self.nvar + id] = rhs.to(device="cuda", dtype=torch.float64)[rows]
        else:
            self.b[rows * self.nvar + id] = float(rhs)
        self._A = None

    def impose_x_ig(self, subset, value, id=0):
        """Initial guess of the solve (impose_x_ig)."""
        if self.x_ig is None:
            self.x_ig = torch.zeros(self.N, dtype=torch.float64, device="cuda")
        rows = _as_index(subset)
        if isinstance(value, torch.Tensor):
            self.x_ig[rows * self.nvar + id] = value.to(device="cuda", dtype=torch.float64)[rows]
        else:
            self.x_ig[rows * self.nvar + id] = float(value)

    def getA(self):
        """The assembled matrix (torch sparse CSR, duplicates summed)."""
        if self._A is None:
            r = torch.cat(self._rows) if self._rows else torch.zeros(0, dtype=torch.int64, device="cuda")
            c = torch.cat(self._cols) if self._cols else torch.zeros(0, dtype=torch.int64, device="cuda")
            v = torch.cat(self._vals) if self._vals else torch.zeros(0, dtype=torch.float64, device="cuda")
            coo = torch.sparse_coo_tensor(torch.stack([r, c]), v, (self.N, self.N)).coalesce()
            self._A = coo.to_sparse_csr()
        return self._A

    def getB(self):
        return self.b

    def solve(self, tol=1e-10, maxiter=20000):
        """Solve A x = b; returns x [n * nvar].  Raises if BiCGSTAB does not
        reach the relative residual tol."""
        A = self.getA()
        x, it, res = bicgstab(A, self.b, self.x_ig, tol=tol, maxiter=maxiter)
        if not (res <= tol):
            raise RuntimeError("BiCGSTAB stopped at relative residual %.3e after %d iterations" % (res, it))
        self.iterations, self.residual = it, res
        return x


def bicgstab(A, b, x0=None, tol=1e-10, maxiter=20000):
    """Jacobi-preconditioned BiCGSTAB (van der Vorst 1992) on the device.
    Returns (x, iterations, relative residual)."""
    d = _diagonal(A)
    dinv = torch.where(d != 0, 1.0 / d, torch.ones_like(d))
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    r = b - A @ x
    bn = torch.linalg.vector_norm(b).item() or 1.0
    rhat = r.clone()
    rho = alpha = omega = 1.0
    v = torch.zeros_like(b)
    p = torch.zeros_like(b)
    res = torch.linalg.vector_norm(r).item() / bn
    it = 0
    while res > tol and it < maxiter:
        it += 1
        rho_new = torch.dot(rhat, r).item()
        if rho_new == 0.0:
            break
        beta = (rho_new / rho) * (alpha / omega) if it > 1 else 0.0
        p = r + beta * (p - omega * v) if it > 1 else r.clone()
        ph = dinv * p
        v = A @ ph
        alpha = rho_new / torch.dot(rhat, v).item()
        s = r - alpha * v
        if torch.linalg.vector_norm(s).item() / bn <= tol:
            x = x + alpha * ph
            r = s
            res = torch.linalg.vector_norm(r).item() / bn
            break
        sh = dinv * s
        t = A @ sh
        tt = torch.dot(t, t).item()
        omega = torch.dot(t, s).item() / tt if tt != 0 else 0.0
        x = x + alpha * ph + omega * sh
        r = s - omega * t
        rho = rho_new
        res = torch.linalg.vector_norm(r).item() / bn
        if omega == 0.0:
            break
    return x, it, res


def _diagonal(A):
    rp = A.crow_indices()
    cols = A.col_indices()
    vals = A.values()
    n = rp.numel() - 1
    row = torch.repeat_interleave(torch.arange(n, device=vals.device), rp[1:] - rp[:-1])
    d = torch.zeros(n, dtype=vals.dtype, device=vals.device)
    m = cols == row
    d[row[m]] = vals[m]
    return d
