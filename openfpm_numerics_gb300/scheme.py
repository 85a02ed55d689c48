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


def bicgstab(A, b, x0=None, tol=1e-10, maxiter=20000, check_every=16):
    """Jacobi-preconditioned BiCGSTAB (van der Vorst 1992) on the device.
    Returns (x, iterations, relative residual).

    The scalars stay on the device: the host reads the residual and a
    breakdown flag once every `check_every` iterations (one synchronisation
    instead of six per iteration), so up to check_every - 1 iterations run
    past convergence, each only reducing the residual further.  A breakdown
    (rho = 0 or omega = 0) freezes the iterate, and the next check stops."""
    d = _diagonal(A)
    dinv = torch.where(d != 0, 1.0 / d, torch.ones_like(d))
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    r = b - A @ x
    bn = torch.linalg.vector_norm(b)
    bn = torch.where(bn > 0, bn, torch.ones_like(bn))
    res = float((torch.linalg.vector_norm(r) / bn).item())
    if not (res > tol) or maxiter <= 0:
        return x, 0, res
    rhat = r.clone()
    zero = torch.zeros((), dtype=b.dtype, device=b.device)
    rho = alpha = omega = torch.ones((), dtype=b.dtype, device=b.device)
    v = torch.zeros_like(b)
    p = torch.zeros_like(b)
    live = torch.ones((), dtype=torch.bool, device=b.device)  # no breakdown yet

    def safe_div(num, den):
        ok = den != 0
        return torch.where(ok, num / torch.where(ok, den, torch.ones_like(den)), zero), ok

    it = 0
    while it < maxiter:
        for _ in range(min(check_every, maxiter - it)):
            it += 1
            rho_new = torch.dot(rhat, r)
            live = live & (rho_new != 0)
            if it == 1:
                p = r.clone()
            else:
                q1, _ = safe_div(rho_new, rho)
                q2, _ = safe_div(alpha, omega)
                p = r + (q1 * q2) * (p - omega * v)
            ph = dinv * p
            v = A @ ph
            alpha_n, ok_a = safe_div(rho_new, torch.dot(rhat, v))
            live = live & ok_a
            a_ = torch.where(live, alpha_n, zero)
            s = r - a_ * v
            sh = dinv * s
            t = A @ sh
            omega_n, _ = safe_div(torch.dot(t, s), torch.dot(t, t))
            o_ = torch.where(live, omega_n, zero)
            x = x + a_ * ph + o_ * sh
            r = s - o_ * t
            live = live & (omega_n != 0)
            rho = torch.where(live, rho_new, rho)
            alpha = torch.where(live, alpha_n, alpha)
            omega = torch.where(live, omega_n, omega)
        state = torch.stack([torch.linalg.vector_norm(r) / bn, live.to(b.dtype)]).cpu()
        res = float(state[0])
        if not (res > tol) or state[1] == 0:
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
