"""Operator matrices for implicit solves (value_nz / DCPSE_scheme) on the GPU.

Bars: the CSR rows of dcpse_operator_csr equal the oracle's restatement of
value_nz + impose_git bit for bit (columns, values, row offsets); A f
reproduces the operator apply to 1e-12; the reference's Dirichlet Poisson
scenario (DCPSE_op_Solver_test.cpp:437-611) meets its bar worst < 0.03.
"""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import operators as O
from openfpm_numerics_gb300 import scheme as S
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["lap2d", "dx2d_self", "dz3d_rows", "lap3d_nvar"])
def test_operator_csr_bitexact(cuda, orc, case):
    if case.endswith("3d_rows") or case.endswith("3d_nvar"):
        pos, h = W.lattice(10, 3, jitter=0.15, seed=41)
        rcut = 2.8 * h
    else:
        pos, h = W.lattice(20, 2, jitter=0.15, seed=42)
        rcut = 3.1 * h
    dim = pos.shape[1]
    sigs = {"lap2d": [(2, 0), (0, 2)], "dx2d_self": [(1, 0)], "dz3d_rows": [(0, 0, 1)],
            "lap3d_nvar": [(2, 0, 0), (0, 2, 0), (0, 0, 2)]}[case]
    coeff = {"lap2d": 1.0, "dx2d_self": 2.5, "dz3d_rows": -0.75, "lap3d_nvar": 1.0}[case]
    nvar, var = (3, 1) if case == "lap3d_nvar" else (1, 0)
    plan = DcpsePlan(dim, [sigs], order=2)
    pt = torch.tensor(pos, device="cuda")
    if case == "dx2d_self":
        plan.set_support(None, self_skip=False)
    plan.build_neighbors(pt, rcut)
    plan.assemble(pt, C.STORE_TERMS_F64 | C.STORE_OUT_F64)
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    rows = None
    if case == "dz3d_rows":
        rows = np.random.default_rng(43).permutation(pos.shape[0])[:200]
    terms = [orc.assemble(pos, rp, cols, s, 2) for s in sigs]
    R, Cc, V = orc.operator_csr(rp, cols, [t[2] for t in terms], [t[1] for t in terms], [sum(s) for s in sigs],
                                coeff=coeff, rows=rows, nvar=nvar, var=var)
    rt = None if rows is None else torch.tensor(rows, device="cuda")
    gr, gc, gv = (x.cpu().numpy() for x in plan.operator_csr(0, coeff, rows=rt, nvar=nvar, var=var))
    assert np.array_equal(gr, R) and np.array_equal(gc, Cc) and np.array_equal(gv, V)
    if rows is None and nvar == 1:
        # A f equals the apply of the operator (sign and diagonal conventions)
        import scipy.sparse as sp

        A = sp.csr_matrix((gv, gc, gr), shape=(pos.shape[0], pos.shape[0]))
        f = np.sin(3 * pos[:, 0]) + pos[:, 1] ** 2
        ref = plan.apply_output_f64(0, torch.tensor(f, device="cuda")).cpu().numpy() * coeff
        assert np.abs(A @ f - ref).max() <= 1e-12 * np.abs(ref).max()
    plan.close()


def test_poisson_dirichlet_reference_scenario(cuda):
    """DCPSE_op_Solver_test.cpp:437-611: 81^2 lattice on [0,1]^2, rCut 3.1h,
    Lap(v) = -2 pi^2 sin(pi x) sin(pi y) in the bulk, v = the same analytic
    solution sin(pi x) sin(pi y) (zero) on the four edges; worst < 0.03."""
    nside = 81
    h = 1.0 / (nside - 1)
    pos, _ = W.lattice(nside, 2, h=h)
    parts = O.ParticleSet(pos)
    vl = parts.getVerlet(3.1 * h)
    Lap = O.Laplacian(parts, vl, 2, 3.1 * h)
    x, y = pos[:, 0], pos[:, 1]
    edge = (x < h / 2) | (x > 1 - h / 2) | (y < h / 2) | (y > 1 - h / 2)
    bulk = np.where(~edge)[0]
    bnd = np.where(edge)[0]
    rhs = torch.tensor(-2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y), device="cuda")
    exact = np.sin(np.pi * x) * np.sin(np.pi * y)
    solver = S.DCPSE_scheme(parts)
    solver.impose(Lap, bulk, rhs)
    solver.impose(S.IDENTITY, bnd, torch.tensor(exact, device="cuda"))
    sol = solver.solve(tol=1e-10).cpu().numpy()
    assert np.abs(sol - exact).max() < 0.03
    # the assembled matrix has the imposed structure
    A = solver.getA()
    assert A.shape == (nside * nside, nside * nside)
    Lap.deallocate()


def test_scheme_two_unknowns(cuda):
    """Two coupled unknowns per particle (Sys_eqs::nvar = 2): u - Lap(w) = a,
    w = b; rows and columns interleave as p * nvar + var."""
    nside = 24
    h = 1.0 / (nside - 1)
    pos, _ = W.lattice(nside, 2, h=h)
    parts = O.ParticleSet(pos)
    vl = parts.getVerlet(3.1 * h)
    Lap = O.Laplacian(parts, vl, 2, 3.1 * h)
    n = pos.shape[0]
    wv = np.cos(pos[:, 0]) * pos[:, 1]
    lapw = Lap(torch.tensor(wv, device="cuda")).cpu().numpy()
    a = torch.tensor(1.0 + pos[:, 0] - lapw, device="cuda")
    solver = S.DCPSE_scheme(parts, nvar=2)
    allp = np.arange(n)
    solver.impose([(1.0, S.IDENTITY, 0), (-1.0, Lap, 1)], allp, a, id=0)
    solver.impose([(1.0, S.IDENTITY, 1)], allp, torch.tensor(wv, device="cuda"), id=1)
    x = solver.solve(tol=1e-12).cpu().numpy()
    assert np.abs(x[1::2] - wv).max() < 1e-9
    assert np.abs(x[0::2] - (1.0 + pos[:, 0])).max() < 1e-8
    Lap.deallocate()
