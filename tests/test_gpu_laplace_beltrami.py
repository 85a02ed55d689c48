"""Laplace_Beltrami (DCPSE_surface_op.hpp:326-347): one SurfaceDcpse of
signature (2, 2, 2), whose basis at order 2 holds all 120 monomials of
degree <= 7 in 3D (7260 Gram entries).  Such bases take the assembly's large
path (the Gram sums continued through batch scratch, the column-pivoting QR
with its work space in global memory); the bar is the same as for the small
bases: neighbour lists, eps, eps^-|alpha|, status and the accumulated kernels
bit-exact with the oracle's pipeline on a small sphere.
"""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import operators as O
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu


def _sphere(n):
    """Fibonacci points with unit normals (DCPSE_op_Surface_tests.cpp:410-431)."""
    ga = np.pi * (3.0 - np.sqrt(5.0))
    i = np.arange(1, n)
    y = 1.0 - (i / (n - 1.0)) * 2.0
    r = np.sqrt(1 - y * y)
    x, z = np.cos(ga * i) * r, np.sin(ga * i) * r
    pos = np.stack([x, y, z], 1)
    return pos, pos / np.linalg.norm(pos, axis=1, keepdims=True)


def _setup(n=600, fac=4.0):
    pos, nrm = _sphere(n)
    h = np.sqrt(4 * np.pi / n)
    rcut = fac * h  # four layers of normal particles each side: 274-293 support points
    return pos, nrm, h, rcut, int(rcut / h)


def test_laplace_beltrami_sphere_bitexact(cuda, orc):
    pos, nrm, h, rcut, nc = _setup()
    sig = (2, 2, 2)
    plan = DcpsePlan(3, [[sig]], order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.set_surface(torch.tensor(nrm, device="cuda"), nc, h)
    plan.build_neighbors(pt, rcut)
    plan.assemble(pt, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    ext = orc.surface_extend(pos, nrm, nc, h)
    rp, cols = orc.neighbors(pos, rcut, support=ext, self_skip=True)
    eps_o, eip_o, K, st_o = orc.assemble(pos, rp, cols, sig, 2, support=ext, nthreads=8)
    rp2, c2, K2 = orc.surface_accumulate(rp, cols, [K], pos.shape[0], nc)
    grp, gcols = (x.cpu().numpy() for x in plan.neighbors())
    assert np.array_equal(grp, rp2) and np.array_equal(gcols, c2)
    assert np.diff(rp).min() >= 120  # every particle has enough support for the basis
    eps, st = (x.cpu().numpy() for x in plan.eps())
    assert np.array_equal(eps, eps_o) and np.array_equal(st, st_o) and np.all(st == 0)
    Kg, eip = (x.cpu().numpy() for x in plan.term_kernels(0))
    assert np.array_equal(eip, eip_o)
    np.testing.assert_array_equal(Kg, K2[0])
    # the FP32 weights follow the FP64 ones within their rounding: per row
    # at most 2^-22 sum_q |w_pq| |f_q - f_p| (the sixth-order weights cancel
    # strongly, so a bar relative to the output's scale would not hold)
    fn = np.sin(3 * pos[:, 0]) + pos[:, 1] * pos[:, 2]
    f = torch.tensor(fn, device="cuda")
    ref = plan.apply_output_f64(0, f).cpu().numpy()
    got = plan.apply(f, C.F32).cpu().numpy()[0]
    w = plan.output_weights(0)[0].cpu().numpy()
    row = np.repeat(np.arange(pos.shape[0]), np.diff(grp))
    bound = np.bincount(row, np.abs(w) * np.abs(fn[gcols] - fn[row]), minlength=pos.shape[0])
    assert np.all(np.abs(got - ref) <= 2.0 ** -22 * bound + 1e-12 * np.abs(ref).max())
    plan.close()


def test_laplace_beltrami_operator(cuda, orc):
    """The reference-facing operator class on a 400-point sphere: getV<1> =
    Laplace_Beltrami(getV<0>) against the oracle's accumulated kernels
    applied in the reference order, within 1e-12 of the output's scale."""
    pos, nrm, h, rcut, nc = _setup(400)
    parts = O.ParticleSet(pos)
    parts.props[2] = torch.tensor(nrm, device="cuda")  # normals
    vl = parts.getVerlet(rcut)
    LB = O.Laplace_Beltrami(parts, vl, 2, rcut, h, nc, normal=2)
    f = np.cos(2 * pos[:, 2]) * pos[:, 0]
    got = LB(torch.tensor(f, device="cuda")).cpu().numpy()
    ext = orc.surface_extend(pos, nrm, nc, h)
    rp, cols = orc.neighbors(pos, rcut, support=ext, self_skip=True)
    eps, eip, K, st = orc.assemble(pos, rp, cols, (2, 2, 2), 2, support=ext, nthreads=8)
    rp2, c2, K2 = orc.surface_accumulate(rp, cols, [K], pos.shape[0], nc)
    ref = orc.apply(f, rp2, c2, K2[0], eip, 6)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    LB.deallocate()
