"""Surface DC-PSE (SurfaceDcpse, the surface operators and surface
interpolation) on the GPU against the oracle and the reference's own
scenarios (DCPSE_op_Surface_tests.cpp).

Bars: the accumulated neighbour lists, eps, eps^-|alpha| and kernels are
bit-exact with the oracle pipeline (extension, two-set lists, assembly,
accumulation); the circle and sphere scenarios keep worst < 0.03.
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


@pytest.mark.parametrize("case", ["circle", "sphere"])
def test_surface_plan_bitexact(cuda, orc, case):
    if case == "circle":
        n, h = 256, 3.0 / 255
        th = np.arange(n) * (2 * np.pi / n)
        pos = np.stack([np.cos(th), np.sin(th)], 1)
        nrm = pos.copy()
        rcut, sigs = 5.1 * h, [(2, 0), (0, 2), (1, 0)]
    else:
        pos, nrm = _sphere(1500)
        h = np.sqrt(4 * np.pi / 1500)
        rcut, sigs = 2.5 * h, [(2, 0, 0), (0, 2, 0), (0, 0, 2)]
    nc = int(rcut / h)
    dim = pos.shape[1]
    plan = DcpsePlan(dim, [[s] for s in sigs], order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.set_surface(torch.tensor(nrm, device="cuda"), nc, h)
    plan.build_neighbors(pt, rcut)
    plan.assemble(pt, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    ext = orc.surface_extend(pos, nrm, nc, h)
    rp, cols = orc.neighbors(pos, rcut, support=ext, self_skip=True)
    terms = [orc.assemble(pos, rp, cols, s, 2, support=ext) for s in sigs]
    rp2, c2, K2 = orc.surface_accumulate(rp, cols, [t[2] for t in terms], pos.shape[0], nc)
    grp, gcols = (x.cpu().numpy() for x in plan.neighbors())
    assert np.array_equal(grp, rp2) and np.array_equal(gcols, c2)
    eps, st = (x.cpu().numpy() for x in plan.eps())
    assert np.array_equal(eps, terms[0][0]) and np.all(st == 0)
    for t in range(len(sigs)):
        K, eip = (x.cpu().numpy() for x in plan.term_kernels(t))
        assert np.array_equal(K, K2[t]) and np.array_equal(eip, terms[t][1])
    # FP32 weights follow from the accumulated FP64 weights
    f = torch.tensor(np.sin(3 * pos[:, 0]) + pos[:, 1], device="cuda")
    ref = torch.stack([plan.apply_output_f64(o, f) for o in range(len(sigs))]).cpu().numpy()
    got = plan.apply(f, C.F32).cpu().numpy()
    for o in range(len(sigs)):
        assert np.abs(got[o] - ref[o]).max() <= 1e-6 * np.abs(ref[o]).max()
    # a second assembly needs a new neighbour build
    with pytest.raises(C.DcpseError):
        plan.assemble(pt, C.STORE_TERMS_F64)
    plan.close()


def test_surface_circle_reference_scenario(cuda):
    """DCPSE_op_Surface_tests.cpp:97-182: SDxx + SDyy of sin(theta) on 512
    particles of the unit circle, worst < 0.03."""
    n, h = 512, 3.0 / 511
    rcut = 5.1 * h
    th = np.arange(n) * (2 * np.pi / n)
    pos = np.stack([np.cos(th), np.sin(th)], 1)
    parts = O.ParticleSet(pos)
    parts.props[2] = torch.tensor(pos, device="cuda")      # normals
    parts.props[3] = torch.tensor(np.sin(th), device="cuda")
    vl = parts.getVerlet(rcut)
    nc = int(rcut / h)
    SDxx = O.SurfaceDerivative_xx(parts, vl, 2, rcut, h, nc, normal=2)
    vl2 = parts.getVerlet(rcut)
    SDyy = O.SurfaceDerivative_yy(parts, vl2, 2, rcut, h, nc, normal=2)
    out = SDxx(parts.props[3]) + SDyy(parts.props[3])
    assert (out + parts.props[3]).abs().max().item() < 0.03
    # the operator replaced the Verlet list with the accumulated one
    assert int(vl.rowptr[-1]) == SDxx.plan.info()["nnz"]
    for op in (SDxx, SDyy):
        op.deallocate()


def test_surface_sphere_reference_scenario(cuda):
    """DCPSE_op_Surface_tests.cpp:390-508: Sdxx + Sdyy + Sdzz of the spherical
    harmonic Y_1^0 on 40960 Fibonacci points, rCut = 2.5 h, nCount = 2:
    -2 Y_1^0 within worst < 0.03."""
    n = 40960
    pos, nrm = _sphere(n)
    h = np.sqrt(4 * np.pi / n)
    rcut = 2.5 * h
    parts = O.ParticleSet(pos)
    parts.props[2] = torch.tensor(nrm, device="cuda")
    y10 = 0.5 * np.sqrt(3 / np.pi) * pos[:, 2]
    f = torch.tensor(y10, device="cuda")
    ops = []
    for cls in (O.SurfaceDerivative_xx, O.SurfaceDerivative_yy, O.SurfaceDerivative_zz):
        ops.append(cls(parts, parts.getVerlet(rcut), 2, rcut, h, int(rcut / h), normal=2))
    out = sum(op(f) for op in ops)
    assert (out + 2 * f).abs().max().item() < 0.03
    for op in ops:
        op.deallocate()


def test_surface_interpolation_sphere(cuda, orc):
    """DCPSE_op_Surface_tests.cpp:1461-1646 (smaller sets): surface p2p of the
    spherical harmonic 0.25 sqrt(105/pi) (x^2 - y^2) z, order 5, from 4096
    Fibonacci points onto 256, rCut = 3.5 h_from, worst < 0.03; bit-exact
    with the oracle pipeline."""
    nf, nt = 4096, 256
    pf, nrm = _sphere(nf + 1)
    pt_, _ = _sphere(nt)
    h = np.sqrt(4 * np.pi / nf)
    rcut = 3.5 * h

    def Y(p):
        return 0.25 * np.sqrt(105 / np.pi) * (p[:, 0] ** 2 - p[:, 1] ** 2) * p[:, 2]

    sup = O.ParticleSet(pf)
    sup.props[0] = torch.tensor(Y(pf), device="cuda")
    sup.props[1] = torch.tensor(nrm, device="cuda")
    dom = O.ParticleSet(pt_)
    vl = O.createVerletTwoPhase(dom, sup, rcut)
    pp = O.PPInterpolation(sup, dom, vl, 5, rcut, nSpacing=h, isSurfaceInterpolation=True, normal=1)
    pp.p2p(0, 0)
    assert (dom.props[0] - torch.tensor(Y(pt_), device="cuda")).abs().max().item() < 0.03
    nc = int(rcut / h)
    ext = orc.surface_extend(pf, nrm, nc, h)
    rp, cols = orc.neighbors(pt_, rcut, support=ext, self_skip=False)
    eps, eip, K, st = orc.assemble(pt_, rp, cols, (0, 0, 0), 5, support=ext)
    rp2, c2, K2 = orc.surface_accumulate(rp, cols, [K], pf.shape[0], nc)
    ref = orc.p2p(Y(pf), rp2, c2, K2[0], eip)
    assert np.array_equal(dom.props[0].cpu().numpy(), ref)
    pp.deallocate()


def test_surface_adaptive_equals_regular_sphere(cuda):
    """DCPSE_op_Surface_tests.cpp:756-900 (dcpse_surface_adaptive_unitSphere):
    Laplace-Beltrami of Y_2^0 on 2000 Fibonacci points with a regular list
    (rCut = 2 h, nSpacing = h, nCount = 2) and with support_options.ADAPTIVE
    (cutoff 2 h per particle in property 0, spacing = property 0 / nCount);
    the reference requires equal L2 and Linf errors within 0.001 %."""
    n = 2000
    h = np.sqrt(4 * np.pi / n)
    ga = np.pi * (3.0 - np.sqrt(5.0))
    i = np.arange(n)
    y = 1.0 - 2.0 * (i / (n - 1.0))
    rad = np.sqrt(1.0 - y * y)
    x, z = np.cos(ga * i) * rad, np.sin(ga * i) * rad
    tb, ph = np.arctan2(np.sqrt(x * x + y * y), z), np.arctan2(y, x)
    pos = np.stack([x, y, z], 1)
    nrm = np.stack([np.sin(tb) * np.cos(ph), np.sin(tb) * np.sin(ph), np.cos(tb)], 1)
    y20 = 0.25 * np.sqrt(5 / np.pi) * (3 * np.cos(tb) ** 2 - 1)
    parts = O.ParticleSet(pos)
    parts.props[0] = torch.full((n,), 2 * h, dtype=torch.float64, device="cuda")
    parts.props[1] = torch.tensor(nrm, device="cuda")
    f = torch.tensor(y20, device="cuda")
    vreg = parts.getVerlet(2 * h)
    vad = O.VerletList(parts, 0.0, rcut_pp=parts.props[0])
    classes = (O.SurfaceDerivative_xx, O.SurfaceDerivative_yy, O.SurfaceDerivative_zz)
    lap_r = sum(c(parts, vreg, 2, 0.0, h, 2, normal=1)(f) for c in classes).cpu().numpy()
    lap_a = sum(c(parts, vad, 2, 0.0, 0.0, 2, O.support_options.ADAPTIVE, normal=1)(f) for c in classes).cpu().numpy()
    er, ea = np.abs(lap_r + 6 * y20), np.abs(lap_a + 6 * y20)
    l2r, l2a = np.sqrt((er ** 2).mean()), np.sqrt((ea ** 2).mean())
    assert abs(l2r - l2a) <= 1e-5 * l2r and abs(er.max() - ea.max()) <= 1e-5 * er.max()
