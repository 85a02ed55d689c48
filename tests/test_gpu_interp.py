"""Particle to particle interpolation (PPInterpolation / Dcpse::p2p) on the
GPU against the CPU oracle.

Bars: two-set neighbour lists, eps, eps^-|alpha|, kernels and the
reference-order p2p (scalar and vector fields) are bit-exact; the batched
p2p from summed weights is within 1e-12 (FP64) and 1e-6 (FP32) of it,
relative to max |f|; the reference's own scenarios
(DCPSE_op_test_base_tests.cpp:245-385) keep their bar worst < 0.03.
"""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import operators as O
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu


def _two_sets(nside=24, seed=21, dim=2, jitter=0.2, nsup_extra=0):
    dom, h = W.lattice(nside, dim)
    rng = np.random.default_rng(seed)
    sup = dom + rng.uniform(-jitter * h, jitter * h, dom.shape)
    if nsup_extra:
        sup = np.concatenate([sup, rng.uniform(0, 1, (nsup_extra, dim))])
    return dom, sup, h


@pytest.mark.parametrize("dim,nside,extra", [(2, 24, 0), (2, 20, 150), (3, 10, 40)])
def test_two_set_assembly_and_p2p_bitexact(cuda, orc, dim, nside, extra):
    dom, sup, h = _two_sets(nside, 21 + dim, dim, nsup_extra=extra)
    rcut = (3.1 if dim == 2 else 2.8) * h
    zero = (0,) * dim
    plan = DcpsePlan(dim, [[zero]], order=2)
    dt = torch.tensor(dom, device="cuda")
    st_ = torch.tensor(sup, device="cuda")
    plan.set_support(st_)
    plan.build_neighbors(dt, rcut)
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    rp_o, cols_o = orc.neighbors(dom, rcut, support=sup, self_skip=False)
    assert np.array_equal(rp, rp_o) and np.array_equal(cols, cols_o)
    assert cols.max() >= dom.shape[0] or extra == 0  # columns index the support set
    plan.assemble(dt, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    eps_o, eip_o, K_o, st_o = orc.assemble(dom, rp, cols, zero, 2, support=sup)
    eps, st = (x.cpu().numpy() for x in plan.eps())
    K, eip = (x.cpu().numpy() for x in plan.term_kernels(0))
    assert np.array_equal(st, st_o)
    assert np.array_equal(eps, eps_o) and np.array_equal(eip, eip_o) and np.array_equal(K, K_o)
    f = np.sin(3 * sup[:, 0]) + np.cos(2 * sup[:, 1])
    fv = np.stack([f, sup[:, 0] ** 2, -sup[:, 1]], 1)
    g = plan.p2p_f64(0, torch.tensor(f, device="cuda")).cpu().numpy()
    assert np.array_equal(g, orc.p2p(f, rp, cols, K_o, eip_o))
    gv = plan.p2p_f64(0, torch.tensor(fv, device="cuda")).cpu().numpy()
    assert np.array_equal(gv, orc.p2p(fv, rp, cols, K_o, eip_o))
    ok = st == 0
    for prec, bar in ((C.F64, 1e-12), (C.F32, 1e-6)):
        b = plan.p2p(torch.tensor(f, device="cuda"), prec)[0].cpu().numpy()
        assert np.abs(b - g)[ok].max() <= bar * np.abs(f).max(), prec
        bv = plan.p2p(torch.tensor(fv, device="cuda"), prec)[0].cpu().numpy()
        assert np.abs(bv - gv)[ok].max() <= bar * np.abs(fv).max(), prec
    # linear fields are reproduced (order 2 moment conditions)
    lin = 0.3 + 2.0 * sup[:, 0] - sup[:, -1]
    gl = plan.p2p_f64(0, torch.tensor(lin, device="cuda")).cpu().numpy()
    assert np.abs(gl - (0.3 + 2.0 * dom[:, 0] - dom[:, -1]))[ok].max() < 1e-10
    # derivative applies need one set
    with pytest.raises(C.DcpseError) as e:
        plan.apply(torch.zeros(dom.shape[0], dtype=torch.float64, device="cuda"), C.F32)
    assert e.value.code == C.ERR_STATE
    plan.close()


def test_self_included_list(cuda, orc):
    """One set with the particle in its own list (getVerlet<VL_NON_SYMMETRIC>)."""
    pos, h = W.lattice(20, 2, jitter=0.1, seed=31)
    plan = DcpsePlan(2, [[(0, 0)], [(1, 0)], [(2, 0), (0, 2)]], order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.set_support(None, self_skip=False)
    plan.build_neighbors(pt, 3.1 * h)
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    rp_o, cols_o = orc.neighbors(pos, 3.1 * h, self_skip=False)
    assert np.array_equal(rp, rp_o) and np.array_equal(cols, cols_o)
    assert all(p in cols[rp[p]:rp[p + 1]] for p in range(0, pos.shape[0], 37))
    plan.assemble(pt, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    f = np.cos(4 * pos[:, 0]) * pos[:, 1]
    ft = torch.tensor(f, device="cuda")
    for t, s in enumerate([(0, 0), (1, 0), (2, 0), (0, 2)]):
        eps_o, eip_o, K_o, _ = orc.assemble(pos, rp, cols, s, 2)
        K, eip = (x.cpu().numpy() for x in plan.term_kernels(t))
        assert np.array_equal(K, K_o) and np.array_equal(eip, eip_o)
        if t == 0:
            assert np.array_equal(plan.p2p_f64(0, ft).cpu().numpy(), orc.p2p(f, rp, cols, K_o, eip_o))
        ref = orc.apply(f, rp, cols, K_o, eip_o, sum(s))
        assert np.array_equal(plan.apply_term_f64(t, ft).cpu().numpy(), ref)
    plan.close()


def _sin_field(pos):
    return np.sin(pos[:, 0]) + np.sin(pos[:, 1])


def test_ppinterpolation_reference_scenarios(cuda, orc):
    """DCPSE_op_test_base_tests.cpp:245-300 (one set, VL_NON_SYMMETRIC list,
    rCut 4.1h) and :302-385 (jittered copy onto the lattice, rCut 3.9h):
    worst |p2p(f) - f| < 0.03 for f = sin x + sin y on 80^2 over [0, 2 pi]^2."""
    nside = 80
    h = 2 * np.pi / (nside - 1)
    pos, _ = W.lattice(nside, 2, h=h)
    dom = O.ParticleSet(pos)
    dom.props[0] = torch.tensor(_sin_field(pos), device="cuda")
    vl = dom.getVerlet(4.1 * h, opt=O.VL_NON_SYMMETRIC)
    Fx = O.PPInterpolation(dom, dom, vl, 2, 4.1 * h)
    Fx.p2p(0, 1)
    assert (dom.props[1] - dom.props[0]).abs().max().item() < 0.03
    Fx.deallocate()

    rng = np.random.default_rng(6666666)
    spos = pos.copy()
    inner = (pos[:, 0] != 0) & (pos[:, 1] != 0) & (pos[:, 0] != pos[:, 0].max()) & (pos[:, 1] != pos[:, 1].max())
    spos[inner] += rng.normal(0.0, h * h / 4, (inner.sum(), 2))
    sup = O.ParticleSet(spos)
    sup.props[0] = torch.tensor(_sin_field(spos), device="cuda")
    sup.props[4] = torch.tensor(np.stack([np.sin(spos[:, 0]), np.cos(spos[:, 1])], 1), device="cuda")
    vl2 = O.createVerletTwoPhase(dom, sup, 3.9 * h)
    Fx2 = O.PPInterpolation(sup, dom, vl2, 2, 3.9 * h)
    Fx2.p2p(0, 1)
    assert (dom.props[1] - dom.props[0]).abs().max().item() < 0.03
    Fx2.p2p(4, 5, N1=2)
    exact = torch.tensor(np.stack([np.sin(pos[:, 0]), np.cos(pos[:, 1])], 1), device="cuda")
    assert (dom.props[5] - exact).abs().max().item() < 0.03
    # the operator equals the oracle's on the same lists
    rp, cols = vl2.rowptr.cpu().numpy(), vl2.cols.cpu().numpy()
    _, eip_o, K_o, _ = orc.assemble(pos, rp, cols, (0, 0), 2, support=spos)
    assert np.array_equal(dom.props[1].cpu().numpy(), orc.p2p(_sin_field(spos), rp, cols, K_o, eip_o))
    f32 = Fx2(sup.props[0], precision="f32")
    assert (f32 - dom.props[1]).abs().max().item() <= 1e-6 * 2
    Fx2.deallocate()


def test_p2p_support_smaller_than_domain(cuda, orc):
    """Interpolation from a coarse support set onto a finer domain set (more
    rows than support particles): the FP32 p2p on the sliced layout pads rows
    with support indices (never a row index), equals the reference-order p2p
    within 1e-6 and reproduces linear fields."""
    dom, h = W.lattice(40, 2)
    sup, hs = W.lattice(18, 2, jitter=0.1, seed=77)
    rcut = 3.1 * hs
    plan = DcpsePlan(2, [[(0, 0)]], order=2)
    plan.set_support(torch.tensor(sup, device="cuda"))
    dt = torch.tensor(dom, device="cuda")
    plan.build_neighbors(dt, rcut)
    plan.assemble(dt, C.STORE_TERMS_F64 | C.STORE_OUT_F32)
    assert dom.shape[0] > sup.shape[0]
    f = np.sin(2 * sup[:, 0]) + sup[:, 1] ** 2
    ft = torch.tensor(f, device="cuda")
    ref = plan.p2p_f64(0, ft).cpu().numpy()
    got = plan.p2p(ft, C.F32)[0].cpu().numpy()
    st = plan.eps()[1].cpu().numpy()
    ok = st == 0
    assert ok.sum() > 0.9 * dom.shape[0]
    assert np.abs(got - ref)[ok].max() <= 1e-6 * np.abs(f).max()
    lin = 0.5 + sup[:, 0] - 2 * sup[:, 1]
    gl = plan.p2p(torch.tensor(lin, device="cuda"), C.F32)[0].cpu().numpy()
    assert np.abs(gl - (0.5 + dom[:, 0] - 2 * dom[:, 1]))[ok].max() < 1e-5
    plan.check()
    plan.close()
