"""Cell-order renumbering of the apply's sliced layout.

A caller whose particles are not stored in spatial order (insertion order,
after a map(), a random shuffle) makes the apply's field gathers scatter
across memory.  The layout built at assembly then renumbers rows and columns
by the particles' cell order (the reference's GPU support builder walks
cells for the same reason, src/DCPSE/SupportBuilder.cuh:14-61).  Each row
keeps its entries and their order, so every result must equal the
caller-numbered layout's bit for bit, and outputs stay in the caller's
numbering.
"""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu

FLAGS = (C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32 | C.STORE_OUT_F32_RESID | C.STORE_OUT_F32_CORR)


def _plan(pos, h, policy, order=0):
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2)
    plan.set_reorder(policy)
    plan.set_reorder_order(order)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 2.8 * h)
    plan.assemble(pt, FLAGS)
    return plan


@pytest.fixture(scope="module")
def shuffled(cuda):
    pos, h = W.lattice(40, 3, jitter=0.15, seed=41)
    perm = np.random.default_rng(42).permutation(pos.shape[0])
    return np.ascontiguousarray(pos[perm]), h, perm


def test_shuffled_set_is_renumbered_and_bit_identical(shuffled):
    pos, h, _ = shuffled
    auto = _plan(pos, h, 0)
    keep = _plan(pos, h, -1)
    renum, d_list, d_cells = auto.reorder_info()
    assert renum and d_cells * 2 < d_list, (d_list, d_cells)
    assert not keep.reorder_info()[0]
    f = torch.tensor(W.field2(pos)[0], device="cuda")
    for prec in (C.F32, C.F32_RESID, C.F32_BUDGET, C.F32_PAIR, C.F64):
        a = auto.apply(f, prec).clone()
        b = keep.apply(f, prec).clone()
        assert torch.equal(a, b), prec
    for plan in (auto, keep):
        plan.set_error_budget(1e-7, C.F32_RESID)
    assert torch.equal(auto.apply(f, C.F32_BUDGET), keep.apply(f, C.F32_BUDGET))
    auto.close()
    keep.close()


def test_renumbering_orders_agree(shuffled):
    """The row-major renumbering (a grid at the mean spacing) gives the Z-order
    renumbering's outputs bit for bit: each row keeps its list order."""
    pos, h, _ = shuffled
    z = _plan(pos, h, 1, 0)
    r = _plan(pos, h, 1, 1)
    assert z.reorder_info()[0] and r.reorder_info()[0]
    f = torch.tensor(W.field2(pos)[0], device="cuda")
    for prec in (C.F32, C.F32_RESID, C.F64):
        assert torch.equal(z.apply(f, prec).clone(), r.apply(f, prec).clone()), prec
    z.close()
    r.close()


def test_shuffled_matches_ordered_set(shuffled):
    """The same particles in lattice order: every row lists its neighbours in
    another order, so the assembly's sums and the apply's sums run in
    another order too; equal within the FP64 assembly's order sensitivity
    (1e-10; boundary rows reach 1.2e-12) and the FP32 bar, not bit for bit."""
    pos, h, perm = shuffled
    ordered = np.empty_like(pos)
    ordered[perm] = pos
    a = _plan(pos, h, 0)
    b = _plan(ordered, h, 0)
    assert not b.reorder_info()[0]
    fa = torch.tensor(W.field2(pos)[0], device="cuda")
    fb = torch.tensor(W.field2(ordered)[0], device="cuda")
    ref = b.apply(fb, C.F64).cpu().numpy()
    for prec, tol in ((C.F64, 1e-10), (C.F32, 1e-6), (C.F32_BUDGET, 1e-6)):
        out = a.apply(fa, prec).cpu().numpy()
        for o in range(4):
            err = np.abs(out[o] - ref[o][perm]).max() / np.abs(ref[o]).max()
            assert err <= tol, (prec, o, err)
    a.close()
    b.close()


def test_renumbered_host_buffers(shuffled):
    pos, h, _ = shuffled
    plan = _plan(pos, h, 1)
    f_np = W.field2(pos)[0]
    dev = plan.apply(torch.tensor(f_np, device="cuda"), C.F32).cpu().numpy()
    hf = torch.empty(f_np.shape[0], dtype=torch.float64, pin_memory=True)
    hf.copy_(torch.from_numpy(f_np))
    hout = torch.empty(dev.shape, dtype=torch.float64, pin_memory=True)
    plan.apply_host(hf.numpy(), hout.numpy(), C.F32)
    assert np.array_equal(hout.numpy(), dev)
    # pageable buffers: row chunks in the caller's numbering (CSR kernels)
    page = plan.apply_host(f_np, precision=C.F32)
    scale = np.abs(dev).max(axis=1, keepdims=True)
    assert np.all(np.abs(page - dev) <= 1e-6 * scale)
    plan.close()


def test_renumbered_plan_keeps_list_order_paths(shuffled):
    """p2p on one set with the particle itself in its list, and applies after
    a change of policy, on a renumbered layout."""
    pos, h, _ = shuffled
    pt = torch.tensor(pos, device="cuda")
    plan = DcpsePlan(3, [[(0, 0, 0)]], order=2)
    plan.set_support(None, self_skip=False)
    plan.set_reorder(1)
    plan.build_neighbors(pt, 2.8 * h)
    plan.assemble(pt, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    f = torch.tensor(W.field2(pos)[0], device="cuda")
    ref = plan.p2p_f64(0, f).cpu().numpy()
    out = plan.p2p(f, C.F32).cpu().numpy()[0]
    assert np.abs(out - ref).max() <= 1e-6 * np.abs(ref).max()
    plan.close()
    grad = _plan(pos, h, 1)
    before = grad.apply(f, C.F32).clone()
    grad.set_reorder(-1)
    assert not grad.reorder_info()[0]
    assert torch.equal(grad.apply(f, C.F32), before)
    grad.close()
