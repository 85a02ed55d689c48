"""The sliced kernels' two schedules: warps taking one slice at a time from a
counter (DCPSE_APPLY_SLICE_WARPS) and one window of 8 slices per block
(DCPSE_APPLY_SLICE_WINDOWS).  A row is summed by one thread in the same
order either way, so the outputs are bit-identical: on a graded cloud (rows
of 5 to 50 entries, renumbered by cell order), on a lattice in caller order,
for every FP32 precision and for interpolation (p2p)."""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu

FLAGS = C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.STORE_OUT_F64 | C.STORE_OUT_F32_RESID | C.STORE_OUT_F32_CORR


def _both(plan, f, prec):
    plan.set_apply_config(0, C.APPLY_SLICE_WARPS)
    a = plan.apply(f, prec).clone()
    plan.set_apply_config(0, C.APPLY_SLICE_WINDOWS)
    b = plan.apply(f, prec).clone()
    plan.set_apply_config(0, 0)
    return a, b


@pytest.mark.parametrize("prec", [C.F32, C.F32_RESID, C.F32_PAIR])
def test_graded_cloud_schedules_agree(cuda, prec):
    cfg = W.config3(60_000, seed=11)
    pos = torch.tensor(cfg["pos"], device="cuda")
    plan = DcpsePlan(2, W.five_ops_2d(), order=2)
    plan.set_reorder(1)
    plan.build_neighbors(pos, 0.0, torch.tensor(cfg["rcut_pp"], device="cuda"))
    plan.assemble(pos, FLAGS)
    k = np.diff(plan.neighbors()[0].cpu().numpy())
    assert k.max() >= 2 * k.min()  # uneven rows: the slices of a window differ in length
    x, y = cfg["pos"][:, 0], cfg["pos"][:, 1]
    f = torch.tensor(np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y), device="cuda")
    a, b = _both(plan, f, prec)
    assert torch.equal(a, b)
    # a second call reuses the counter
    assert torch.equal(plan.apply(f, prec), a)
    plan.close()


def test_lattice_and_p2p_schedules_agree(cuda):
    pos_np, h = W.lattice(30, 3, jitter=0.15, seed=12)
    pos = torch.tensor(pos_np, device="cuda")
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2)
    plan.set_reorder(-1)
    plan.build_neighbors(pos, 2.8 * h)
    plan.assemble(pos, FLAGS)
    f = torch.tensor(W.field2(pos_np)[0], device="cuda")
    for prec in (C.F32, C.F32_PAIR):
        a, b = _both(plan, f, prec)
        assert torch.equal(a, b), prec
    plan.close()
    # interpolation from a lattice onto a jittered copy of it
    tgt_np, _ = W.lattice(20, 3, h=1.0 / 19, jitter=0.3, seed=13)
    sup_np, hs = W.lattice(24, 3, jitter=0.1, seed=14)
    ip = DcpsePlan(3, [[(0, 0, 0)]], order=2)
    ip.set_support(torch.tensor(sup_np, device="cuda"))
    tgt = torch.tensor(tgt_np, device="cuda")
    ip.build_neighbors(tgt, 2.8 * hs)
    ip.assemble(tgt, C.STORE_TERMS_F64 | C.STORE_OUT_F32)
    fs = torch.tensor(np.cos(3 * sup_np[:, 0]) * sup_np[:, 1], device="cuda")
    ip.set_apply_config(0, C.APPLY_SLICE_WARPS)
    a = ip.p2p(fs, C.F32).clone()
    ip.set_apply_config(0, C.APPLY_SLICE_WINDOWS)
    b = ip.p2p(fs, C.F32).clone()
    assert torch.equal(a, b)
    ip.close()


@pytest.mark.parametrize("first", [C.F32, C.F32_RESID])
def test_budget_pass_schedules_agree(cuda, first):
    """The error-budget apply's bound pass under both schedules: the same
    outputs, bounds and maxima, so the same rows corrected."""
    cfg = W.config3(60_000, seed=15)
    pos = torch.tensor(cfg["pos"], device="cuda")
    plan = DcpsePlan(2, W.five_ops_2d(), order=2)
    plan.build_neighbors(pos, 0.0, torch.tensor(cfg["rcut_pp"], device="cuda"))
    plan.assemble(pos, FLAGS)
    plan.set_error_budget(1e-7, first)
    x, y = cfg["pos"][:, 0], cfg["pos"][:, 1]
    f = torch.tensor(np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y), device="cuda")
    res = []
    for mode in (C.APPLY_SLICE_WARPS, C.APPLY_SLICE_WINDOWS):
        plan.set_apply_config(0, mode)
        plan.budget_stats(reset=True)
        out = plan.apply(f, C.F32_BUDGET).clone()
        res.append((out, plan.budget_stats()))
    assert torch.equal(res[0][0], res[1][0])
    assert res[0][1] == res[1][1]
    if first == C.F32:
        assert res[0][1] > 0  # FP32 bounds exceed the budget on some rows of this cloud
    plan.close()


@pytest.mark.parametrize("prec", [C.F64, C.F32])
@pytest.mark.parametrize("cloud", ["lattice", "graded"])
def test_field_vjp_sliced_equals_csr(cuda, prec, cloud):
    """The field VJP on the sliced layout of the transposed list sums each
    row in the CSR kernel's order: bit-identical results, on a lattice and on
    a graded cloud, with FP64 and FP32 weights; a new assembly replaces the
    layout's weights."""
    if cloud == "lattice":
        pos_np, h = W.lattice(24, 3, jitter=0.15, seed=16)
        outputs, dim = W.grad_lap_outputs(3), 3
        build = lambda plan, pos: plan.build_neighbors(pos, 2.8 * h)
    else:
        cfg = W.config3(40_000, seed=17)
        pos_np, outputs, dim = cfg["pos"], W.five_ops_2d(), 2
        rpp = torch.tensor(cfg["rcut_pp"], device="cuda")
        build = lambda plan, pos: plan.build_neighbors(pos, 0.0, rpp)
    pos = torch.tensor(pos_np, device="cuda")
    plan = DcpsePlan(dim, outputs, order=2)
    build(plan, pos)
    plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    g = torch.tensor(np.random.default_rng(18).standard_normal((len(outputs), pos_np.shape[0])), device="cuda")
    plan.set_apply_config(0, 0)
    a = plan.vjp_field(g, prec).clone()
    plan.set_apply_config(0, 1)  # CSR schedule: the thread-per-row CSR kernel
    b = plan.vjp_field(g, prec).clone()
    assert torch.equal(a, b)
    # the weights change with a new assembly: the layout follows
    plan.assemble(pos, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    plan.set_apply_config(0, 0)
    a2 = plan.vjp_field(g, prec).clone()
    plan.set_apply_config(0, 1)
    assert torch.equal(a2, plan.vjp_field(g, prec))
    if prec == C.F64:  # (the two assemblies' FP32 weights can round alike)
        assert not torch.equal(a2, a)
    # and equal a fresh plan's (row sums and transposed weights are rebuilt)
    fresh = DcpsePlan(dim, outputs, order=2)
    build(fresh, pos)
    fresh.assemble(pos, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    assert torch.equal(a2, fresh.vjp_field(g, prec))
    fresh.close()
    plan.close()
