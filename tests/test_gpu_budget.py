"""Budget-driven FP32 apply (DCPSE_F32_BUDGET): FP32 weights with an FP64
residual correction of exactly the rows whose FP32 error bound exceeds the
budget.  Every output of every call must stay within the budget of the FP64
summed-weight apply (normwise: max|a - b| <= eps max|b|), on a graded cloud
where the plain FP32 apply does not, for either first pass (FP32 alone or
with the bf16 residual streams), for the CSR fallback that corrects every
row, and through the host-buffer entry point.  The weights' reference apply
is src/DCPSE/Dcpse.hpp:467-499; graded supports as in Dcpse.hpp:903-909.
"""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu


def normwise(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _graded(n, flags):
    cfg = W.config3(n=n, seed=13)
    pos = torch.tensor(cfg["pos"], device="cuda")
    plan = DcpsePlan(2, W.five_ops_2d(), order=2)
    plan.build_neighbors(pos, 0.0, torch.tensor(cfg["rcut_pp"], device="cuda"))
    plan.assemble(pos, flags)
    return plan, cfg["pos"]


def _fields(pos):
    x, y = pos[:, 0], pos[:, 1]
    return {
        "sin_cos": np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y),
        "gauss": np.exp(-20 * ((x - 0.4) ** 2 + (y - 0.6) ** 2)) + 3.0,
    }


@pytest.fixture(scope="module")
def graded_plan(cuda):
    flags = C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32 | C.STORE_OUT_F32_CORR
    plan, pos = _graded(200_000, flags)
    yield plan, pos
    plan.close()


@pytest.mark.parametrize("budget", [1e-6, 1e-7, 1e-4])
def test_budget_holds_on_graded_cloud(graded_plan, budget):
    """Budgets down to 1e-7: below about 1e-8 this cloud's worst-conditioned
    rows reach the rounding floor shared by the corrected FP32 result and the
    FP64 reference itself (both about 2^-48 sum_q |w| |f_q - f_p|)."""
    plan, pos = graded_plan
    plan.set_error_budget(budget)
    for name, f_np in _fields(pos).items():
        f = torch.tensor(f_np, device="cuda")
        ref = plan.apply(f, C.F64).cpu().numpy()
        plan.budget_stats(reset=True)
        out = plan.apply(f, C.F32_BUDGET).cpu().numpy()
        pairs = plan.budget_stats()
        for o in range(ref.shape[0]):
            err = normwise(out[o], ref[o])
            assert err <= budget, (name, o, err, budget, pairs)
        assert pairs > 0, (name, pairs)
    plan.set_error_budget(1e-6)


def test_budget_first_derivatives_of_a_linear_field(graded_plan):
    """A linear field: first derivatives within the budget.  (Its second
    derivatives vanish, so their FP64 values are rounding noise, below the
    2^-48 floor of the FP32 residuals; no relative budget applies there.)"""
    plan, pos = graded_plan
    f = torch.tensor(2.0 * pos[:, 0] - 0.5 * pos[:, 1], device="cuda")
    ref = plan.apply(f, C.F64).cpu().numpy()
    out = plan.apply(f, C.F32_BUDGET).cpu().numpy()
    for o in (0, 1):
        assert normwise(out[o], ref[o]) <= 1e-6, o


def test_plain_fp32_misses_the_budget_that_the_correction_meets(graded_plan):
    """The reason for the correction: on this graded cloud plain FP32 second
    derivatives exceed 1e-6 normwise."""
    plan, pos = graded_plan
    f = torch.tensor(_fields(pos)["sin_cos"], device="cuda")
    ref = plan.apply(f, C.F64).cpu().numpy()
    plain = plan.apply(f, C.F32).cpu().numpy()
    fixed = plan.apply(f, C.F32_BUDGET).cpu().numpy()
    worst_plain = max(normwise(plain[o], ref[o]) for o in range(5))
    worst_fixed = max(normwise(fixed[o], ref[o]) for o in range(5))
    assert worst_plain > 1e-6 and worst_fixed <= 1e-6, (worst_plain, worst_fixed)


def test_budget_on_bf16_residual_first_pass(cuda):
    """With the bf16 residual streams stored the first pass adds them (bound
    2^-32 instead of 2^-24): far fewer rows need FP64, same guarantee."""
    flags = C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32 | C.STORE_OUT_F32_CORR
    plain, pos = _graded(100_000, flags)
    resid, _ = _graded(100_000, flags | C.STORE_OUT_F32_RESID)
    f = torch.tensor(_fields(pos)["sin_cos"], device="cuda")
    ref = plain.apply(f, C.F64).cpu().numpy()
    counts = []
    resid.set_error_budget(1e-6, C.F32_RESID)
    for plan in (plain, resid):
        plan.budget_stats(reset=True)
        out = plan.apply(f, C.F32_BUDGET).cpu().numpy()
        counts.append(plan.budget_stats())
        for o in range(5):
            assert normwise(out[o], ref[o]) <= 1e-6, (o, normwise(out[o], ref[o]))
    assert counts[1] * 20 < counts[0], counts
    plain.close()
    resid.close()


def test_budget_csr_fallback_corrects_every_row(cuda):
    flags = C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32 | C.STORE_OUT_F32_CORR
    plan, pos = _graded(50_000, flags)
    plan.set_apply_config(0, 1)  # CSR kernel: no bounds, every row corrected
    f = torch.tensor(_fields(pos)["gauss"], device="cuda")
    ref = plan.apply(f, C.F64).cpu().numpy()
    plan.budget_stats(reset=True)
    out = plan.apply(f, C.F32_BUDGET).cpu().numpy()
    assert plan.budget_stats() == 5 * pos.shape[0]
    for o in range(5):
        assert normwise(out[o], ref[o]) <= 1e-7, o
    plan.close()


def test_budget_host_buffers_equal_device(cuda):
    pos, h = W.lattice(48, 3, jitter=0.15, seed=31)
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 2.8 * h)
    plan.assemble(pt, C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32 | C.STORE_OUT_F32_CORR)
    f_np = W.field2(pos)[0]
    dev = plan.apply(torch.tensor(f_np, device="cuda"), C.F32_BUDGET).cpu().numpy()
    ref = plan.apply(torch.tensor(f_np, device="cuda"), C.F64).cpu().numpy()
    for o in range(4):
        assert normwise(dev[o], ref[o]) <= 1e-6
    pageable = plan.apply_host(f_np, precision=C.F32_BUDGET)
    assert np.array_equal(pageable, dev)
    hf = torch.empty(f_np.shape[0], dtype=torch.float64, pin_memory=True)
    hf.copy_(torch.from_numpy(f_np))
    hout = torch.empty(dev.shape, dtype=torch.float64, pin_memory=True)
    plan.apply_host(hf.numpy(), hout.numpy(), C.F32_BUDGET)
    assert np.array_equal(hout.numpy(), dev)
    plan.close()


def test_budget_needs_the_residuals(cuda):
    pos, h = W.lattice(24, 2, jitter=0.1, seed=32)
    plan = DcpsePlan(2, [[(2, 0), (0, 2)]], order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 3.1 * h)
    plan.assemble(pt, C.ASSEMBLE_FAST | C.STORE_OUT_F32)
    with pytest.raises(C.DcpseError) as e:
        plan.apply(torch.zeros(pos.shape[0], dtype=torch.float64, device="cuda"), C.F32_BUDGET)
    assert e.value.code == C.ERR_STATE
    with pytest.raises(C.DcpseError):
        plan.set_error_budget(0.0)
    plan.set_error_budget(1e-6, C.F32_RESID)  # the bf16 first pass needs its streams
    plan2 = DcpsePlan(2, [[(2, 0), (0, 2)]], order=2)
    plan2.build_neighbors(pt, 3.1 * h)
    plan2.assemble(pt, C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.STORE_OUT_F32_CORR)
    plan2.set_error_budget(1e-6, C.F32_RESID)
    with pytest.raises(C.DcpseError) as e:
        plan2.apply(torch.zeros(pos.shape[0], dtype=torch.float64, device="cuda"), C.F32_BUDGET)
    assert e.value.code == C.ERR_STATE
    plan2.close()
    plan.close()
