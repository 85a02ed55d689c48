"""DCPSE_F32_PAIR: the summed weights as FP32 pairs w32 + (w64 - w32) (48
significant bits), the field in 62-bit fixed point (exact differences, each
as a float pair) and compensated FP32 sums over every output.  Its bar is
the batched FP64
apply's (Dcpse.hpp:467-499 summed per output): within 1e-12 normwise of the
reference-order outputs, which the oracle's per-term kernels give bit for
bit (checked against the oracle on a small set, at the benchmark size
against the plan's reference-order terms).  Without the sliced layout the
batched FP64 apply serves, bit for bit.
"""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu

# reference-order assembly (per-term kernels kept), summed weights in FP64
# and as FP32 pairs
FLAGS = C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32 | C.STORE_OUT_F32_CORR


def _rel(a, b):
    return max(float(np.abs(a[o] - b[o]).max() / np.abs(b[o]).max()) for o in range(b.shape[0]))


def _reference_order(plan, f, nout):
    """Each output as the reference sums it: one FP64 pass per Dcpse term."""
    return np.stack([plan.apply_output_f64(o, f).cpu().numpy() for o in range(nout)])


def test_pair_against_oracle(cuda, orc):
    pos, h = W.lattice(20, 3, jitter=0.15, seed=61)
    outputs = W.grad_lap_outputs(3)
    plan = DcpsePlan(3, outputs, order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 2.8 * h)
    plan.assemble(pt, FLAGS)
    fn = W.field2(pos)[0]
    f = torch.tensor(fn, device="cuda")
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    sigs = [s for out in outputs for s in out]
    tout = [o for o, out in enumerate(outputs) for _ in out]
    terms = []
    for sg in sigs:
        eps, eip, K, st = orc.assemble(pos, rp, cols, sg, 2, nthreads=8)
        terms.append((K, eip, sum(sg)))
    ref = orc.MultiApply(rp, cols, terms, tout, len(outputs), fn)(8)
    got = plan.apply(f, C.F32_PAIR).cpu().numpy()
    assert _rel(got, ref) <= 1e-12
    # the FP32 weights alone are at the FP32 level
    assert _rel(plan.apply(f, C.F32).cpu().numpy(), ref) > 1e-10
    plan.close()


def test_pair_full_size(cuda):
    cfg = W.config2(128)
    pos = torch.tensor(cfg["pos"], device="cuda")
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2)
    plan.build_neighbors(pos, cfg["rcut"])
    plan.assemble(pos, FLAGS)
    f = torch.tensor(W.field2(cfg["pos"])[0], device="cuda")
    ref = _reference_order(plan, f, 4)
    got = plan.apply(f, C.F32_PAIR).cpu().numpy()
    b64 = plan.apply(f, C.F64).cpu().numpy()
    assert _rel(got, ref) <= 1e-12
    assert _rel(b64, ref) <= 1e-12
    plan.close()


def test_pair_falls_back_to_fp64_without_the_sliced_layout(cuda):
    pos, h = W.lattice(16, 3, jitter=0.15, seed=62)
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 2.8 * h)
    plan.assemble(pt, FLAGS)
    f = torch.tensor(W.field2(pos)[0], device="cuda")
    plan.set_apply_config(0, 1)  # a CSR schedule: no sliced layout
    assert torch.equal(plan.apply(f, C.F32_PAIR), plan.apply(f, C.F64))
    plan.close()


def test_pair_needs_the_fp32_residuals(cuda):
    pos, h = W.lattice(10, 3, jitter=0.15, seed=63)
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 2.8 * h)
    plan.assemble(pt, C.STORE_OUT_F64 | C.STORE_OUT_F32)
    with pytest.raises(C.DcpseError):
        plan.apply(torch.tensor(W.field2(pos)[0], device="cuda"), C.F32_PAIR)
    plan.close()


def _small_plan(nside=12, seed=64):
    pos, h = W.lattice(nside, 3, jitter=0.15, seed=seed)
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 2.8 * h)
    plan.assemble(pt, FLAGS)
    return plan, pos


def test_pair_is_exact_under_power_of_two_scaling(cuda):
    """The fixed-point field takes its scale from the call's largest |f|: a
    field scaled by 2^k gives the same integers, so the outputs scale by 2^k
    bit for bit (far above and below the FP32 range)."""
    plan, pos = _small_plan()
    f = torch.tensor(W.field2(pos)[0], device="cuda")
    base = plan.apply(f, C.F32_PAIR)
    for k in (700, -900, 40):
        assert torch.equal(plan.apply(f * 2.0 ** k, C.F32_PAIR), base * 2.0 ** k)
    plan.close()


def test_pair_non_finite_field_gives_nan(cuda):
    plan, pos = _small_plan(8)
    f = torch.tensor(W.field2(pos)[0], device="cuda")
    for bad in (float("nan"), float("inf")):
        g = f.clone()
        g[5] = bad
        assert torch.isnan(plan.apply(g, C.F32_PAIR)).all()
    # the plan stays usable
    assert torch.isfinite(plan.apply(f, C.F32_PAIR)).all()
    plan.close()


def test_pair_zero_field(cuda):
    plan, pos = _small_plan(8)
    out = plan.apply(torch.zeros(pos.shape[0], dtype=torch.float64, device="cuda"), C.F32_PAIR)
    assert torch.count_nonzero(out) == 0
    plan.close()

