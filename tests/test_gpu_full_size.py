"""Checks at the full benchmark size (128^3 = 2,097,152 jittered particles in
the unit cube, rCut = 2.8 h, Gradient + Laplacian of order 2), where the
oracle would take minutes: properties that hold at any size.

* neighbour lists: rows strictly ascending, no self entry, the relation
  symmetric (|x_p - x_q|^2 is the same number both ways), and each sampled
  row equal to a brute-force scan of all particles with the predicate
  |x_p - x_q|^2 < rCut^2 (openfpm_data VerletList, VL_SKIP_REF_PART);
* polynomial reproduction: an order-2 DC-PSE operator of derivative order
  |alpha| satisfies the moment conditions for every monomial of degree
  1 .. |alpha| + 1 (Dcpse.hpp:745-782, DcpseRhs.hpp:26-60), so it is exact on
  a quadratic field up to rounding (the oracle at 14^3 with the same spacing:
  gradient 5e-12, Laplacian 2.5e-9 normwise);
* linearity of the FP64 batched apply (up to the rounding of its sums);
* FP32 (sliced ELL, the default schedule) and the CSR schedules within the
  1e-6 normwise bar of the FP64 batched apply on a smooth field;
* the host-buffer apply (pinned field and outputs) equal to the device apply
  bit for bit.
Bars are max |a - b| / max |b| per output.
"""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return ((a - b).abs().amax(dim=-1) / b.abs().amax(dim=-1)).max().item()


@pytest.fixture(scope="module")
def full(cuda):
    cfg = W.config2(128)
    pos = torch.tensor(cfg["pos"], device="cuda")
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2)
    plan.build_neighbors(pos, cfg["rcut"])
    rc = plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32 | C.STORE_OUT_F32_RESID)
    assert rc == C.OK
    yield dict(cfg=cfg, pos=pos, plan=plan)
    plan.close()


def test_neighbors_full_size(full):
    plan, pos, rcut = full["plan"], full["pos"], full["cfg"]["rcut"]
    rowptr, cols = plan.neighbors()
    n = pos.shape[0]
    counts = rowptr[1:] - rowptr[:-1]
    assert counts.min().item() > 0 and rowptr[-1].item() == cols.numel()
    rows = torch.repeat_interleave(torch.arange(n, device="cuda"), counts)
    cl = cols.to(torch.int64)
    assert not bool((cl == rows).any())
    # strictly ascending (row, col) keys: rows sorted, no duplicates
    key = rows * n + cl
    assert bool((key[1:] > key[:-1]).all())
    # symmetric relation
    tkey, _ = torch.sort(cl * n + rows)
    assert torch.equal(tkey, key)
    del tkey, rows, cl
    # brute force on a sample of rows, every particle a candidate
    rc2 = rcut * rcut
    sample = torch.tensor(np.random.default_rng(21).choice(n, 256, replace=False), device="cuda")
    rp = rowptr.cpu().numpy()
    for b in range(0, sample.numel(), 32):
        ps = sample[b:b + 32]
        d = pos[None, :, :] - pos[ps][:, None, :]
        d2 = d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2]
        del d
        band = (d2 - rc2).abs() <= 1e-12 * rc2
        inside = d2 < rc2
        inside[torch.arange(ps.numel(), device="cuda"), ps] = False
        for i, p in enumerate(ps.tolist()):
            got = torch.zeros(n, dtype=torch.bool, device="cuda")
            got[cols[int(rp[p]):int(rp[p + 1])].to(torch.int64)] = True
            keep = ~band[i]
            assert torch.equal(got[keep], inside[i][keep])


def test_polynomial_reproduction_full_size(full):
    plan, pos = full["plan"], full["pos"]
    x, y, z = pos[:, 0], pos[:, 1], pos[:, 2]
    f = 1 + 3 * x - 2 * y + 0.5 * z + 7 * x * x - 5 * y * z + 11 * z * z + 4 * x * y
    exact = torch.stack([3 + 14 * x + 4 * y, -2 - 5 * z + 4 * x, 0.5 - 5 * y + 22 * z,
                         torch.full_like(x, 36.0)])
    got = plan.apply(f, C.F64)
    assert _rel(got[:3], exact[:3]) < 1e-9
    assert _rel(got[3:], exact[3:]) < 1e-7
    # FP32 weights with the bf16 residual: weight error ~2^-32 relative
    got = plan.apply(f, C.F32_RESID)
    assert _rel(got, exact) < 1e-5


def test_linearity_full_size(full):
    plan, pos = full["plan"], full["pos"]
    f = torch.tensor(W.field2(full["cfg"]["pos"])[0], device="cuda")
    g = torch.sin(7 * pos[:, 1]) * pos[:, 2]
    lf, lg = plan.apply(f, C.F64), plan.apply(g, C.F64)
    lc = plan.apply(2.0 * f - 3.0 * g, C.F64)
    # exact up to rounding of sums whose terms are ~1e3 times the Laplacian
    # (measured 1.7e-12); a wrong weight or column gives ~1e-3
    assert _rel(lc, 2.0 * lf - 3.0 * lg) < 1e-10


def test_fp32_schedules_full_size(full):
    plan = full["plan"]
    f = torch.tensor(W.field2(full["cfg"]["pos"])[0], device="cuda")
    ref = plan.apply(f, C.F64)
    plan.set_apply_config(0, 0)
    default = plan.apply(f, C.F32)
    assert _rel(default, ref) < 1e-6
    assert _rel(plan.apply(f, C.F32_RESID), ref) < 1e-8
    for lanes, mode in ((4, 1), (8, 1), (0, 4)):
        plan.set_apply_config(lanes, mode)
        assert _rel(plan.apply(f, C.F32), ref) < 1e-6
    plan.set_apply_config(0, 0)


def test_host_apply_full_size(full):
    plan = full["plan"]
    f_np = W.field2(full["cfg"]["pos"])[0]
    dev = plan.apply(torch.tensor(f_np, device="cuda"), C.F32).cpu()
    f_pin = torch.tensor(f_np).pin_memory()
    out_pin = torch.full((plan.n_outputs, f_np.shape[0]), float("nan"), dtype=torch.float64).pin_memory()
    plan.apply_host(f_pin.numpy(), out_pin.numpy(), precision=C.F32)
    assert torch.equal(out_pin, dev)
    # pageable buffers take the copy pipeline
    assert np.array_equal(plan.apply_host(f_np, precision=C.F32), dev.numpy())
