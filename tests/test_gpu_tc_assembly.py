"""Fast assembly with the Gram products on the tensor cores (DCPSE_ASSEMBLE_TC).

The tensor-core Gram is exact up to a 62-bit fixed-point representation of
B and one final rounding, so it is more accurate than the sequential FP64
sum of the reference's order (Dcpse.hpp:745-757) but not bit-identical to
it.  The kernels solve the normal equations, so on ill-conditioned moment
systems (boundary and strongly graded particles) any change of the Gram's
rounding moves them: the oracle run once with the reference's sum and once
with a double-double sum rounded once (the correctly rounded Gram) measures
that sensitivity.  The tests require
  * the weights within 1e-12 (interior rows) and 1e-9 (all rows), normwise
    per output, of the FP64-sum fast assembly (identical B);
  * the applied operators at least as close to the correctly-rounded-Gram
    oracle as the FP64-sum fast assembly is (maximum and 99th percentile,
    with 1e-10 of the output's scale as the floor and 25% slack);
  * the applied operators within the reference's own Gram-rounding
    sensitivity of its reference-order outputs.
"""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu

FAST = C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32


def _weights(plan, nout):
    return [plan.output_weights(o)[0].cpu().numpy().copy() for o in range(nout)]


def _row_norm_err(a, b, rp, rows):
    worst = 0.0
    for r in rows:
        s = slice(rp[r], rp[r + 1])
        if rp[r + 1] > rp[r]:
            worst = max(worst, float(np.abs(a[s] - b[s]).max() / max(np.abs(b[s]).max(), 1e-300)))
    return worst


@pytest.mark.parametrize("case", ["lattice3d", "graded2d"])
def test_tc_assembly_matches_fp64_assembly_and_oracle(cuda, orc, case):
    if case == "lattice3d":
        pos, h = W.lattice(20, 3, jitter=0.15, seed=51)
        outputs, rcut, rpp = W.grad_lap_outputs(3), 2.8 * h, None
        f = W.field2(pos)[0]
    else:
        cfg = W.config3(n=20000, seed=52)
        pos, outputs, rcut, rpp = cfg["pos"], W.five_ops_2d(), 0.0, cfg["rcut_pp"]
        f = np.sin(2 * np.pi * pos[:, 0]) * np.cos(2 * np.pi * pos[:, 1])
    pt = torch.tensor(pos, device="cuda")
    rpt = None if rpp is None else torch.tensor(rpp, device="cuda")
    nout = len(outputs)
    plans = {}
    for name, flags in (("simt", FAST), ("tc", FAST | C.ASSEMBLE_TC)):
        plan = DcpsePlan(pos.shape[1], outputs, order=2)
        plan.build_neighbors(pt, rcut, rpt)
        plan.assemble(pt, flags)
        plans[name] = plan
    assert plans["tc"].gram_on_tensor_cores() and not plans["simt"].gram_on_tensor_cores()
    rp = plans["simt"].neighbors()[0].cpu().numpy()
    status = plans["simt"].eps()[1].cpu().numpy()
    assert np.array_equal(status, plans["tc"].eps()[1].cpu().numpy())
    margin = float(np.max(rpp)) if rpp is not None else rcut
    inner = np.where(np.all((pos > margin) & (pos < pos.max(axis=0) - margin), axis=1) & (status == 0))[0]
    allr = np.where(status == 0)[0]
    ws, wt = _weights(plans["simt"], nout), _weights(plans["tc"], nout)
    for o in range(nout):
        assert _row_norm_err(wt[o], ws[o], rp, inner) <= 1e-12, ("interior", o)
        assert _row_norm_err(wt[o], ws[o], rp, allr) <= 1e-9, ("all rows", o)
    # applied operators against the oracle, with its Gram summed in the
    # reference's order and in double-double
    cols = plans["simt"].neighbors()[1].cpu().numpy()
    sigs = [s for out in outputs for s in out]
    tout = [o for o, out in enumerate(outputs) for _ in out]
    refs = []
    for exact in (False, True):
        terms = []
        for sg in sigs:
            eps, eip, K, st = orc.assemble(pos, rp, cols, sg, 2, nthreads=8, exact_gram=exact)
            terms.append((K, eip, sum(sg)))
        refs.append(orc.MultiApply(rp, cols, terms, tout, nout, f)(8))
    ref, refx = refs
    ft = torch.tensor(f, device="cuda")
    got = plans["tc"].apply(ft, C.F64).cpu().numpy()
    fp64 = plans["simt"].apply(ft, C.F64).cpu().numpy()
    m = status == 0
    for o in range(nout):
        scale = np.abs(ref[o][m]).max()
        dev = lambda x, y: np.abs(x[o][m] - y[o][m]) / scale
        tc_x, fp64_x, ref_x = dev(got, refx), dev(fp64, refx), dev(ref, refx)
        assert tc_x.max() <= max(1e-10, 1.25 * fp64_x.max()), (o, tc_x.max(), fp64_x.max())
        assert np.percentile(tc_x, 99) <= max(1e-12, 1.25 * np.percentile(fp64_x, 99)), o
        sens = ref_x.max()
        assert dev(got, ref).max() <= max(1e-10, 2 * sens + dev(fp64, ref).max()), (o, sens)
    for p in plans.values():
        p.close()


def test_tc_assembly_falls_back_beyond_its_limits(cuda):
    """More than 128 neighbours: the FP64 Gram kernel serves, bit for bit."""
    pos, h = W.lattice(14, 3, jitter=0.1, seed=53)
    pt = torch.tensor(pos, device="cuda")
    out = []
    for flags in (C.ASSEMBLE_FAST | C.STORE_OUT_F64, C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.ASSEMBLE_TC):
        plan = DcpsePlan(3, [[(2, 0, 0), (0, 2, 0), (0, 0, 2)]], order=2)
        plan.build_neighbors(pt, 3.5 * h)
        assert plan.info()["max_neighbors"] > 128
        plan.assemble(pt, flags)
        assert not plan.gram_on_tensor_cores()
        out.append(plan.output_weights(0)[0].cpu().numpy().copy())
        plan.close()
    assert np.array_equal(out[0], out[1])


def test_tc_assembly_with_status_failures(cuda):
    """Particles that cannot be assembled (too few neighbours) keep zero
    weights and their status; the others are assembled on the tensor cores."""
    rng = np.random.default_rng(54)
    pos = np.concatenate([W.lattice(16, 2, jitter=0.1, seed=54)[0], rng.uniform(3.0, 4.0, (5, 2))])
    h = 1.0 / 15
    pt = torch.tensor(pos, device="cuda")
    plan = DcpsePlan(2, W.five_ops_2d(), order=2)
    plan.build_neighbors(pt, 3.1 * h)
    plan.assemble(pt, FAST | C.ASSEMBLE_TC)
    assert plan.gram_on_tensor_cores()
    st = plan.eps()[1].cpu().numpy()
    assert (st[-5:] != 0).all() and (st[:-5] == 0).all()
    plan.close()
