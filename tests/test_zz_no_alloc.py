"""The allocation-free batched FP32 apply (dcpse_apply_batched_f32_noalloc).

It serves callers that cannot call cudaMalloc at the point where they apply
an operator (allocator callbacks, host functions enqueued on a stream,
latency-critical loops, processes whose device memory another framework
owns).  It must give exactly what the ordinary entry point gives, on
consecutive calls sharing its fixed scratch array, and refuse sizes beyond
that array.  The inputs are prepared with the ordinary plan API (which does
allocate); only the call under test is allocation-free.
"""
import ctypes

import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_apply_matches_plan_apply(cuda):
    lib = C.load()
    pos, h = W.lattice(40, 2, jitter=0.15, seed=21)
    outputs = [[(1, 0)], [(0, 1)], [(2, 0), (0, 2)]]
    plan = DcpsePlan(2, outputs, order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 3.1 * h)
    plan.assemble(pt, C.STORE_OUT_F32)
    rowptr, cols = plan.neighbors()
    _, w32 = plan.output_weights(0)          # base of the [outputs][nnz] FP32 weights
    nnz = plan.info()["nnz"]
    n = pos.shape[0]
    rng = np.random.default_rng(3)
    for call in range(2):                    # two calls in a row share the scratch
        f = torch.tensor(rng.standard_normal(n) + call, device="cuda")
        plan.set_apply_config(0, 0)          # the plan's default schedule: within the FP32 bar
        ref_default = plan.apply(f, C.F32).clone()
        plan.set_apply_config(0, 1 | 16)     # same schedule as the allocation-free call: identical
        ref = plan.apply(f, C.F32)
        out = torch.full((len(outputs), n), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.dcpse_apply_batched_f32_noalloc(n, len(outputs), _p(rowptr), _p(cols), _p(w32), nnz, _p(f),
                                                 _p(out), None)
        assert rc == C.OK, lib.dcpse_last_error()
        torch.cuda.synchronize()
        assert torch.equal(out, ref), "call %d" % call
        scale = ref_default.abs().amax(dim=1, keepdim=True)
        assert bool(((out - ref_default).abs() <= 1e-6 * scale).all()), "call %d" % call
    plan.close()


def test_noalloc_rejects_oversize(cuda):
    lib = C.load()
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = lib.dcpse_apply_batched_f32_noalloc(2097152 + 1, 1, _p(dummy), _p(dummy), _p(dummy), 0, _p(dummy),
                                             _p(dummy), None)
    assert rc == C.ERR_CAPACITY
    assert b"DCPSE_NOALLOC_MAX_PARTICLES" in lib.dcpse_last_error()
