"""The allocation-free batched FP32 apply (dcpse_apply_batched_f32_noalloc).

It serves callers that cannot call cudaMalloc at the point where they apply
an operator (allocator callbacks, latency-critical loops, processes whose
device memory another framework owns).  It must give exactly what the
ordinary entry point gives, on consecutive calls sharing its fixed scratch
array, leave the device's free memory unchanged once warmed up, and refuse
sizes beyond that array.  The inputs are prepared with the ordinary plan API
(which does allocate); only the call under test is allocation-free.
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


def _warm_up(lib):
    # n = 0: places the scratch array and the kernels on this device
    rc = lib.dcpse_apply_batched_f32_noalloc(0, 1, None, None, None, 0, None, None, None)
    assert rc == C.OK, lib.dcpse_last_error()


def test_noalloc_apply_matches_plan_apply(cuda):
    lib = C.load()
    _warm_up(lib)
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


def test_noalloc_leaves_free_memory_unchanged(cuda):
    """After the warm-up and one call, further calls change the device's
    free memory by not one byte (cudaMemGetInfo)."""
    lib = C.load()
    _warm_up(lib)
    pos, h = W.lattice(32, 2, jitter=0.1, seed=22)
    plan = DcpsePlan(2, [[(1, 0)], [(2, 0), (0, 2)]], order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 3.1 * h)
    plan.assemble(pt, C.STORE_OUT_F32)
    rowptr, cols = plan.neighbors()
    _, w32 = plan.output_weights(0)
    nnz = plan.info()["nnz"]
    n = pos.shape[0]
    f = torch.tensor(np.cos(3.0 * pos[:, 0]) + pos[:, 1] ** 2, device="cuda")
    out = torch.empty((2, n), dtype=torch.float64, device="cuda")
    args = (n, 2, _p(rowptr), _p(cols), _p(w32), nnz, _p(f), _p(out), None)
    assert lib.dcpse_apply_batched_f32_noalloc(*args) == C.OK, lib.dcpse_last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert lib.dcpse_apply_batched_f32_noalloc(*args) == C.OK, lib.dcpse_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    plan.close()


def test_noalloc_one_output_zero_stride(cuda):
    """One output with w_stride = 0 (no second stream to step over): within
    the FP32 bar of the plan's own FP32 apply, on two calls in a row."""
    lib = C.load()
    _warm_up(lib)
    pos, h = W.lattice(36, 2, jitter=0.12, seed=23)
    plan = DcpsePlan(2, [[(2, 0), (0, 2)]], order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 3.1 * h)
    plan.assemble(pt, C.STORE_OUT_F32)
    rowptr, cols = plan.neighbors()
    _, w32 = plan.output_weights(0)
    n = pos.shape[0]
    rng = np.random.default_rng(5)
    for call in range(2):
        f = torch.tensor(np.sin(2 * np.pi * pos[:, 0]) + 0.1 * call * rng.standard_normal(n), device="cuda")
        ref = plan.apply(f, C.F32).clone()
        out = torch.full((1, n), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.dcpse_apply_batched_f32_noalloc(n, 1, _p(rowptr), _p(cols), _p(w32), 0, _p(f), _p(out), None)
        assert rc == C.OK, lib.dcpse_last_error()
        torch.cuda.synchronize()
        scale = ref.abs().max()
        assert bool(((out - ref).abs() <= 1e-6 * scale).all()), "call %d" % call
    plan.close()


def test_noalloc_rejects_oversize_and_overlapping_streams(cuda):
    lib = C.load()
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = lib.dcpse_apply_batched_f32_noalloc(2097152 + 1, 1, _p(dummy), _p(dummy), _p(dummy), 0, _p(dummy),
                                             _p(dummy), None)
    assert rc == C.ERR_CAPACITY
    assert b"DCPSE_NOALLOC_MAX_PARTICLES" in lib.dcpse_last_error()
    # two outputs with a zero stride would read one weight stream twice
    rc = lib.dcpse_apply_batched_f32_noalloc(2, 2, _p(dummy), _p(dummy), _p(dummy), 0, _p(dummy), _p(dummy), None)
    assert rc == C.ERR_ARG
