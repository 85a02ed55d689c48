"""The C-ABI library builds for sm_103a, loads, and exports every symbol the
header declares (no compute calls: runs without a GPU)."""
import ctypes

from openfpm_numerics_gb300 import _capi as C


def test_library_exports_declared_symbols():
    lib = C.load()
    declared = C.declared_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    assert set(declared) <= set(C.SIGNATURES), set(declared) - set(C.SIGNATURES)


def test_host_only_calls():
    lib = C.load()
    assert lib.dcpse_version() >= 1
    # argument validation runs on the host and reports through the status
    h = ctypes.c_void_p()
    rc = lib.dcpse_plan_create(ctypes.byref(h), 4, 1, (ctypes.c_int * 1)(1), (ctypes.c_uint * 4)(1, 0, 0, 0), 2, 0.9)
    assert rc == C.ERR_ARG and b"dim" in lib.dcpse_last_error()
    rc = lib.dcpse_plan_create(None, 2, 1, (ctypes.c_int * 1)(1), (ctypes.c_uint * 2)(1, 0), 2, 0.9)
    assert rc == C.ERR_ARG
    rc = lib.dcpse_plan_destroy(None)
    assert rc == C.OK
    rc = lib.dcpse_apply_batched(None, None, None, 0)
    assert rc == C.ERR_ARG


def test_python_length_checks():
    """The Python plan checks array lengths and output shapes before any
    bare-pointer C-ABI call (host logic only)."""
    import pytest
    import torch

    from openfpm_numerics_gb300.plan import DcpsePlan

    DcpsePlan._check_rows(5, 5, "field")
    DcpsePlan._check_rows(7, None, "field")  # no list yet: the library reports the state
    DcpsePlan._check_rows(7, -1, "field")
    with pytest.raises(ValueError):
        DcpsePlan._check_rows(4, 5, "field")
    out = torch.empty((2, 5), dtype=torch.float64)
    assert DcpsePlan._check_out(out, (2, 5)) is out
    for bad in (torch.empty((2, 4), dtype=torch.float64), torch.empty((2, 5), dtype=torch.float32)):
        with pytest.raises(ValueError):
            DcpsePlan._check_out(bad, (2, 5))


def test_python_constants_match_the_header():
    """Every DCPSE_* constant the Python binding mirrors has the header's
    value (store flags, precisions, apply schedule bits, status codes)."""
    import re

    text = open(C.HEADER).read()
    defines = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define DCPSE_([A-Z0-9_]+)\s+(\d+)\b", text)}
    for name in ("F32_PAIR", "APPLY_SLICE_WINDOWS", "APPLY_SLICE_WARPS", "STORE_OUT_F32_CORR", "ASSEMBLE_TC"):
        assert name in defines and hasattr(C, name), name
    mismatched = {n: (v, getattr(C, n)) for n, v in defines.items() if hasattr(C, n) and getattr(C, n) != v}
    assert not mismatched, mismatched
