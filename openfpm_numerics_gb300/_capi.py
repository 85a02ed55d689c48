"""ctypes binding of the DC-PSE C-ABI (include/openfpm_dcpse/dcpse_capi.h).

The shared library is built in-tree by :mod:`openfpm_numerics_gb300.build`.
There is no fallback: if the library cannot be loaded every call raises.
"""
from __future__ import annotations

import ctypes
import os
import re

from . import build as _build

HEADER = os.path.join(_build.INCLUDE, "openfpm_dcpse", "dcpse_capi.h")

_c = ctypes
_P = _c.c_void_p
_I = _c.c_int
_I64 = _c.c_int64
_D = _c.c_double
_PI = _c.POINTER(_c.c_int)
_PI64 = _c.POINTER(_c.c_int64)
_PU = _c.POINTER(_c.c_uint)
_PP = _c.POINTER(_c.c_void_p)

# name -> (restype, argtypes)
SIGNATURES = {
    "dcpse_last_error": (_c.c_char_p, []),
    "dcpse_version": (_I, []),
    "dcpse_plan_create": (_I, [_PP, _I, _I, _PI, _PU, _c.c_uint, _D]),
    "dcpse_plan_destroy": (_I, [_P]),
    "dcpse_plan_set_stream": (_I, [_P, _P]),
    "dcpse_plan_set_box": (_I, [_P, _c.POINTER(_D), _c.POINTER(_D), _PI]),
    "dcpse_plan_set_support": (_I, [_P, _P, _I64, _I]),
    "dcpse_plan_set_surface": (_I, [_P, _P, _I, _D, _P]),
    "dcpse_plan_info": (_I, [_P, _PI64, _PI64, _PI, _PI, _PI]),
    "dcpse_term_basis": (_I, [_P, _I, _PU, _I, _PI]),
    "dcpse_build_neighbors": (_I, [_P, _P, _I64, _D, _P]),
    "dcpse_set_neighbors": (_I, [_P, _I64, _I64, _P, _P]),
    "dcpse_neighbors_ptr": (_I, [_P, _PP, _PP]),
    "dcpse_assemble": (_I, [_P, _P, _P, _I]),
    "dcpse_particle_status": (_I, [_P, _PI64, _PI64, _PI]),
    "dcpse_plan_assembly_info": (_I, [_P, _PI]),
    "dcpse_eps_ptr": (_I, [_P, _PP, _PP]),
    "dcpse_term_kernels_ptr": (_I, [_P, _I, _PP, _PP]),
    "dcpse_output_weights_ptr": (_I, [_P, _I, _PP, _PP]),
    "dcpse_apply_term_f64": (_I, [_P, _I, _P, _P]),
    "dcpse_apply_output_f64": (_I, [_P, _I, _P, _P]),
    "dcpse_apply_batched": (_I, [_P, _P, _P, _I]),
    "dcpse_apply_batched_host": (_I, [_P, _P, _P, _I]),
    "dcpse_plan_set_error_budget": (_I, [_P, _D, _I]),
    "dcpse_plan_budget_stats": (_I, [_P, _PI64, _I]),
    "dcpse_plan_set_reorder": (_I, [_P, _I]),
    "dcpse_plan_set_reorder_order": (_I, [_P, _I]),
    "dcpse_plan_reorder_info": (_I, [_P, _PI, _c.POINTER(_D), _c.POINTER(_D)]),
    "dcpse_apply_batched_f32_noalloc": (_I, [_I64, _I, _P, _P, _P, _I64, _P, _P, _P]),
    "dcpse_p2p_f64": (_I, [_P, _I, _P, _I, _P]),
    "dcpse_p2p": (_I, [_P, _P, _I, _P, _I]),
    "dcpse_operator_csr": (_I, [_P, _I, _D, _P, _I64, _I, _I, _P, _P, _P, _PI64]),
    "dcpse_set_term_kernels": (_I, [_P, _I, _P, _P, _P]),
    "dcpse_vjp_field": (_I, [_P, _P, _P, _I]),
    "dcpse_vjp_positions": (_I, [_P, _P, _P, _P, _P, _P]),
    "dcpse_rk4_gs_stage": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _c.POINTER(_D)]),
    "dcpse_rk4_gs_adjoint_prepare": (_I, [_P, _I]),
    "dcpse_rk4_gs_adjoint_stage": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _D, _D, _c.POINTER(_D)]),
    "dcpse_rk4_gs_reverse_step": (_I, [_P, _I, _c.POINTER(_P), _P, _P, _P, _P, _c.POINTER(_D)]),
    "dcpse_device_alloc": (_I, [_PP, _c.c_uint64]),
    "dcpse_device_free": (_I, [_P]),
    "dcpse_host_alloc": (_I, [_PP, _c.c_uint64]),
    "dcpse_host_free": (_I, [_P]),
    "dcpse_copy": (_I, [_P, _P, _c.c_uint64]),
    "dcpse_plan_set_timing": (_I, [_P, _I]),
    "dcpse_plan_set_apply_config": (_I, [_P, _I, _I]),
    "dcpse_plan_set_assembly_config": (_I, [_P, _I, _I, _I]),
    "dcpse_measure_fp64_peak": (_I, [_P, _c.POINTER(_D)]),
    "dcpse_plan_check": (_I, [_P]),
    "dcpse_plan_timing": (_I, [_P, _I, _c.POINTER(_D), _PI64]),
    "dcpse_plan_reset_timing": (_I, [_P]),
}

K_APPLY_BATCHED, K_SPLIT, K_ASSEMBLE, K_APPLY_TERM, K_NEIGHBORS, K_CORRECT = range(6)

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_STATE = 3
ERR_CAPACITY = 4
ERR_IO = 5
ERR_PARTICLES = 6
ERR_TIMEOUT = 7

STORE_TERMS_F64 = 1
STORE_OUT_F64 = 2
STORE_OUT_F32 = 4
ASSEMBLE_FAST = 8
ASSEMBLE_ASYNC = 16
STORE_OUT_F32_RESID = 32
STORE_OUT_F32_CORR = 64
ASSEMBLE_TC = 128

F64 = 0
F32 = 1
F32_RESID = 2
F32_BUDGET = 3
F32_PAIR = 4

# apply schedule bits (dcpse_plan_set_apply_config mode)
APPLY_COMPENSATE_ALL = 16
APPLY_STREAM_HINT_ON = 32
APPLY_STREAM_HINT_OFF = 64
APPLY_SLICE_WINDOWS = 128
APPLY_SLICE_WARPS = 256

PART_OK, PART_TOO_FEW, PART_BAD_EPS, PART_SINGULAR, PART_NONFINITE = range(5)


class DcpseError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("DC-PSE error %d: %s" % (code, msg))
        self.code = code


_lib = None


def declared_symbols():
    """Function names declared in the C header."""
    with open(HEADER) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"\b(dcpse_[a-z0-9_]+)\s*\(", text)))


def load(build_if_missing: bool = True):
    """Load (building first if needed) the extension; raises if impossible."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise OSError("DC-PSE CUDA extension not built: %s" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, allow=()):
    if rc != OK and rc not in allow:
        raise DcpseError(rc, load().dcpse_last_error().decode())
    return rc


def call(name, *args, allow=()):
    return check(getattr(load(), name)(*args), allow=allow)
