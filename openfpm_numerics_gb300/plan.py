"""Python host side of the DC-PSE C-ABI: a plan object over torch tensors.

PyTorch is only plumbing here (device memory, streams).  Every computation is
a call into ``libdcpse_gb300.so``; there is no CPU or PyTorch fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi as C


class _DevView:
    """Zero-copy view of a plan-owned device array for torch.as_tensor.  The
    tensor keeps this object, and through ``owner`` the plan, alive: a view
    never outlives the memory it reads (until the plan is closed explicitly
    or re-assembled)."""

    def __init__(self, ptr, shape, typestr, owner=None):
        self.owner = owner
        self.__cuda_array_interface__ = {
            "shape": tuple(int(s) for s in shape),
            "typestr": typestr,
            "data": (int(ptr), False),
            "version": 3,
            "strides": None,
        }


def _view(ptr, shape, dtype, owner=None):
    ts = {torch.float64: "<f8", torch.float32: "<f4", torch.int64: "<i8", torch.int32: "<i4"}[dtype]
    if int(np.prod(shape)) == 0 or not ptr:
        return torch.empty(shape, dtype=dtype, device="cuda")
    return torch.as_tensor(_DevView(ptr, shape, ts, owner), device="cuda")


def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return ctypes.c_void_p(t.data_ptr())


def _stream_ptr(stream):
    if stream is None:
        return None
    return ctypes.c_void_p(stream.cuda_stream)


class DcpsePlan:
    """One particle set, its neighbour list and a set of DC-PSE outputs.

    ``outputs`` is a list of outputs, each a list of signatures (one per
    reference Dcpse term); e.g. a 3D Gradient + Laplacian is
    ``[[(1,0,0)], [(0,1,0)], [(0,0,1)], [(2,0,0),(0,2,0),(0,0,2)]]``.
    """

    def __init__(self, dim, outputs, order=2, h_over_eps=0.9, box=None, stream=None):
        self.dim = int(dim)
        self.outputs = [[tuple(int(x) for x in s) for s in o] for o in outputs]
        self.order = int(order)
        self.h_over_eps = float(h_over_eps)
        terms = [len(o) for o in self.outputs]
        sigs = [x for o in self.outputs for s in o for x in s]
        for o in self.outputs:
            for s in o:
                if len(s) != self.dim:
                    raise ValueError("signature %r does not have %d entries" % (s, self.dim))
        tarr = (ctypes.c_int * len(terms))(*terms)
        sarr = (ctypes.c_uint * len(sigs))(*sigs)
        h = ctypes.c_void_p()
        C.call("dcpse_plan_create", ctypes.byref(h), self.dim, len(terms), tarr, sarr, self.order,
               self.h_over_eps)
        self._h = h
        self.stream = stream
        C.call("dcpse_plan_set_stream", self._h, _stream_ptr(stream))
        self.box = None
        # bumped by every call that changes the list or the weights (see
        # generation): lets a caller tell whether the plan still holds what
        # it assembled
        self._gen = 0
        if box is not None:
            self.set_box(*box)
        self.n = None

    @property
    def generation(self):
        """A counter bumped by every call that changes the neighbour list or
        the weights (set_box, set_support, set_surface, build_neighbors,
        set_neighbors, assemble, set_term_kernels)."""
        return self._gen

    # -- lifetime -------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            C.load().dcpse_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- set-up ---------------------------------------------------------
    def set_stream(self, stream):
        """Enqueue the plan's work on a torch.cuda.Stream (None = legacy default)."""
        C.call("dcpse_plan_set_stream", self._h, _stream_ptr(stream))
        self.stream = stream

    def set_box(self, lo, hi, periodic=None):
        lo = (ctypes.c_double * self.dim)(*[float(x) for x in lo])
        hi = (ctypes.c_double * self.dim)(*[float(x) for x in hi])
        per = (ctypes.c_int * self.dim)(*([int(bool(p)) for p in periodic] if periodic is not None else
                                          [0] * self.dim))
        self._gen += 1
        C.call("dcpse_plan_set_box", self._h, lo, hi, per)
        self.box = (tuple(lo), tuple(hi), tuple(per))

    @property
    def n_terms(self):
        return sum(len(o) for o in self.outputs)

    @property
    def n_outputs(self):
        return len(self.outputs)

    def info(self):
        n, nnz = ctypes.c_int64(), ctypes.c_int64()
        nt, no, mk = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        C.call("dcpse_plan_info", self._h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nt), ctypes.byref(no),
               ctypes.byref(mk))
        return {"n": n.value, "nnz": nnz.value, "terms": nt.value, "outputs": no.value, "max_neighbors": mk.value}

    def term_basis(self, term):
        cap = 64
        ex = (ctypes.c_uint * (cap * self.dim))()
        n = ctypes.c_int()
        C.call("dcpse_term_basis", self._h, int(term), ex, cap, ctypes.byref(n))
        return np.array(ex[: n.value * self.dim], dtype=np.uint32).reshape(n.value, self.dim)

    def set_support(self, pos_support=None, self_skip=True):
        """Columns of the neighbour lists: a second particle set (two-set
        operator, as PPInterpolation's Dcpse) or, with None, the domain set
        itself, where self_skip=False keeps each particle in its own list (a
        plain VL_NON_SYMMETRIC list).  The plan keeps a reference to the
        tensor; the neighbour list must be built again."""
        if pos_support is not None:
            pos_support = self._check_pos(pos_support)
            self._gen += 1
            C.call("dcpse_plan_set_support", self._h, _ptr(pos_support), pos_support.shape[0], int(bool(self_skip)))
        else:
            self._gen += 1
            C.call("dcpse_plan_set_support", self._h, None, 0, int(bool(self_skip)))
        self._support = pos_support
        self.n = None

    def set_surface(self, normals=None, n_count=0, n_spacing=0.0, n_spacings=None):
        """Surface operator (SurfaceDcpse): unit normals [n_base, dim] of the
        support particles, n_count virtual particles on each side at spacing
        n_spacing (or per particle n_spacings).  None switches it off.  The
        plan keeps references; the neighbour list must be built again."""
        if normals is not None:
            normals = normals.to(device="cuda", dtype=torch.float64).contiguous()
            if n_spacings is not None:
                n_spacings = n_spacings.to(device="cuda", dtype=torch.float64).contiguous()
            self._gen += 1
            C.call("dcpse_plan_set_surface", self._h, _ptr(normals), int(n_count), float(n_spacing),
                   _ptr(n_spacings))
        else:
            self._gen += 1
            C.call("dcpse_plan_set_surface", self._h, None, 0, 0.0, None)
        self._surface = (normals, n_spacings)
        self.n = None

    def build_neighbors(self, pos, rcut, rcut_pp=None):
        pos = self._check_pos(pos)
        if rcut_pp is not None:
            rcut_pp = rcut_pp.contiguous().to(torch.float64)
        self._gen += 1
        C.call("dcpse_build_neighbors", self._h, _ptr(pos), pos.shape[0], float(rcut), _ptr(rcut_pp))
        self.n = pos.shape[0]

    def set_neighbors(self, rowptr, cols):
        rowptr = rowptr.contiguous().to(device="cuda", dtype=torch.int64)
        cols = cols.contiguous().to(device="cuda", dtype=torch.int32)
        n = rowptr.numel() - 1
        self._gen += 1
        C.call("dcpse_set_neighbors", self._h, n, cols.numel(), _ptr(rowptr), _ptr(cols))
        self.n = n

    def neighbors(self):
        """(rowptr, cols) as torch views of the plan's arrays."""
        rp, cl = ctypes.c_void_p(), ctypes.c_void_p()
        C.call("dcpse_neighbors_ptr", self._h, ctypes.byref(rp), ctypes.byref(cl))
        info = self.info()
        return (_view(rp.value, (info["n"] + 1,), torch.int64, self),
                _view(cl.value, (info["nnz"],), torch.int32, self))

    # -- assembly -------------------------------------------------------
    def assemble(self, pos, flags=C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32, eps_fixed=None,
                 allow_failed_particles=True):
        pos = self._check_pos(pos)
        self._check_rows(pos.shape[0], self.n, "positions")
        if eps_fixed is not None:
            eps_fixed = eps_fixed.contiguous().to(torch.float64)
            self._check_rows(eps_fixed.numel(), self.n, "eps_fixed")
        allow = (C.ERR_PARTICLES,) if allow_failed_particles else ()
        self._gen += 1
        return C.call("dcpse_assemble", self._h, _ptr(pos), _ptr(eps_fixed), int(flags), allow=allow)

    def gram_on_tensor_cores(self):
        """Whether the last assembly took its Gram products on the tensor cores."""
        v = ctypes.c_int()
        C.call("dcpse_plan_assembly_info", self._h, ctypes.byref(v))
        return bool(v.value)

    def particle_status(self):
        nb, fb, fc = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        C.call("dcpse_particle_status", self._h, ctypes.byref(nb), ctypes.byref(fb), ctypes.byref(fc))
        return nb.value, fb.value, fc.value

    def eps(self):
        e, s = ctypes.c_void_p(), ctypes.c_void_p()
        C.call("dcpse_eps_ptr", self._h, ctypes.byref(e), ctypes.byref(s))
        n = self.info()["n"]
        return _view(e.value, (n,), torch.float64, self), _view(s.value, (n,), torch.int32, self)

    def term_kernels(self, term):
        k, e = ctypes.c_void_p(), ctypes.c_void_p()
        C.call("dcpse_term_kernels_ptr", self._h, int(term), ctypes.byref(k), ctypes.byref(e))
        info = self.info()
        K = _view(k.value, (info["nnz"],), torch.float64, self) if k.value else None
        return K, _view(e.value, (info["n"],), torch.float64, self)

    def set_term_kernels(self, term, K, eps, eip):
        """Install kernels of one term (Dcpse::load): K [nnz], eps and
        eps^-|alpha| [n], host numpy or device tensors."""
        def dev(x):
            return torch.as_tensor(x, dtype=torch.float64).to("cuda").contiguous()
        K, eps, eip = dev(K), dev(eps), dev(eip)
        self._gen += 1
        C.call("dcpse_set_term_kernels", self._h, int(term), _ptr(K), _ptr(eps), _ptr(eip))

    def output_weights(self, output):
        w64, w32 = ctypes.c_void_p(), ctypes.c_void_p()
        C.call("dcpse_output_weights_ptr", self._h, int(output), ctypes.byref(w64), ctypes.byref(w32))
        nnz = self.info()["nnz"]
        return (_view(w64.value, (nnz,), torch.float64, self) if w64.value else None,
                _view(w32.value, (nnz,), torch.float32, self) if w32.value else None)

    # -- apply ----------------------------------------------------------
    def apply_term_f64(self, term, f, out=None):
        f = self._check_field(f)
        out = torch.empty_like(f) if out is None else self._check_out(out, f.shape)
        C.call("dcpse_apply_term_f64", self._h, int(term), _ptr(f), _ptr(out))
        return out

    def apply_output_f64(self, output, f, out=None):
        f = self._check_field(f)
        out = torch.empty_like(f) if out is None else self._check_out(out, f.shape)
        C.call("dcpse_apply_output_f64", self._h, int(output), _ptr(f), _ptr(out))
        return out

    def apply(self, f, precision=C.F32, out=None):
        """All outputs in one pass: returns a [n_outputs, n] float64 tensor."""
        f = self._check_field(f)
        if out is None:
            out = torch.empty((self.n_outputs, f.shape[0]), dtype=torch.float64, device=f.device)
        else:
            self._check_out(out, (self.n_outputs, f.shape[0]))
        C.call("dcpse_apply_batched", self._h, _ptr(f), _ptr(out), int(precision))
        return out

    def apply_host(self, f_host, out_host=None, precision=C.F32):
        """Host numpy arrays in and out (the copies are part of the call)."""
        f_host = np.ascontiguousarray(f_host, dtype=np.float64)
        if f_host.ndim != 1:
            raise ValueError("fields are float64 [n] arrays")
        self._check_rows(f_host.shape[0], self.n, "field")
        if out_host is None:
            out_host = np.empty((self.n_outputs, f_host.shape[0]), dtype=np.float64)
        elif (out_host.dtype != np.float64 or out_host.shape != (self.n_outputs, f_host.shape[0])
              or not out_host.flags.c_contiguous or not out_host.flags.writeable):
            raise ValueError("out_host must be a writeable C-contiguous float64 array of shape %s"
                             % ((self.n_outputs, f_host.shape[0]),))
        C.call("dcpse_apply_batched_host", self._h, f_host.ctypes.data_as(ctypes.c_void_p),
               out_host.ctypes.data_as(ctypes.c_void_p), int(precision))
        return out_host

    def set_error_budget(self, budget=1e-6, first_pass=C.F32):
        """Relative error budget per output of the F32_BUDGET applies (the
        FP32 result against the FP64 summed weights, normwise) and their
        first pass: C.F32 (FP32 weights alone) or C.F32_RESID (also the bf16
        residual streams, for sets where many rows would need correcting)."""
        C.call("dcpse_plan_set_error_budget", self._h, float(budget), int(first_pass))

    def budget_stats(self, reset=False):
        """(row, output) pairs the F32_BUDGET applies corrected in FP64 since
        the last reset."""
        n = ctypes.c_int64()
        C.call("dcpse_plan_budget_stats", self._h, ctypes.byref(n), int(bool(reset)))
        return n.value

    def set_reorder(self, policy=0):
        """Numbering of the apply's sliced layout: 0 automatic (cell order
        when the caller's numbering scatters the field reads), 1 always the
        cell order, -1 never."""
        C.call("dcpse_plan_set_reorder", self._h, int(policy))

    def set_reorder_order(self, order=0):
        """The renumbering order the next build_neighbors computes: 0 the
        Z-order of the list's cells, 1 row-major order of a grid at the
        particles' mean spacing."""
        C.call("dcpse_plan_set_reorder_order", self._h, int(order))

    def reorder_info(self):
        """(renumbered, mean |q - p| in the caller's numbering, the same in
        the cell order)."""
        r, a, b = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        C.call("dcpse_plan_reorder_info", self._h, ctypes.byref(r), ctypes.byref(a), ctypes.byref(b))
        return bool(r.value), a.value, b.value

    # -- particle to particle interpolation -----------------------------
    def _check_support_field(self, f):
        if f.dtype != torch.float64 or f.dim() not in (1, 2):
            raise ValueError("support fields are float64 [n_support] or [n_support, ncomp] CUDA tensors")
        sup = getattr(self, "_support", None)
        self._check_rows(f.shape[0], sup.shape[0] if sup is not None else self.n, "support field")
        return f.contiguous()

    def p2p_f64(self, term, f, out=None):
        """Dcpse::p2p of one term in the reference's order: eps^-|a| sum_q
        f_q K_pq on the domain rows; f is [n_support] or [n_support, ncomp]."""
        f = self._check_support_field(f)
        ncomp = 1 if f.dim() == 1 else f.shape[1]
        n = self.info()["n"]
        shape = (n,) if f.dim() == 1 else (n, ncomp)
        out = torch.empty(shape, dtype=torch.float64, device=f.device) if out is None else self._check_out(out, shape)
        C.call("dcpse_p2p_f64", self._h, int(term), _ptr(f), int(ncomp), _ptr(out))
        return out

    def p2p(self, f, precision=C.F32, out=None):
        """Every output's interpolation in one pass from the summed weights:
        [n_outputs, n] (or [n_outputs, n, ncomp] for vector fields)."""
        f = self._check_support_field(f)
        ncomp = 1 if f.dim() == 1 else f.shape[1]
        n = self.info()["n"]
        shape = (self.n_outputs, n) if f.dim() == 1 else (self.n_outputs, n, ncomp)
        out = torch.empty(shape, dtype=torch.float64, device=f.device) if out is None else self._check_out(out, shape)
        C.call("dcpse_p2p", self._h, _ptr(f), int(ncomp), _ptr(out), int(precision))
        return out

    # -- operator matrices ----------------------------------------------
    def operator_csr(self, output=0, coeff=1.0, rows=None, nvar=1, var=0):
        """CSR rows (value_nz order) of one output times coeff for the
        particles ``rows`` (int64 CUDA tensor; None = all) -> (rowptr int64
        [nrows+1], cols int64, vals float64) on the device; column index =
        particle * nvar + var."""
        if rows is not None:
            rows = rows.contiguous().to(device="cuda", dtype=torch.int64)
            nrows = rows.numel()
        else:
            nrows = self.info()["n"]
        rp = torch.empty(nrows + 1, dtype=torch.int64, device="cuda")
        nnz = ctypes.c_int64()
        args = (self._h, int(output), float(coeff), _ptr(rows), int(nrows), int(nvar), int(var), _ptr(rp))
        C.call("dcpse_operator_csr", *args, None, None, ctypes.byref(nnz))
        cols = torch.empty(max(nnz.value, 1), dtype=torch.int64, device="cuda")
        vals = torch.empty(max(nnz.value, 1), dtype=torch.float64, device="cuda")
        C.call("dcpse_operator_csr", *args, _ptr(cols), _ptr(vals), ctypes.byref(nnz))
        return rp, cols[: nnz.value], vals[: nnz.value]

    # -- adjoint --------------------------------------------------------
    def vjp_field(self, g, precision=C.F64, out=None):
        """sum_o L_o^T g_o for a cotangent g [n_outputs, n] -> [n]."""
        g = g.contiguous().to(torch.float64)
        if g.dim() == 1:
            g = g.unsqueeze(0)
        self._check_cotangent(g)
        out = torch.empty(g.shape[1], dtype=torch.float64, device=g.device) if out is None else \
            self._check_out(out, (g.shape[1],))
        C.call("dcpse_vjp_field", self._h, _ptr(g), _ptr(out), int(precision))
        return out

    def vjp_positions(self, pos, f, g, eps_fixed=None):
        """d/dpos of sum_o,p g[o,p] (L_o f)_p with the neighbour list fixed
        -> [n, dim] (FP64; pos must be the assembled positions)."""
        pos = self._check_pos(pos)
        self._check_rows(pos.shape[0], self.n, "positions")
        f = self._check_field(f)
        g = g.contiguous().to(torch.float64)
        if g.dim() == 1:
            g = g.unsqueeze(0)
        self._check_cotangent(g)
        if eps_fixed is not None:
            eps_fixed = eps_fixed.contiguous().to(torch.float64)
            self._check_rows(eps_fixed.numel(), self.n, "eps_fixed")
        grad = torch.empty_like(pos)
        C.call("dcpse_vjp_positions", self._h, _ptr(pos), _ptr(eps_fixed), _ptr(f), _ptr(g), _ptr(grad))
        return grad

    # -- timing ---------------------------------------------------------
    def set_timing(self, enable=True):
        C.call("dcpse_plan_set_timing", self._h, int(bool(enable)))

    def set_apply_config(self, lanes=0, mode=0):
        """lanes per row (0 = automatic, else 4/8/16/32); mode 0 = automatic
        (direct loads), 1 = direct loads, 2 = TMA-staged, 3 = direct loads in
        8-deep batches; | 16 = compensated sums for every output."""
        C.call("dcpse_plan_set_apply_config", self._h, int(lanes), int(mode))

    def set_assembly_config(self, bin_width=0, warps=4, qr_lanes=0):
        """Assembly schedule: neighbour-count bins of width bin_width (0 =
        index order), CTAs of 2/4/8 warps for the Gram and weight kernels,
        qr_lanes lanes per particle in the QR kernel (0 = automatic)."""
        C.call("dcpse_plan_set_assembly_config", self._h, int(bin_width), int(warps), int(qr_lanes))

    def check(self):
        """Synchronise; raise if a kernel's bounded device wait ran out."""
        C.call("dcpse_plan_check", self._h)

    def reset_timing(self):
        C.call("dcpse_plan_reset_timing", self._h)

    def timing(self, kernel):
        """(total device ms, launches) of a kernel id since the last reset."""
        ms, n = ctypes.c_double(), ctypes.c_int64()
        C.call("dcpse_plan_timing", self._h, int(kernel), ctypes.byref(ms), ctypes.byref(n))
        return ms.value, n.value

    # -- helpers --------------------------------------------------------
    def _check_pos(self, pos):
        if pos.dtype != torch.float64 or pos.dim() != 2 or pos.shape[1] != self.dim:
            raise ValueError("positions must be a float64 [n, %d] CUDA tensor" % self.dim)
        return pos.contiguous()

    def _check_field(self, f):
        if f.dtype != torch.float64 or f.dim() != 1:
            raise ValueError("fields are float64 [n] CUDA tensors")
        self._check_rows(f.shape[0], self.n, "field")
        return f.contiguous()

    # The C-ABI takes bare pointers sized by the plan's particle count, so
    # lengths are checked here: a short array would be read or written out of
    # bounds on the device.  (No list yet: the library reports the state.)
    @staticmethod
    def _check_rows(rows, n, what):
        if n is not None and n >= 0 and rows != n:
            raise ValueError("%s has %d rows, the plan's particle set has %d" % (what, rows, n))

    def _check_cotangent(self, g):
        if g.dim() != 2 or g.shape[0] != self.n_outputs:
            raise ValueError("cotangents are [n_outputs, n] = [%d, n] tensors" % self.n_outputs)
        self._check_rows(g.shape[1], self.n, "cotangent")

    @staticmethod
    def _check_out(out, shape):
        if out.dtype != torch.float64 or tuple(out.shape) != tuple(shape):
            raise ValueError("out must be a float64 tensor of shape %s, not %s %s"
                             % (tuple(shape), out.dtype, tuple(out.shape)))
        return out
