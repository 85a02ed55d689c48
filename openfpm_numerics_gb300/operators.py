"""Python mirror of openfpm_numerics' DC-PSE operator API.

Same names, constructor arguments and semantics as
src/DCPSE/DCPSE_op/DCPSE_op.hpp (Derivative_x_T ... Laplacian_T, Gradient_T,
Derivative_G_T; CPU aliases at :3485-3508, GPU aliases at :3510-3530):

    parts = ParticleSet(pos)                    # vector_dist stand-in (GPU)
    vl = parts.getVerlet(rCut)                  # getVerlet<VL_NON_SYMMETRIC|VL_SKIP_REF_PART>
    Lap = Laplacian(parts, vl, 2, rCut)         # assembles on the GPU
    d2f = Lap(f)                                # getV<1>(parts) = Lap(getV<0>(parts))
    Lap.update(parts)                           # after particles moved (initializeUpdate)

Calling an operator applies it in FP64 in the reference's operation order
(bit-exact with the CPU oracle).  ``op(f, precision="f32")`` uses the batched
FP32-weight path instead, ``"f32-pair"`` the FP32 weight pairs (FP64-class
results off the FP64 pipe) and ``"f64-batched"`` the batched FP64 apply.  Errors follow the reference: too few neighbours
raise ``ValueError`` (std::length_error in Vandermonde.hpp:109-112) unless the
operator was built with ``allow_failed_particles=True``.
"""
from __future__ import annotations

import enum

import numpy as np

import torch

from . import _capi as C
from .plan import DcpsePlan

# what the operators store at assembly: the reference's per-term kernels, the
# summed FP64 and FP32 weights and the FP32 residuals of the weight pairs
_OP_FLAGS = C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32 | C.STORE_OUT_F32_CORR
# the batched applies by name
_BATCHED = {"f32": C.F32, "f32-pair": C.F32_PAIR, "f64-batched": C.F64}
_PREC_MSG = "precision must be 'f64', 'f64-batched', 'f32' or 'f32-pair'"

dcpse_oversampling_factor = 1.9  # DCPSE_op.hpp:20
rcut_verlet = 3.1                # DCPSE_op.hpp:21


class support_options(enum.IntEnum):
    """src/DCPSE/SupportBuilder.hpp:13-19"""
    RADIUS = 0
    LOAD = 1
    ADAPTIVE = 2
    AT_LEAST_N_PARTICLES = 3


# Verlet-list options of openfpm's vector_dist::getVerlet<opt> that decide
# the DC-PSE supports (flag values are this mirror's own)
VL_NON_SYMMETRIC = 1
VL_SKIP_REF_PART = 2


class VerletList:
    """Neighbour lists in CSR form (rowptr int64 [n+1], cols int32), built on
    the device: every q with |x_p - x_q|^2 < rCut^2 in ascending q, without
    q == p when VL_SKIP_REF_PART is set.  With ``support`` the rows are the
    particles of ``parts`` and the columns those of ``support``
    (createVerletTwoPhase)."""

    def __init__(self, parts, rCut, rcut_pp=None, opt=VL_NON_SYMMETRIC | VL_SKIP_REF_PART, support=None):
        self.rCut = float(rCut)
        self.support = support
        self.skip_ref = bool(opt & VL_SKIP_REF_PART) and support is None
        self.rcut_pp = rcut_pp
        plan = DcpsePlan(parts.dims, [[(1,) + (0,) * (parts.dims - 1)]], box=parts.box)
        if support is not None:
            plan.set_support(support.getPosTensor())
        else:
            plan.set_support(None, self_skip=bool(opt & VL_SKIP_REF_PART))
        plan.build_neighbors(parts.getPosTensor(), self.rCut, rcut_pp)
        rp, cl = plan.neighbors()
        self.rowptr = rp.clone()
        self.cols = cl.clone()
        plan.close()

    def getNNPart(self, p):
        return int(self.rowptr[p + 1] - self.rowptr[p])

    def get(self, p, j):
        return int(self.cols[int(self.rowptr[p]) + j])


class ParticleSet:
    """Minimal stand-in for openfpm's vector_dist on one GPU: positions as a
    float64 [n, dim] CUDA tensor, optional box with periodicity, and named
    properties."""

    def __init__(self, pos, box=None, periodic=None):
        if not isinstance(pos, torch.Tensor):
            pos = torch.as_tensor(pos, dtype=torch.float64)
        self.pos = pos.to(device="cuda", dtype=torch.float64).contiguous()
        self.dims = self.pos.shape[1]
        self.box = None
        if box is not None:
            lo, hi = box
            self.box = (tuple(lo), tuple(hi), tuple(periodic) if periodic is not None else (0,) * self.dims)
        self.props = {}
        self._map_ctr = 0

    def size_local(self):
        return self.pos.shape[0]

    def getPosTensor(self):
        return self.pos

    def getPos(self, p):
        return self.pos[p]

    def setPos(self, pos):
        self.pos = pos.to(device="cuda", dtype=torch.float64).contiguous()
        self._map_ctr += 1

    def getVerlet(self, rCut, opt=VL_NON_SYMMETRIC | VL_SKIP_REF_PART):
        return VerletList(self, rCut, opt=opt)

    def ghost_get_subset(self):
        """No-op: a single GPU holds all particles; periodic images are
        handled by minimum-image offsets."""


def _unit(dim, axis, power=1):
    return tuple(power if d == axis else 0 for d in range(dim))


class _DcpseOp:
    """Common machinery: one plan holding the operator's reference terms."""

    _kind = None  # "single" | "sum" | "vector"
    # True for the *_gpu classes: the terms follow the reference's Dcpse_gpu
    _gpu_semantics = False

    def __init__(self, parts, verletList, ord, rCut, opt=support_options.RADIUS, *, outputs, kind,
                 allow_failed_particles=False, h_over_eps=0.9):
        if opt not in (support_options.RADIUS, support_options.LOAD):
            raise NotImplementedError("support option %r" % (opt,))
        if self._gpu_semantics:
            h_over_eps = 0.5  # eps = 2 <h> (Dcpse.cuh:799-807); Dcpse_gpu has no HOverEpsilon
        self.dim = parts.dims
        self.ord = int(ord)
        self.rCut = float(rCut)
        self._outputs = outputs
        self._kind = kind
        self._allow = allow_failed_particles
        self.HOverEpsilon = h_over_eps
        self.verletList = verletList
        self.plan = DcpsePlan(self.dim, outputs, order=self.ord, h_over_eps=h_over_eps, box=parts.box)
        self._assembled = False
        self._prepare(parts)
        if opt == support_options.RADIUS:
            self._assemble(parts)

    def _prepare(self, parts):
        """Hand the neighbour list to the plan (before every assembly).  A
        *_gpu operator builds its own support from rCut, as the reference's
        SupportBuilderGPU does (SupportBuilder.cuh:14-107: |x_p - x_q| <
        rCut, p excluded), and ignores the list it was given."""
        if self._gpu_semantics:
            self.verletList = VerletList(parts, self.rCut)
        self.plan.set_neighbors(self.verletList.rowptr, self.verletList.cols)

    def _assemble(self, parts):
        rc = self.plan.assemble(parts.getPosTensor(), _OP_FLAGS)
        if rc == C.ERR_PARTICLES and not self._allow:
            nb, first, code = self.plan.particle_status()
            if code == C.PART_TOO_FEW:
                raise ValueError("Not enough neighbour points passed for Vandermonde matrix construction! "
                                 "(%d particles, first %d)" % (nb, first))
            raise RuntimeError("DC-PSE assembly failed for %d particles (first %d, status %d)" % (nb, first, code))
        self._assembled = True

    def update(self, parts, verletList=None):
        """initializeUpdate (Dcpse.hpp:675-687): re-assemble after particles
        moved; pass the updated Verlet list (the reference requires
        updateVerlet first)."""
        if verletList is not None:
            self.verletList = verletList
        self._prepare(parts)
        self._assemble(parts)

    def deallocate(self, parts=None):
        self.plan.close()

    # Dcpse::save / load (Dcpse.hpp:302-379) through the operators'
    # save(parts, file) / load(parts, file) (DCPSE_op.hpp:759-773): one file
    # per term, file + "_0" for an operator of one term (the reference's
    # name), file + "_term<t>_0" for each term of a sum or vector operator
    def _term_file(self, file, t):
        return file + "_0" if self.plan.n_terms == 1 else "%s_term%d_0" % (file, t)

    def save(self, parts, file):
        from . import kernel_file

        eps = self.plan.eps()[0].cpu().numpy()
        offsets = self.verletList.rowptr[:-1].cpu().numpy().astype(np.uint64)
        for t in range(self.plan.n_terms):
            K, eip = self.plan.term_kernels(t)
            kernel_file.write(self._term_file(file, t), eps, eip.cpu().numpy(), K.cpu().numpy(), offsets)

    def load(self, parts, file):
        from . import kernel_file

        rp = self.verletList.rowptr.cpu().numpy()
        data = []
        for t in range(self.plan.n_terms):
            eps, eip, K, offsets = kernel_file.read(self._term_file(file, t))
            if (eps.size != rp.size - 1 or eip.size != eps.size or K.size != rp[-1]
                    or not np.array_equal(offsets, rp[:-1].astype(np.uint64))):
                raise ValueError("%s does not match this operator's neighbour list" % self._term_file(file, t))
            data.append((K, eps, eip))
        for t, (K, eps, eip) in enumerate(data):
            self.plan.set_term_kernels(t, K, eps, eip)
        self._assembled = True

    def __call__(self, f, precision="f64"):
        if not self._assembled:
            raise RuntimeError("operator not assembled (support_options.LOAD without update)")
        if isinstance(f, str):
            raise TypeError("pass the field tensor")
        f = f.to(device="cuda", dtype=torch.float64).contiguous()
        if precision == "f64":
            res = [self.plan.apply_output_f64(o, f) for o in range(len(self._outputs))]
            out = torch.stack(res) if len(res) > 1 else res[0]
        elif precision in _BATCHED:
            out = self.plan.apply(f, _BATCHED[precision])
            out = out if len(self._outputs) > 1 else out[0]
        else:
            raise ValueError(_PREC_MSG)
        return out

    # accessors of the reference (Dcpse.hpp:507-550), for the first term
    def getNumNN(self, p):
        return self.verletList.getNNPart(p)

    def getIndexNN(self, p, j):
        return self.verletList.get(p, j)

    def getCoeffNN(self, p, j, term=0):
        K, _ = self.plan.term_kernels(term)
        return float(K[int(self.verletList.rowptr[p]) + j])

    def getEpsilonInvPrefactor(self, p, term=0):
        _, eip = self.plan.term_kernels(term)
        return float(eip[p])

    def getSign(self, term=0):
        order = sum(self._outputs_flat()[term])
        return -1.0 if (order % 2 == 0 and order != 0) else 1.0

    def _outputs_flat(self):
        return [s for o in self._outputs for s in o]


class Derivative_G(_DcpseOp):
    """Derivative_G_T (DCPSE_op.hpp:3387-3482): arbitrary signature p."""

    def __init__(self, parts, verletList, ord, rCut, p, opt=support_options.RADIUS, **kw):
        super().__init__(parts, verletList, ord, rCut, opt, outputs=[[tuple(p)]], kind="single", **kw)


def _single(name, sig_fn, ref):
    def init(self, parts, verletList, ord, rCut, opt=support_options.RADIUS, **kw):
        _DcpseOp.__init__(self, parts, verletList, ord, rCut, opt, outputs=[[sig_fn(parts.dims)]], kind="single",
                          **kw)

    return type(name, (_DcpseOp,), {"__init__": init, "__doc__": "%s (%s)" % (name, ref)})


Derivative_x = _single("Derivative_x", lambda d: _unit(d, 0), "DCPSE_op.hpp:649-797")
Derivative_y = _single("Derivative_y", lambda d: _unit(d, 1), "DCPSE_op.hpp:799-941")
Derivative_z = _single("Derivative_z", lambda d: _unit(d, 2), "DCPSE_op.hpp:943-1079")
Derivative_xx = _single("Derivative_xx", lambda d: _unit(d, 0, 2), "DCPSE_op.hpp:2216-2358")
Derivative_yy = _single("Derivative_yy", lambda d: _unit(d, 1, 2), "DCPSE_op.hpp:2360-2502")
Derivative_zz = _single("Derivative_zz", lambda d: _unit(d, 2, 2), "DCPSE_op.hpp:2504-2634")
Derivative_xy = _single("Derivative_xy", lambda d: tuple(1 if i < 2 else 0 for i in range(d)),
                        "DCPSE_op.hpp:1783-1925")
Derivative_yz = _single("Derivative_yz", lambda d: tuple(1 if i in (1, 2) else 0 for i in range(d)),
                        "DCPSE_op.hpp:1927-2069")
Derivative_xz = _single("Derivative_xz", lambda d: tuple(1 if i in (0, 2) else 0 for i in range(d)),
                        "DCPSE_op.hpp:2071-2214")
Derivative_xxx = _single("Derivative_xxx", lambda d: _unit(d, 0, 3), "DCPSE_op.hpp:2636-2774")
Derivative_yyy = _single("Derivative_yyy", lambda d: _unit(d, 1, 3), "DCPSE_op.hpp:3056-3192")
Derivative_xxy = _single("Derivative_xxy", lambda d: tuple({0: 2, 1: 1}.get(i, 0) for i in range(d)),
                         "DCPSE_op.hpp:2776-2914")
Derivative_yyx = _single("Derivative_yyx", lambda d: tuple({0: 1, 1: 2}.get(i, 0) for i in range(d)),
                         "DCPSE_op.hpp:2916-3054")
Derivative_xxxx = _single("Derivative_xxxx", lambda d: _unit(d, 0, 4), "DCPSE_op.hpp:3194-3256")
Derivative_yyyy = _single("Derivative_yyyy", lambda d: _unit(d, 1, 4), "DCPSE_op.hpp:3258-3320")
Derivative_xxyy = _single("Derivative_xxyy", lambda d: tuple({0: 2, 1: 2}.get(i, 0) for i in range(d)),
                          "DCPSE_op.hpp:3322-3385")


class Laplacian(_DcpseOp):
    """Laplacian_T (DCPSE_op.hpp:1350-1500): sum of dim Dcpse objects with
    signatures 2e_i, evaluated as VECT_DCPSE_V_SUM (:388-399)."""

    def __init__(self, parts, verletList, ord, rCut, opt=support_options.RADIUS, **kw):
        d = parts.dims
        super().__init__(parts, verletList, ord, rCut, opt, outputs=[[_unit(d, i, 2) for i in range(d)]],
                         kind="sum", **kw)


class Gradient(_DcpseOp):
    """Gradient_T (DCPSE_op.hpp:1081-1224): dim Dcpse objects e_i evaluated as
    VECT_DCPSE_V (:144-153); the result is a [dim, n] tensor."""

    def __init__(self, parts, verletList, ord, rCut, opt=support_options.RADIUS, **kw):
        d = parts.dims
        super().__init__(parts, verletList, ord, rCut, opt, outputs=[[_unit(d, i)] for i in range(d)],
                         kind="vector", **kw)


class Divergence(_DcpseOp):
    """Divergence_T (DCPSE_op.hpp:1503-1630): dim Dcpse objects e_i applied
    to the components of a vector field and summed, VECT_DCPSE_V_DIV
    (:446-475): div = ((0 + D_0 v_0) + D_1 v_1) + ..."""

    def __init__(self, parts, verletList, ord, rCut, opt=support_options.RADIUS, **kw):
        d = parts.dims
        super().__init__(parts, verletList, ord, rCut, opt, outputs=[[_unit(d, i)] for i in range(d)],
                         kind="div", **kw)

    def __call__(self, v, precision="f64"):
        if not self._assembled:
            raise RuntimeError("operator not assembled (support_options.LOAD without update)")
        v = v.to(device="cuda", dtype=torch.float64)
        out = torch.zeros(v.shape[0], dtype=torch.float64, device=v.device)
        for i in range(self.dim):
            out = out + self._component(i, v[:, i].contiguous(), precision)
        return out

    def _component(self, i, f, precision):
        if precision == "f64":
            return self.plan.apply_output_f64(i, f)
        if precision in _BATCHED:
            return self.plan.apply(f, _BATCHED[precision])[i]
        raise ValueError(_PREC_MSG)


class Advection(Divergence):
    """Advection_T (DCPSE_op.hpp:1632-1781): (v . grad) f with dim Dcpse
    objects e_i, VECT_DCPSE_V_DOT (:531-565): adv = ((0 + v_0 D_0 f) +
    v_1 D_1 f) + ...; f may be a vector field [n, m] (component-wise)."""

    def __call__(self, v, f, precision="f64"):
        if not self._assembled:
            raise RuntimeError("operator not assembled (support_options.LOAD without update)")
        v = v.to(device="cuda", dtype=torch.float64)
        f = f.to(device="cuda", dtype=torch.float64)
        cols = [f] if f.dim() == 1 else [f[:, c].contiguous() for c in range(f.shape[1])]
        res = []
        for fc in cols:
            out = torch.zeros(v.shape[0], dtype=torch.float64, device=v.device)
            for i in range(self.dim):
                out = out + v[:, i] * self._component(i, fc.contiguous(), precision)
            res.append(out)
        return res[0] if f.dim() == 1 else torch.stack(res, 1)


class Curl2D(_DcpseOp):
    """Curl2D_T (DCPSE_op.hpp:1227-1340): Dcpse objects e_1 and e_0,
    VECT_DCPSE_V_CURL2D (:206-233): (D_y f, -D_x f) as a [2, n] tensor."""

    def __init__(self, parts, verletList, ord, rCut, opt=support_options.RADIUS, **kw):
        d = parts.dims
        super().__init__(parts, verletList, ord, rCut, opt, outputs=[[_unit(d, 1)], [_unit(d, 0)]],
                         kind="vector", **kw)

    def __call__(self, f, precision="f64"):
        out = _DcpseOp.__call__(self, f, precision)
        return torch.stack([out[0], -out[1]])


class OperatorSet(_DcpseOp):
    """Several operators assembled and applied together over one neighbour
    list (one persistent assembly launch, one apply pass).  ``ops`` is a list
    of operator names ('x','y','z','xx',...,'laplacian','gradient')."""

    def __init__(self, parts, verletList, ord, rCut, ops, opt=support_options.RADIUS, **kw):
        d = parts.dims
        outs = []
        for name in ops:
            if name == "laplacian":
                outs.append([_unit(d, i, 2) for i in range(d)])
            elif name == "gradient":
                outs.extend([[_unit(d, i)] for i in range(d)])
            else:
                axes = {"x": 0, "y": 1, "z": 2}
                sig = [0] * d
                for ch in name:
                    sig[axes[ch]] += 1
                outs.append([tuple(sig)])
        super().__init__(parts, verletList, ord, rCut, opt, outputs=outs, kind="vector", **kw)


class _SurfaceOp(_DcpseOp):
    """Surface DC-PSE operator (SurfaceDcpse, Dcpse.hpp:829-1085): the
    support of every particle is extended by nCount virtual particles on each
    side along its normal, the operator is assembled on the extended support
    and the virtual particles' kernels are added onto their surface particle.
    The Verlet list passed in gives the cutoff (its rCut, or per-particle
    radii) and whether a particle is its own neighbour; like the reference,
    the operator replaces its lists with the accumulated ones."""

    def __init__(self, parts, verletList, ord, rCut, nSpacing, nCount, opt=support_options.RADIUS, *, sig,
                 normal, **kw):
        if opt not in (support_options.RADIUS, support_options.LOAD, support_options.ADAPTIVE):
            raise NotImplementedError("support option %r" % (opt,))
        self.nSpacing = float(nSpacing)
        self.nCount = int(nCount)
        self.normal = normal
        self._adaptive = opt == support_options.ADAPTIVE
        if self._adaptive and verletList.rcut_pp is None:
            raise ValueError("support_options.ADAPTIVE needs a Verlet list with per-particle radii")
        _DcpseOp.__init__(self, parts, verletList, ord, rCut,
                          support_options.LOAD if opt == support_options.LOAD else support_options.RADIUS,
                          outputs=[[tuple(sig)]], kind="single", **kw)

    def _prepare(self, parts):
        normals = parts.props[self.normal]
        spacings = None
        if self._adaptive:
            # nSpacing_p = property 0 / nCount (Dcpse.hpp:1057-1066)
            spacings = parts.props[0].to(torch.float64) / self.nCount
        self.plan.set_support(None, self_skip=self.verletList.skip_ref)
        self.plan.set_surface(normals, self.nCount, self.nSpacing, spacings)
        rpp = self.verletList.rcut_pp
        self.plan.build_neighbors(parts.getPosTensor(), self.verletList.rCut if rpp is None else 0.0, rpp)

    def _assemble(self, parts):
        _DcpseOp._assemble(self, parts)
        rp, cl = self.plan.neighbors()
        self.verletList.rowptr = rp.clone()
        self.verletList.cols = cl.clone()


def _surface(name, sig_fn, ref):
    def init(self, parts, verletList, ord, rCut, nSpacing, nCount, opt=support_options.RADIUS, *, normal, **kw):
        _SurfaceOp.__init__(self, parts, verletList, ord, rCut, nSpacing, nCount, opt, sig=sig_fn(parts.dims),
                            normal=normal, **kw)

    return type(name, (_SurfaceOp,), {"__init__": init, "__doc__": "%s (%s); normal = property holding the "
                                                                   "unit normals (NORMAL_ID)" % (name, ref)})


SurfaceDerivative_x = _surface("SurfaceDerivative_x", lambda d: _unit(d, 0), "DCPSE_surface_op.hpp:11-109")
SurfaceDerivative_y = _surface("SurfaceDerivative_y", lambda d: _unit(d, 1), "DCPSE_surface_op.hpp:125-209")
SurfaceDerivative_z = _surface("SurfaceDerivative_z", lambda d: _unit(d, 2), "DCPSE_surface_op.hpp:225-309")
SurfaceDerivative_xx = _surface("SurfaceDerivative_xx", lambda d: _unit(d, 0, 2), "DCPSE_surface_op.hpp:426-509")
SurfaceDerivative_yy = _surface("SurfaceDerivative_yy", lambda d: _unit(d, 1, 2), "DCPSE_surface_op.hpp:525-607")
SurfaceDerivative_zz = _surface("SurfaceDerivative_zz", lambda d: _unit(d, 2, 2), "DCPSE_surface_op.hpp:623-706")
SurfaceDerivative_xy = _surface("SurfaceDerivative_xy", lambda d: tuple(1 if i < 2 else 0 for i in range(d)),
                                "DCPSE_surface_op.hpp:709-819")
SurfaceDerivative_yz = _surface("SurfaceDerivative_yz", lambda d: tuple(1 if i in (1, 2) else 0 for i in range(d)),
                                "DCPSE_surface_op.hpp:821-919")
SurfaceDerivative_xz = _surface("SurfaceDerivative_xz", lambda d: tuple(1 if i in (0, 2) else 0 for i in range(d)),
                                "DCPSE_surface_op.hpp:921-1020")
# the reference builds Laplace_Beltrami as one Dcpse of signature (2, 2, 2)
# (DCPSE_surface_op.hpp:326-347), kept as is
Laplace_Beltrami = _surface("Laplace_Beltrami", lambda d: (2,) * d, "DCPSE_surface_op.hpp:326-410")


class SurfaceDerivative_G(_SurfaceOp):
    """SurfaceDerivative_G (DCPSE_surface_op.hpp:1022-1100): signature p."""

    def __init__(self, parts, verletList, ord, rCut, nSpacing, nCount, p, opt=support_options.RADIUS, *, normal,
                 **kw):
        super().__init__(parts, verletList, ord, rCut, nSpacing, nCount, opt, sig=tuple(p), normal=normal, **kw)


def createVerletTwoPhase(particlesDomain, particlesSupport, rCut, cellList=None):
    """Lists of the support particles within rCut of every domain particle
    (openfpm's createVerletTwoPhase, used by the two-set tests of
    DCPSE_op_test_base_tests.cpp:369-372).  The cell list argument of the
    reference is accepted and ignored: the lists are built on the device."""
    return VerletList(particlesDomain, rCut, support=particlesSupport)


class PPInterpolation:
    """PPInterpolation (src/DCPSE/DcpseInterpolation.hpp:28-195): DC-PSE
    particle to particle interpolation from particlesSupport to
    particlesDomain, i.e. a Dcpse with signature 0 on two particle sets
    (Dcpse.hpp:113-131) evaluated by p2p (Dcpse.hpp:198-297).

        Fx = PPInterpolation(support, domain, verletList, 2, rCut)
        Fx.p2p(0, 1)        # domain.props[1] = interpolation of support.props[0]
        g = Fx(f_support)   # the same on tensors

    The neighbour list rows are the domain particles, the columns the support
    particles (createVerletTwoPhase, or getVerlet of one set that is both)."""

    def __init__(self, particlesSupport, particlesDomain, verletList, ord, rCut, opt=support_options.RADIUS,
                 *, allow_failed_particles=False, h_over_eps=0.9, nSpacing=None, isSurfaceInterpolation=False,
                 normal=None):
        """With isSurfaceInterpolation=True (the reference's surface
        constructor, DcpseInterpolation.hpp:94-113) the support particles are
        extended along their normals (property ``normal`` of the support
        set) with nCount = int(rCut / nSpacing) virtual particles per side."""
        if opt not in (support_options.RADIUS, support_options.LOAD):
            raise NotImplementedError("support option %r" % (opt,))
        self._surface = bool(isSurfaceInterpolation)
        if self._surface and (nSpacing is None or normal is None):
            raise ValueError("surface interpolation needs nSpacing and the normal property")
        self.nSpacing = None if nSpacing is None else float(nSpacing)
        self.normal = normal
        self.particlesSupport = particlesSupport
        self.particlesDomain = particlesDomain
        self.verletList = verletList
        self.dim = particlesDomain.dims
        self.ord = int(ord)
        self.rCut = float(rCut)
        self._allow = allow_failed_particles
        self.plan = DcpsePlan(self.dim, [[(0,) * self.dim]], order=self.ord, h_over_eps=h_over_eps,
                              box=particlesDomain.box)
        self._assembled = False
        if opt == support_options.RADIUS:
            self.update()

    def update(self, verletList=None):
        """initializeUpdate(particlesSupport, particlesDomain)
        (DcpseInterpolation.hpp:187-190): re-assemble on the current positions."""
        if verletList is not None:
            self.verletList = verletList
        two = self.particlesSupport is not self.particlesDomain
        self.plan.set_support(self.particlesSupport.getPosTensor() if two else None,
                              self_skip=getattr(self.verletList, "skip_ref", False))
        if self._surface:
            n_count = int(self.rCut / self.nSpacing)
            self.plan.set_surface(self.particlesSupport.props[self.normal], n_count, self.nSpacing)
            self.plan.build_neighbors(self.particlesDomain.getPosTensor(), self.verletList.rCut)
        else:
            self.plan.set_neighbors(self.verletList.rowptr, self.verletList.cols)
        rc = self.plan.assemble(self.particlesDomain.getPosTensor(), _OP_FLAGS)
        if rc == C.ERR_PARTICLES and not self._allow:
            nb, first, code = self.plan.particle_status()
            if code == C.PART_TOO_FEW:
                raise ValueError("Not enough neighbour points passed for Vandermonde matrix construction! "
                                 "(%d particles, first %d)" % (nb, first))
            raise RuntimeError("DC-PSE assembly failed for %d particles (first %d, status %d)" % (nb, first, code))
        if self._surface:
            rp, cl = self.plan.neighbors()
            self.verletList.rowptr = rp.clone()
            self.verletList.cols = cl.clone()
        self._assembled = True

    def __call__(self, f, precision="f64"):
        """Interpolated field on the domain set: f is [n_support] or
        [n_support, N1] (vector property, p2p<prp1,prp2,N1>)."""
        if not self._assembled:
            raise RuntimeError("operator not assembled (support_options.LOAD without update)")
        f = f.to(device="cuda", dtype=torch.float64).contiguous()
        if precision == "f64":
            return self.plan.p2p_f64(0, f)
        if precision in ("f32", "f64-batched"):
            return self.plan.p2p(f, C.F32 if precision == "f32" else C.F64)[0]
        raise ValueError("precision must be 'f64', 'f64-batched' or 'f32'")

    def p2p(self, propSupport, propDomain, N1=None):
        """p2p<propSupport, propDomain>() and p2p<propSupport, propDomain, N1>()
        (DcpseInterpolation.hpp:133-160) on the sets' named properties."""
        f = self.particlesSupport.props[propSupport]
        if N1 is not None and (f.dim() != 2 or f.shape[1] != N1):
            raise ValueError("property %r is not a vector of %d components" % (propSupport, N1))
        self.particlesDomain.props[propDomain] = self(f)

    def deallocate(self):
        self.plan.close()


def _gpu_class(cls):
    """The reference's cls_gpu (DCPSE_op.hpp:3510-3530: cls_T over Dcpse_gpu).
    Dcpse_gpu (Dcpse.cuh:563-875) differs from Dcpse in what it computes:
    eps = 2 <h> instead of <h> / 0.9, and the support is built from rCut by
    the class itself.  Its moment systems are solved by an unpivoted batched
    LU; here they go through the same column-pivoting QR as every other
    operator, which gives the same kernels up to the systems' conditioning."""
    return type(cls.__name__ + "_gpu", (cls,), {"_gpu_semantics": True, "__doc__": _gpu_class.__doc__,
                                                "__module__": __name__})


Derivative_x_gpu, Derivative_y_gpu, Derivative_z_gpu = map(_gpu_class, (Derivative_x, Derivative_y, Derivative_z))
Derivative_xx_gpu, Derivative_yy_gpu, Derivative_zz_gpu = map(_gpu_class, (Derivative_xx, Derivative_yy,
                                                                           Derivative_zz))
Derivative_xy_gpu, Derivative_yz_gpu, Derivative_xz_gpu = map(_gpu_class, (Derivative_xy, Derivative_yz,
                                                                           Derivative_xz))
Laplacian_gpu, Gradient_gpu, Derivative_G_gpu = map(_gpu_class, (Laplacian, Gradient, Derivative_G))
Divergence_gpu, Advection_gpu, Curl2D_gpu = map(_gpu_class, (Divergence, Advection, Curl2D))
Derivative_xxx_gpu, Derivative_xxy_gpu = map(_gpu_class, (Derivative_xxx, Derivative_xxy))
Derivative_yyx_gpu, Derivative_yyy_gpu = map(_gpu_class, (Derivative_yyx, Derivative_yyy))
