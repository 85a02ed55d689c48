"""RK4 time stepping with DC-PSE operators (the role of boost::numeric::odeint
runge_kutta4 over openfpm state types in src/OdeIntegrators).

* ``runge_kutta4(rhs, y, t, dt)``: one classic RK4 step of any right-hand
  side written with plan applies and torch arithmetic (odeint's do_step).
* ``GrayScottRK4``: the two-species Gray-Scott system with the fused stage
  kernels of the C-ABI (``dcpse_rk4_gs_stage``: Laplacian gathers of both
  species, reaction terms and stage update in one launch), steps captured in
  a CUDA graph, and a checkpointed adjoint (``dcpse_rk4_gs_adjoint_stage``)
  for gradients of a final-state functional with respect to an earlier state.
"""
from __future__ import annotations

import ctypes

import torch

from . import _capi as C


def runge_kutta4(rhs, y, t, dt):
    """y(t + dt) from y(t) for dy/dt = rhs(y, t); y a tensor or a tuple."""
    tup = isinstance(y, (tuple, list))
    Y = tuple(y) if tup else (y,)

    def R(state, tt):
        r = rhs(state if tup else state[0], tt)
        return tuple(r) if tup else (r,)

    k1 = R(Y, t)
    k2 = R(tuple(a + 0.5 * dt * b for a, b in zip(Y, k1)), t + 0.5 * dt)
    k3 = R(tuple(a + 0.5 * dt * b for a, b in zip(Y, k2)), t + 0.5 * dt)
    k4 = R(tuple(a + dt * b for a, b in zip(Y, k3)), t + dt)
    out = tuple(a + (dt / 6.0) * (b1 + 2 * b2 + 2 * b3 + b4) for a, b1, b2, b3, b4 in zip(Y, k1, k2, k3, k4))
    return out if tup else out[0]


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class GrayScottRK4:
    """du = Du L u - u v^2 + F (1 - u), dv = Dv L v + u v^2 - (F + k) v with
    L = output 0 of ``plan`` (a Laplacian, assembled with FP32 weights for
    float32 state or FP64 output weights for float64 state)."""

    def __init__(self, plan, u, v, Du, Dv, F, k, dt):
        self.plan = plan
        self.dtype = u.dtype
        self.prec = C.F32 if u.dtype == torch.float32 else C.F64
        self.u, self.v = u.contiguous().clone(), v.contiguous().clone()
        self.params = (ctypes.c_double * 5)(Du, Dv, F, k, dt)
        self.dt = dt
        z = lambda: torch.empty_like(self.u)  # noqa: E731
        self.Ya, self.Yb, self.acc = (z(), z()), (z(), z()), (z(), z())
        self.graph = None
        self.graph_steps = 0

    # ------------------------------------------------------------ forward --
    def _stage(self, s, Y, out):
        C.call("dcpse_rk4_gs_stage", self.plan._h, s, self.prec, _vp(Y[0]), _vp(Y[1]), _vp(self.u), _vp(self.v),
               _vp(self.acc[0]), _vp(self.acc[1]), _vp(out[0]), _vp(out[1]), self.params)

    def step(self, record=None):
        """One RK4 step in place; record = 4 (u, v) buffers receiving Y1..Y4."""
        y = (self.u, self.v)
        if record is not None:
            record[0][0].copy_(self.u)
            record[0][1].copy_(self.v)
            self._stage(0, y, record[1])
            self._stage(1, record[1], record[2])
            self._stage(2, record[2], record[3])
            self._stage(3, record[3], y)
        else:
            self._stage(0, y, self.Ya)
            self._stage(1, self.Ya, self.Yb)
            self._stage(2, self.Yb, self.Ya)
            self._stage(3, self.Ya, y)

    def capture(self, steps, stream):
        """Capture `steps` steps in one CUDA graph on `stream` (which must be
        the plan's stream); replay with run()."""
        self.graph = torch.cuda.CUDAGraph()
        self.graph_steps = steps
        with torch.cuda.stream(stream):
            self.step()  # warm-up outside capture
            torch.cuda.current_stream().synchronize()
            with torch.cuda.graph(self.graph, stream=stream):
                for _ in range(steps):
                    self.step()

    def run(self, steps):
        if self.graph is not None and steps % self.graph_steps == 0:
            for _ in range(steps // self.graph_steps):
                self.graph.replay()
        else:
            for _ in range(steps):
                self.step()

    # ------------------------------------------------------------ adjoint --
    def prepare_adjoint(self):
        C.call("dcpse_rk4_gs_adjoint_prepare", self.plan._h, self.prec)

    def _adj_stage(self, Y, kb, yb, acc, nxt, cy, cY):
        C.call("dcpse_rk4_gs_adjoint_stage", self.plan._h, self.prec, _vp(Y[0]), _vp(Y[1]), _vp(kb[0]), _vp(kb[1]),
               _vp(yb[0]), _vp(yb[1]), _vp(acc[0]), _vp(acc[1]), _vp(nxt[0]) if nxt else None,
               _vp(nxt[1]) if nxt else None, float(cy), float(cY), self.params)

    def reverse_step(self, stages, ybar):
        """ybar of y_n from ybar of y_{n+1} and the step's stage states."""
        dt = self.dt
        acc = (ybar[0].clone(), ybar[1].clone())
        k_a = ((dt / 6.0) * ybar[0], (dt / 6.0) * ybar[1])
        k_b = (torch.empty_like(ybar[0]), torch.empty_like(ybar[1]))
        self._adj_stage(stages[3], k_a, ybar, acc, k_b, dt / 3.0, dt)        # Ybar4 -> kbar3
        self._adj_stage(stages[2], k_b, ybar, acc, k_a, dt / 3.0, dt / 2.0)  # Ybar3 -> kbar2
        self._adj_stage(stages[1], k_a, ybar, acc, k_b, dt / 6.0, dt / 2.0)  # Ybar2 -> kbar1
        self._adj_stage(stages[0], k_b, ybar, acc, None, 0.0, 0.0)           # Ybar1
        return acc

    def _reverse_step_into(self, stages, yb, acc, k_a=None, k_b=None):
        """reverse_step with preallocated buffers: yb (ybar of y_{n+1}) is
        replaced by ybar of y_n (one fused call: the four adjoint stages with
        their kbar scalings and copies; k_a and k_b are not needed)."""
        ptrs = (ctypes.c_void_p * 8)(*[_vp(stages[st][sp]) for st in range(4) for sp in range(2)])
        C.call("dcpse_rk4_gs_reverse_step", self.plan._h, self.prec, ptrs, _vp(yb[0]), _vp(yb[1]), _vp(acc[0]),
               _vp(acc[1]), self.params)

    def _reverse_step_stages(self, stages, yb, acc, k_a, k_b):
        """The same reverse step as four separate adjoint stages (reference
        for the fused call)."""
        dt = self.dt
        acc[0].copy_(yb[0])
        acc[1].copy_(yb[1])
        torch.mul(yb[0], dt / 6.0, out=k_a[0])
        torch.mul(yb[1], dt / 6.0, out=k_a[1])
        self._adj_stage(stages[3], k_a, yb, acc, k_b, dt / 3.0, dt)
        self._adj_stage(stages[2], k_b, yb, acc, k_a, dt / 3.0, dt / 2.0)
        self._adj_stage(stages[1], k_a, yb, acc, k_b, dt / 6.0, dt / 2.0)
        self._adj_stage(stages[0], k_b, yb, acc, None, 0.0, 0.0)
        yb[0].copy_(acc[0])
        yb[1].copy_(acc[1])

    def backward(self, checkpoints, every, ybar, stream=None):
        """Reverse over len(checkpoints) * every steps: checkpoints[i] is the
        (u, v) state at the start of segment i (segments of `every` steps,
        the last ending at the current state); returns ybar at checkpoints[0].
        Each segment is recomputed forward from its checkpoint with the stage
        states recorded, then reversed step by step.  With a stream, which
        must be the plan's stream, one segment's recompute and reversal are
        captured in a CUDA graph and replayed for the other segments."""
        self.prepare_adjoint()
        u_save, v_save = self.u.clone(), self.v.clone()
        hist = [[(torch.empty_like(self.u), torch.empty_like(self.v)) for _ in range(4)] for _ in range(every)]
        yb = (ybar[0].clone(), ybar[1].clone())
        acc, k_a, k_b = [(torch.empty_like(self.u), torch.empty_like(self.v)) for _ in range(3)]

        def segment():
            for s in range(every):
                self.step(record=hist[s])
            for s in reversed(range(every)):
                self._reverse_step_into(hist[s], yb, acc, k_a, k_b)

        segs = list(reversed(range(len(checkpoints))))
        if stream is None or not segs:
            for seg in segs:
                self.u.copy_(checkpoints[seg][0])
                self.v.copy_(checkpoints[seg][1])
                segment()
        else:
            with torch.cuda.stream(stream):
                # the last segment runs eagerly (warming up every call), the
                # others replay its graph
                self.u.copy_(checkpoints[segs[0]][0])
                self.v.copy_(checkpoints[segs[0]][1])
                segment()
                if len(segs) > 1:
                    stream.synchronize()
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g, stream=stream):  # records, runs nothing
                        segment()
                    for seg in segs[1:]:
                        self.u.copy_(checkpoints[seg][0])
                        self.v.copy_(checkpoints[seg][1])
                        g.replay()
        self.u.copy_(u_save)
        self.v.copy_(v_save)
        return yb
