"""Autotuner of the batched apply schedule.

Sweeps the lanes that share a neighbour row (4/8/16/32) and the loading mode
of the CSR kernels (direct loads, TMA-staged tiles, 8-deep batches), and the
sliced ELL kernel (a row per thread, lanes do not apply), for a plan and a
field; times each candidate with CUDA events on the plan's stream, keeps the
fastest and sets it on the plan.  All candidates compute the same result up
to the order of the FP32 partial sums (identical bits for the same CSR lane
count).
"""
from __future__ import annotations

import torch

from . import _capi as C

MODES = {1: "direct", 2: "tma-staged", 3: "direct-x8", 4: "sliced-ell"}


def tune_apply(plan, f, precision=C.F32, lanes=(4, 8, 16), modes=(1, 2, 3, 4), reps=10, warmup=2):
    out = torch.empty((plan.n_outputs, f.shape[0]), dtype=torch.float64, device=f.device)
    stream = plan.stream or torch.cuda.current_stream()
    table = []
    best = None
    cands = [(ln, md) for ln in lanes for md in modes if md != 4] + ([(0, 4)] if 4 in modes else [])
    for ln, md in cands:
        plan.set_apply_config(ln, md)
        try:
            plan.apply(f, precision, out)
        except C.DcpseError as e:
            if e.code != C.ERR_CAPACITY:
                raise
            table.append({"lanes": ln, "mode": MODES[md], "ms": None, "skipped": "tiles do not fit"})
            continue
        for _ in range(warmup):
            plan.apply(f, precision, out)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            plan.apply(f, precision, out)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        table.append({"lanes": ln, "mode": MODES[md], "ms": ms})
        if best is None or ms < best[2]:
            best = (ln, md, ms)
    plan.set_apply_config(best[0], best[1])
    plan.check()
    return {"lanes": best[0], "mode": MODES[best[1]], "ms": best[2], "sweep": table}


def tune_assembly(plan, pos, flags, bin_widths=(0, 4, 16), warps=(2, 4, 8), qr_lanes=(2, 4, 8, 16), reps=1):
    """Sweeps the neighbour-count bin width and the warps per CTA of the
    Gram and weight kernels, then the lanes per particle of the QR kernel
    (device time from the plan's event timers); keeps the fastest.  Lane
    counts whose work space does not fit in shared memory are skipped."""
    plan.set_timing(True)
    table = []

    def timed(bw, wp, ql):
        plan.set_assembly_config(bw, wp, ql)
        try:
            plan.assemble(pos, flags)  # warm-up (and the binning for this width)
        except C.DcpseError as e:
            if e.code != C.ERR_CAPACITY:
                raise
            return None
        plan.reset_timing()
        for _ in range(reps):
            plan.assemble(pos, flags)
        ms = plan.timing(C.K_ASSEMBLE)[0] / reps
        table.append({"bin_width": bw, "warps": wp, "qr_lanes": ql, "ms": ms})
        return ms

    best = None
    for bw in bin_widths:
        for wp in warps:
            ms = timed(bw, wp, 0)
            if ms is not None and (best is None or ms < best[3]):
                best = (bw, wp, 0, ms)
    for ql in qr_lanes:
        ms = timed(best[0], best[1], ql)
        if ms is not None and ms < best[3]:
            best = (best[0], best[1], ql, ms)
    plan.set_assembly_config(best[0], best[1], best[2])
    return {"bin_width": best[0], "warps": best[1], "qr_lanes": best[2], "ms": best[3], "sweep": table}
