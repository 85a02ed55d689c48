#!/usr/bin/env python
"""DC-PSE hot-path benchmark on one GB300 (or N independent replicas).

Workload: 128^3 = 2,097,152 jittered 3D particles (h = 1/127, jitter
U(+-0.15h), seed 2), order 2, rCut = 2.8h, Gradient (3 outputs) + Laplacian
(1 output, sum of 3 reference terms): 4 particle-ops per particle.

A step is one batched FP32-weight apply of all 4 outputs over the whole
particle set, inputs resident in HBM; the 2.9 GB weight stream is larger
than L2, so no flush is needed between steps.  Also reported: the plain FP64
GPU path (one pass per reference Dcpse object, the reference's order), the
batched FP64 path, device assembly throughput (faithful and fast), the
end-to-end call through the host-buffer C-ABI entry point, and the CPU oracle
(the reference algorithm restated) on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DC-PSE apply Gparticle-ops/s & assembly Mparticles/s: FP32-batched vs FP64 @≤1e-6"
UNIT = "Gparticle-ops/s"
NOUT = 4
# one protocol for every CPU timing (the cpu_baseline leg and the reference
# arm): the first CPU_SAMPLE particles' rows with their full neighbourhoods,
# CPU_WARM untimed and CPU_STEPS timed applies on all host cores
CPU_SAMPLE = 32768
CPU_STEPS = 20
CPU_WARM = 3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nside", type=int, default=128)
    ap.add_argument("--cpu-sample", type=int, default=CPU_SAMPLE, help="particles in the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the graded-cloud, adjoint, Gray-Scott and shuffled-order sections")
    ap.add_argument("--only", choices=["apply", "apply-pair", "apply64", "assemble", "assemble-tc", "gray-scott", "graded",
                                       "interp", "vjp"],
                    default=None,
                    help="small-footprint run of one kernel family (for profiler captures)")
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--mode", type=int, default=0, help="apply kernel: 0 auto, 1 CSR direct, 2 CSR TMA-staged, 3 CSR 8-deep, 4 sliced ELL")
    ap.add_argument("--qr-lanes", type=int, default=0, help="assembly QR lanes per particle (0 = automatic)")
    return ap.parse_args()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling (200 ms) during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(times, dist=None, device="cpu"):
    """Per-rank times -> their maxima over all ranks (the slowest rank sets
    the job's time); unchanged in a single process."""
    if dist is None:
        return [float(t) for t in times]
    import torch

    t = torch.tensor([float(x) for x in times], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_value(world, n, nout, t):
    """Whole-job throughput in Gparticle-ops/s: every rank applies nout
    outputs to its own n particles in time t (replicas, weak scaling)."""
    return world * n * nout / t / 1e9


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# ----------------------------------------------------------------- CPU leg --
SIGS6 = [(1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (0, 2, 0), (0, 0, 2)]


def cpu_oracle_run(pos, rcut, f, sample, steps, warmup, nthreads):
    """The reference algorithm restated on the CPU (oracle/): the S first
    particles' rows (full neighbourhoods), 6 reference Dcpse objects
    (Dx, Dy, Dz, Dxx, Dyy, Dzz), each assembled with the dense E of the
    reference; a step applies the 4 outputs (Laplacian = sum of 3).  Also
    returns the lists, kernels and outputs, against which the GPU's rows are
    checked."""
    import oracle

    S = min(sample, pos.shape[0])
    rp, cols = oracle.neighbors(pos[:S], rcut, support=pos)
    t0 = time.perf_counter()
    terms = [oracle.assemble(pos[:S], rp, cols, s, 2, support=pos, nthreads=nthreads) for s in SIGS6]
    t_asm = time.perf_counter() - t0
    multi = oracle.MultiApply(rp, cols, [(t[2], t[1], sum(s)) for t, s in zip(terms, SIGS6)],
                              [0, 1, 2, 3, 3, 3], NOUT, f, f_dom=f[:S])

    def step():
        return multi(nthreads)

    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    t_apply = (time.perf_counter() - t0) / max(steps, 1)
    return dict(S=S, nnz=int(rp[-1]), t_asm=t_asm, t_apply=t_apply,
                apply_value=S * NOUT / t_apply / 1e9, asm_value=S / t_asm / 1e6,
                rp=rp, cols=cols, kernels=[t[2] for t in terms], out=multi.out.copy())


def cpu_sample_text(r, n, steps):
    return ("first %d of %d particles (full neighbourhoods, %d entries), 6 reference Dcpse objects, "
            "%d timed applies after %d untimed" % (r["S"], n, r["nnz"], steps, CPU_WARM))


def host_cores():
    return os.cpu_count() or 1


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from openfpm_numerics_gb300 import workloads as W

    cfg = W.config2(args.nside)
    pos = cfg["pos"]
    f, _, _ = W.field2(pos)
    cores = host_cores()
    steps, warm = CPU_STEPS, CPU_WARM
    r = cpu_oracle_run(pos, cfg["rcut"], f, args.cpu_sample, steps, warm, cores)
    sample = cpu_sample_text(r, pos.shape[0], steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": r["apply_value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": r["t_apply"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "128^3 jittered 3D particles, Gradient+Laplacian (6 reference Dcpse objects), "
                               "order 2, rCut=2.8h", "particles": int(pos.shape[0])},
        "cpu_baseline": {"value": r["apply_value"], "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "assembly": {"value": r["asm_value"], "unit": "Mparticles/s", "sample": sample},
        "e2e": {"value": r["apply_value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "openfpm_numerics cannot be built here (openfpm_data/pdata, Eigen, Boost, MPI absent); "
                "its CPU Dcpse algorithm is timed as restated in oracle/",
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU leg --
def run_ours(args):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    from openfpm_numerics_gb300 import _capi as C
    from openfpm_numerics_gb300 import workloads as W
    from openfpm_numerics_gb300.plan import DcpsePlan

    cfg = W.config2(args.nside)
    pos_np = cfg["pos"]
    N = pos_np.shape[0]
    f_np, grad_np, lap_np = W.field2(pos_np)
    stream = torch.cuda.current_stream()
    pos = torch.tensor(pos_np, device=dev)
    f = torch.tensor(f_np, device=dev)
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2, stream=stream)
    plan.set_timing(True)

    # neighbour lists (device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan.build_neighbors(pos, cfg["rcut"])
    torch.cuda.synchronize()
    t_nbr = time.perf_counter() - t0
    info = plan.info()
    nnz = info["nnz"]
    kbar = nnz / N

    # faithful assembly (per reference Dcpse object, bit-exact with the oracle)
    plan.reset_timing()
    plan.assemble(pos, C.STORE_TERMS_F64 | C.STORE_OUT_F64)
    t_asm_ref = plan.timing(C.K_ASSEMBLE)[0] / 1e3
    nbad, first_bad, code = plan.particle_status()
    # the rows the CPU oracle recomputes: their lists and per-term kernels
    S = min(args.cpu_sample, N)
    g_rp, g_cols = plan.neighbors()
    g_rp = g_rp[: S + 1].cpu().numpy()
    g_cols = g_cols[: int(g_rp[-1])].cpu().numpy()
    g_kernels = [plan.term_kernels(t)[0][: int(g_rp[-1])].cpu().numpy() for t in range(6)]

    # plain FP64 GPU path: the reference's apply, one pass per Dcpse object
    out64 = torch.empty((NOUT, N), dtype=torch.float64, device=dev)

    def plain_step():
        for o in range(NOUT):
            plan.apply_output_f64(o, f, out64[o])

    for _ in range(3):
        plain_step()
    plan.reset_timing()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nplain = max(3, min(args.steps, 50))
    ev0.record(stream)
    for _ in range(nplain):
        plain_step()
    ev1.record(stream)
    torch.cuda.synchronize()
    t_plain = ev0.elapsed_time(ev1) / 1e3 / nplain
    ref_out = out64.cpu().numpy()

    # batched FP64 apply
    outb = torch.empty((NOUT, N), dtype=torch.float64, device=dev)
    for _ in range(3):
        plan.apply(f, C.F64, outb)
    ev0.record(stream)
    for _ in range(nplain):
        plan.apply(f, C.F64, outb)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_b64 = ev0.elapsed_time(ev1) / 1e3 / nplain
    b64 = outb.cpu().numpy()

    # fast assembly with the Gram products on the tensor cores (warm-up call
    # first: it sizes the scratch for B), and its FP32 outputs against those
    # of the FP64-Gram assembly below
    plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.ASSEMBLE_TC)
    plan.reset_timing()
    plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.ASSEMBLE_TC)
    t_asm_tc = plan.timing(C.K_ASSEMBLE)[0] / 1e3
    tc_used = plan.gram_on_tensor_cores()
    out_tc = torch.empty((NOUT, N), dtype=torch.float64, device=dev)
    plan.apply(f, C.F32, out_tc)

    # fast assembly (summed right-hand sides) -> FP32 weights for the headline
    plan.reset_timing()
    plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32)
    t_asm_fast = plan.timing(C.K_ASSEMBLE)[0] / 1e3
    out_fast = torch.empty((NOUT, N), dtype=torch.float64, device=dev)
    plan.apply(f, C.F32, out_fast)
    tc_vs_fp64_gram = float(max(((out_tc[o] - out_fast[o]).abs().max() / out_fast[o].abs().max()).item()
                                for o in range(NOUT)))
    del out_tc, out_fast
    # the same with the residual streams of the corrected FP32 applies (and
    # the FP64 weights, the yardstick of the weight pairs' apply)
    plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.STORE_OUT_F32_RESID | C.STORE_OUT_F32_CORR |
                  C.STORE_OUT_F64)

    # schedule autotuning (untimed): lanes per row x direct / TMA-staged loads
    from openfpm_numerics_gb300 import autotune

    tuned = autotune.tune_apply(plan, f, C.F32, reps=5, warmup=2)
    # the timed steps use the plan's default schedule (what a caller gets: the
    # sliced ELL kernel when its copy of the weights fits); the sweep is
    # reported beside it
    plan.set_apply_config(0, 0)

    # FP32 with the bf16 residual correction (near-FP64 accuracy)
    outr = torch.empty((NOUT, N), dtype=torch.float64, device=dev)
    for _ in range(3):
        plan.apply(f, C.F32_RESID, outr)
    ev0.record(stream)
    for _ in range(nplain):
        plan.apply(f, C.F32_RESID, outr)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_resid = ev0.elapsed_time(ev1) / 1e3 / nplain
    resr = outr.cpu().numpy()

    # FP32 weight pairs with the fixed-point field (FP64-class results off the
    # FP64 pipe), against the batched FP64 apply of the same weights
    outp = torch.empty((NOUT, N), dtype=torch.float64, device=dev)
    for _ in range(3):
        plan.apply(f, C.F32_PAIR, outp)
    plan.reset_timing()
    ev0.record(stream)
    for _ in range(nplain):
        plan.apply(f, C.F32_PAIR, outp)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_pair = ev0.elapsed_time(ev1) / 1e3 / nplain
    pair_k = plan.timing(C.K_APPLY_BATCHED)
    resp = outp.cpu().numpy()
    plan.apply(f, C.F64, outp)
    b64_fast = outp.cpu().numpy()
    pair_vs_b64 = max(rel_err(resp[o], b64_fast[o]) for o in range(NOUT))
    b64_fast_vs_ref = max(rel_err(b64_fast[o], ref_out[o]) for o in range(NOUT))
    del outp, b64_fast

    # budget-driven FP32 (rows whose FP32 error bound exceeds 1e-6 corrected
    # toward the FP64 weights; FP32 first pass); kernel times from the plan's
    # timers
    outg = torch.empty((NOUT, N), dtype=torch.float64, device=dev)
    plan.set_error_budget(1e-6, C.F32)
    for _ in range(3):
        plan.apply(f, C.F32_BUDGET, outg)
    plan.budget_stats(reset=True)
    plan.reset_timing()
    ev0.record(stream)
    for _ in range(nplain):
        plan.apply(f, C.F32_BUDGET, outg)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_budget = ev0.elapsed_time(ev1) / 1e3 / nplain
    budget_pairs = plan.budget_stats() / nplain
    budget_k = plan.timing(C.K_APPLY_BATCHED)[0] / nplain
    budget_c = plan.timing(C.K_CORRECT)[0] / nplain
    resg = outg.cpu().numpy()

    out = torch.empty((NOUT, N), dtype=torch.float64, device=dev)
    clocks = Clocks(local)
    clocks.start()
    for _ in range(args.warmup):
        plan.apply(f, C.F32, out)
    plan.reset_timing()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        plan.apply(f, C.F32, out)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_step = ev0.elapsed_time(ev1) / 1e3 / args.steps
    k_ms, k_launch = plan.timing(C.K_APPLY_BATCHED)
    s_ms, s_launch = plan.timing(C.K_SPLIT)
    clk = clocks.stop()
    plan.check()
    (t_step,) = max_over_ranks([t_step], dist, dev)
    res32 = out.cpu().numpy()

    # end to end through the host-buffer entry point (pinned host memory)
    hf = torch.empty(N, dtype=torch.float64, pin_memory=True)
    hf.copy_(f.cpu())
    hout = torch.empty((NOUT, N), dtype=torch.float64, pin_memory=True)
    hf_np, hout_np = hf.numpy(), hout.numpy()
    for _ in range(3):
        plan.apply_host(hf_np, hout_np, C.F32)
    n_e2e = max(3, min(args.steps, 200))
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(n_e2e):
        plan.apply_host(hf_np, hout_np, C.F32)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_e2e = ev0.elapsed_time(ev1) / 1e3 / n_e2e
    (t_e2e,) = max_over_ranks([t_e2e], dist, dev)
    assert np.array_equal(hout_np, res32)

    # accuracy
    inner = W.interior_mask(pos_np, cfg["rcut"])
    analytic = [grad_np[:, 0], grad_np[:, 1], grad_np[:, 2], lap_np]
    errors = {
        "fp32_vs_fp64_reference_order_normwise": max(rel_err(res32[o], ref_out[o]) for o in range(NOUT)),
        "fp32_vs_fp64_reference_order_rms": max(float(np.sqrt(np.mean((res32[o] - ref_out[o]) ** 2)) /
                                                    np.sqrt(np.mean(ref_out[o] ** 2))) for o in range(NOUT)),
        "fp32_per_output_normwise": [rel_err(res32[o], ref_out[o]) for o in range(NOUT)],
        "fp32_resid_vs_fp64_reference_order_normwise": max(rel_err(resr[o], ref_out[o]) for o in range(NOUT)),
        "fp32_budget_vs_fp64_reference_order_normwise": max(rel_err(resg[o], ref_out[o]) for o in range(NOUT)),
        "fp64_batched_vs_reference_order_normwise": max(rel_err(b64[o], ref_out[o]) for o in range(NOUT)),
        "fp32_pair_vs_fp64_reference_order_normwise": max(rel_err(resp[o], ref_out[o]) for o in range(NOUT)),
        "fp32_pair_vs_fp64_batched_same_weights_normwise": pair_vs_b64,
        "fp64_analytic_interior_normwise": [rel_err(ref_out[o][inner], analytic[o][inner]) for o in range(NOUT)],
        "fp32_analytic_interior_normwise": [rel_err(res32[o][inner], analytic[o][inner]) for o in range(NOUT)],
        "definition": "max|a-b| / max|b| per output, max over the 4 outputs",
    }

    hbm, peak_kind = peaks()
    bytes_apply = W.apply_bytes(N, nnz, NOUT, 4, fbytes=8, obytes=8)
    t_kernel = k_ms / 1e3 / max(k_launch, 1)
    achieved = bytes_apply / t_kernel / 1e9
    traffic = None
    kname = "apply_sell_kernel"  # the default schedule of FP32 applies
    tf = os.path.join(ROOT, "profiles", "apply_sell_grad_lap_128cube.txt")
    if os.path.exists(tf):
        for ln in open(tf):
            if ln.startswith("traffic_bytes_per_launch:"):
                traffic = float(ln.split(":")[1])
    flops_fast = W.assembly_flops(N, kbar, [(10, 3), (19, 1)])
    flops_ref = W.assembly_flops(N, kbar, [(10, 3), (19, 3)])
    import ctypes as _ct

    _pk = _ct.c_double()
    C.call("dcpse_measure_fp64_peak", _ct.c_void_p(stream.cuda_stream), _ct.byref(_pk))
    fp64_peak = _pk.value
    value = job_value(world, N, NOUT, t_step)

    cpu = None
    oracle_rows = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r = cpu_oracle_run(pos_np, cfg["rcut"], f_np, args.cpu_sample, CPU_STEPS, CPU_WARM, host_cores())
        cpu = {"value": r["apply_value"], "unit": UNIT, "cores": host_cores(), "kind": "port",
               "sample": cpu_sample_text(r, N, CPU_STEPS), "assembly_mparticles_s": r["asm_value"]}
        # the GPU's rows against the oracle's on the same sample
        S = r["S"]
        o_out = r["out"]

        def vs_orc(a):
            # normalised by the largest output over all rows, as the metric's
            # normwise error (the GPU's reference-order output, bit-exact with
            # the oracle on these rows)
            return max(float(np.abs(a[o][:S] - o_out[o]).max() / np.abs(ref_out[o]).max()) for o in range(NOUT))

        oracle_rows = {
            "rows": S, "entries": r["nnz"],
            "neighbor_lists_equal": bool(np.array_equal(r["rp"], g_rp) and np.array_equal(r["cols"], g_cols)),
            "term_kernels_bit_exact": bool(all(np.array_equal(a, b) for a, b in zip(r["kernels"], g_kernels))),
            "fp64_reference_order_bit_exact": bool(np.array_equal(ref_out[:, :S], o_out)),
            "fp64_batched_normwise": vs_orc(b64), "fp32_normwise": vs_orc(res32),
            "fp32_resid_normwise": vs_orc(resr), "fp32_budget_normwise": vs_orc(resg),
            "definition": "max over the sample rows |gpu - oracle| / max over all rows |FP64 reference-order "
                          "output|, max over the 4 outputs"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "128^3 jittered 3D particles (h=1/127, +-0.15h, seed 2), Gradient+Laplacian, "
                                   "order 2, rCut=2.8h, FP32 weights, 4 outputs per particle",
                       "particles": N, "neighbor_entries": nnz, "mean_neighbors": kbar,
                       "max_neighbors": info["max_neighbors"],
                       "l2": "inputs larger than L2 (%.2f GB of weights streamed per step)" % (NOUT * nnz * 4 / 1e9),
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": traffic, "peak_source": peak_kind,
                         "kernel": kname,
                         "algorithmic_bytes_per_launch": bytes_apply, "kernel_ms": t_kernel * 1e3},
            "e2e": {"value": job_value(world, N, NOUT, t_e2e), "unit": UNIT, "h2d_bytes_per_step": N * 8,
                    "d2h_bytes_per_step": NOUT * N * 8, "ms_per_step": t_e2e * 1e3,
                    "api": "dcpse_apply_batched_host"},
            "gpu_launches": int(k_launch + s_launch),
            "clocks": clk,
            "assembly": {"value": N / t_asm_fast / 1e6, "unit": "Mparticles/s", "mode": "fast (summed rhs), FP32 out",
                         "ms": t_asm_fast * 1e3, "fp64_tflops": flops_fast / t_asm_fast / 1e12,
                         "fp64_peak_tflops_measured": fp64_peak,
                         "fp64_frac": flops_fast / t_asm_fast / 1e12 / fp64_peak,
                         "flop_model": "per basis k n(n+1) + 4/3 n^3 + 2 n^2 R + 2 k n R; "
                                       "bases (n=10, R=3) and (n=19, R=1)",
                         "reference_order": {"value": N / t_asm_ref / 1e6, "ms": t_asm_ref * 1e3,
                                             "fp64_tflops": flops_ref / t_asm_ref / 1e12},
                         "tensor_core_gram": {"value": N / t_asm_tc / 1e6, "ms": t_asm_tc * 1e3,
                                              "tensor_cores_used": bool(tc_used),
                                              "fp32_outputs_vs_fp64_gram_normwise": tc_vs_fp64_gram,
                                              "note": "DCPSE_ASSEMBLE_TC: Gram from 8-bit digit planes of a "
                                                      "62-bit fixed-point B on tcgen05, FP32 accumulators"},
                         "failed_particles": nbad, "neighbors_ms": t_nbr * 1e3},
            "fp64_plain": {"value": N * NOUT / t_plain / 1e9, "ms_per_step": t_plain * 1e3,
                           "note": "one pass per reference Dcpse object (6), reference order"},
            "fp64_batched": {"value": N * NOUT / t_b64 / 1e9, "ms_per_step": t_b64 * 1e3},
            "fp32_pair": {"value": N * NOUT / t_pair / 1e9, "ms_per_step": t_pair * 1e3,
                          "kernel_ms": pair_k[0] / max(pair_k[1], 1),
                          "hbm_frac": W.apply_bytes(N, nnz, NOUT, 8, fbytes=8, obytes=8) /
                                      (pair_k[0] / 1e3 / max(pair_k[1], 1)) / 1e9 / hbm,
                          "error_vs_fp64_batched_same_weights": pair_vs_b64,
                          "error_vs_fp64_reference_order": errors["fp32_pair_vs_fp64_reference_order_normwise"],
                          "fp64_batched_same_weights_vs_reference_order": b64_fast_vs_ref,
                          "note": "DCPSE_F32_PAIR: FP32 weight pairs (8 B/entry/output), field in 62-bit "
                                  "fixed point, compensated FP32 sums"},
            "fp32_resid": {"value": N * NOUT / t_resid / 1e9, "ms_per_step": t_resid * 1e3,
                           "note": "FP32 weights + bf16 residual stream (2 B/entry/output)"},
            "fp32_budget": {"value": N * NOUT / t_budget / 1e9, "ms_per_step": t_budget * 1e3,
                            "first_pass_kernel_ms": budget_k, "correction_ms": budget_c,
                            "pairs_corrected_per_call": budget_pairs,
                            "fraction_corrected": budget_pairs / (N * NOUT), "budget": 1e-6,
                            "error_vs_fp64_reference_order": errors["fp32_budget_vs_fp64_reference_order_normwise"],
                            "note": "FP32 first pass with per-row error bounds, FP64-weight residual "
                                    "correction of the rows over the budget"},
            "autotune": tuned,
            "speedup_fp32_batched_vs_fp64_plain": t_plain / t_step,
            "errors": errors,
            "oracle_rows": oracle_rows,
            "cpu_baseline": cpu,
        }
    plan.close()
    del plan
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and not args.no_extras:
        line["graded"] = extra_graded(args)
        line["adjoint"] = extra_adjoint(args, pos_np, cfg["rcut"])
        line["gray_scott"] = extra_gray_scott(args)
        line["shuffled"] = extra_shuffled(args, pos_np, cfg["rcut"], f_np, res32)
        line["cpp_dropin"] = extra_cpp_dropin(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


# ------------------------------------------------------- extra workloads --
def _events_ms(stream, fn, reps, warm=3):
    """Mean CUDA-event time of fn on stream in ms (warm-up calls first)."""
    import torch

    for _ in range(warm):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _pct(a, b, mask=None):
    """|a - b| / max|b| over the rows in mask: p50, p99, max."""
    if mask is not None:
        a, b = a[mask], b[mask]
    e = np.abs(a - b) / max(float(np.abs(b).max()), 1e-300)
    return {"p50": float(np.percentile(e, 50)), "p99": float(np.percentile(e, 99)), "max": float(e.max())}


def extra_graded(args):
    """Graded 2D cloud (1,000,000 particles, density growing 4x along x by
    inverse-CDF sampling, seed 3, per-particle cutoff 3.1 h_p): Dx, Dy, Dxx,
    Dyy, Dxy assembled in one FP64 pass (bins and CTA sizes autotuned),
    applied in FP32, budget-driven FP32 and FP64; errors against the FP64
    apply, the analytic derivatives and the oracle on 2000 sampled rows."""
    import torch

    import oracle
    from openfpm_numerics_gb300 import _capi as C
    from openfpm_numerics_gb300 import autotune
    from openfpm_numerics_gb300 import workloads as W
    from openfpm_numerics_gb300.plan import DcpsePlan

    cfg = W.config3()
    pos_np, rpp_np = cfg["pos"], cfg["rcut_pp"]
    N = pos_np.shape[0]
    stream = torch.cuda.current_stream()
    pos = torch.tensor(pos_np, device="cuda")
    rpp = torch.tensor(rpp_np, device="cuda")
    plan = DcpsePlan(2, W.five_ops_2d(), order=2, stream=stream)
    plan.set_timing(True)
    plan.build_neighbors(pos, 0.0, rpp)
    plan.reset_timing()
    plan.build_neighbors(pos, 0.0, rpp)
    t_nbr = plan.timing(C.K_NEIGHBORS)[0]
    rp_t, cols_t = plan.neighbors()
    k = (rp_t[1:] - rp_t[:-1]).cpu().numpy()
    nnz = plan.info()["nnz"]
    flags = C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.STORE_OUT_F64 | C.STORE_OUT_F32_RESID | C.STORE_OUT_F32_CORR
    tuned = autotune.tune_assembly(plan, pos, flags)
    plan.assemble(pos, flags)
    # most second-derivative rows of this cloud exceed the budget in FP32
    # alone: the first pass also streams the bf16 residuals
    plan.set_error_budget(1e-6, C.F32_RESID)
    nbad = plan.particle_status()[0]
    ok = plan.eps()[1].cpu().numpy() == 0
    x, y = pos_np[:, 0], pos_np[:, 1]
    f_np = np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)
    f = torch.tensor(f_np, device="cuda")
    out = torch.empty((5, N), dtype=torch.float64, device="cuda")
    res = {"particles": N, "nnz": nnz, "k_min": int(k.min()), "k_mean": float(k.mean()), "k_max": int(k.max()),
           "failed_particles": nbad, "neighbors_ms": t_nbr, "assembly_ms": tuned["ms"],
           "assembly_mparticles_s": N / tuned["ms"] / 1e3,
           "assembly_schedule": {kk: tuned[kk] for kk in ("bin_width", "warps", "qr_lanes")},
           "reorder": plan.reorder_info()}
    t64 = _events_ms(stream, lambda: plan.apply(f, C.F64, out), 20)
    o64 = out.cpu().numpy()
    t32 = _events_ms(stream, lambda: plan.apply(f, C.F32, out), 20)
    o32 = out.cpu().numpy()
    # the same with one window of 8 slices per block (the schedule whose
    # barrier waits for each window's longest slice)
    plan.set_apply_config(0, C.APPLY_SLICE_WINDOWS)
    t32w = _events_ms(stream, lambda: plan.apply(f, C.F32, out), 20)
    plan.set_apply_config(0, 0)
    tpair = _events_ms(stream, lambda: plan.apply(f, C.F32_PAIR, out), 20)
    opair = out.cpu().numpy()
    plan.apply(f, C.F32_BUDGET, out)
    plan.budget_stats(reset=True)
    plan.reset_timing()
    tb = _events_ms(stream, lambda: plan.apply(f, C.F32_BUDGET, out), 20, warm=0)
    pairs = plan.budget_stats() / 20
    tbk = plan.timing(C.K_APPLY_BATCHED)[0] / 20
    tbc = plan.timing(C.K_CORRECT)[0] / 20
    ob = out.cpu().numpy()
    tp = 2 * np.pi
    sx, cx, sy, cy = np.sin(tp * x), np.cos(tp * x), np.sin(tp * y), np.cos(tp * y)
    exact = [tp * cx * cy, -tp * sx * sy, -tp * tp * sx * cy, -tp * tp * sx * cy, -tp * tp * cx * sy]
    margin = float(rpp_np.max())
    inner = (x > margin) & (x < 1 - margin) & (y > margin) & (y < 1 - margin) & ok
    res["apply_ms"] = {"fp64": t64, "fp32": t32, "fp32_window_schedule": t32w, "fp32_pair": tpair, "fp32_budget": tb,
                       "budget_first_pass_kernel": tbk, "budget_correction": tbc}
    res["gparticle_ops_s"] = {"fp64": N * 5 / t64 / 1e6, "fp32": N * 5 / t32 / 1e6, "fp32_pair": N * 5 / tpair / 1e6,
                              "fp32_budget": N * 5 / tb / 1e6}
    res["budget"] = {"budget": 1e-6, "pairs_corrected_per_call": pairs, "fraction_corrected": pairs / (N * 5)}
    res["fp32_vs_fp64"] = [_pct(o32[o], o64[o], ok) for o in range(5)]
    res["fp32_budget_vs_fp64"] = [_pct(ob[o], o64[o], ok) for o in range(5)]
    res["fp32_budget_max_normwise"] = max(_pct(ob[o], o64[o], ok)["max"] for o in range(5))
    res["fp32_pair_vs_fp64"] = [_pct(opair[o], o64[o], ok) for o in range(5)]
    res["fp32_pair_max_normwise"] = max(_pct(opair[o], o64[o], ok)["max"] for o in range(5))
    res["fp64_vs_analytic_interior"] = [_pct(o64[o], exact[o], inner) for o in range(5)]
    # the oracle on 2000 sampled rows (lists, per-term reference assembly,
    # reference-order apply)
    rows = np.sort(np.random.default_rng(8).choice(N, 2000, replace=False))
    # lists of the sampled rows against the whole set: the oracle's self test
    # compares indices, so the sample keeps its particle and drops it here
    a_rp, a_cols = oracle.neighbors(pos_np[rows], 0.0, support=pos_np, rcut_pp=rpp_np[rows], self_skip=False)
    keep = np.ones(a_cols.size, bool)
    for i, r in enumerate(rows):
        seg = slice(a_rp[i], a_rp[i + 1])
        keep[seg] = a_cols[seg] != r
    o_cols = a_cols[keep]
    o_rp = np.concatenate([[0], np.cumsum([keep[a_rp[i]:a_rp[i + 1]].sum() for i in range(rows.size)])])
    g_rp = rp_t.cpu().numpy()
    g_cols = cols_t.cpu().numpy()
    same = all(np.array_equal(o_cols[o_rp[i]:o_rp[i + 1]], g_cols[g_rp[r]:g_rp[r + 1]]) for i, r in enumerate(rows))
    sigs = [s_[0] for s_ in W.five_ops_2d()]
    terms = [oracle.assemble(pos_np[rows], o_rp, o_cols, sg, 2, support=pos_np, nthreads=host_cores())
             for sg in sigs]
    multi = oracle.MultiApply(o_rp, o_cols, [(t[2], t[1], sum(sg)) for t, sg in zip(terms, sigs)],
                              [0, 1, 2, 3, 4], 5, f_np, f_dom=f_np[rows])
    o_ref = multi(host_cores())
    okr = ok[rows] & np.all([t[3] == 0 for t in terms], axis=0)

    def vs_orc(a):
        return max(float(np.abs(a[o][rows][okr] - o_ref[o][okr]).max() / np.abs(o64[o][ok]).max())
                   for o in range(5))

    res["oracle_rows"] = {"rows": int(rows.size), "neighbor_lists_equal": bool(same),
                          "fp64_normwise": vs_orc(o64), "fp32_normwise": vs_orc(o32), "fp32_budget_normwise": vs_orc(ob),
                          "fp32_pair_normwise": vs_orc(opair),
                          "definition": "max over assembled sample rows |gpu - oracle| / max over all rows |FP64 "
                                        "output|, max over the 5 operators"}
    hbm, _ = peaks()
    b32 = W.apply_bytes(N, nnz, 5, 4)
    res["roofline_fp32"] = {"algorithmic_bytes": b32, "achieved_gbs": b32 / t32 / 1e6, "frac": b32 / t32 / 1e6 / hbm}
    bp = W.apply_bytes(N, nnz, 5, 8)
    res["roofline_fp32_pair"] = {"algorithmic_bytes": bp, "achieved_gbs": bp / tpair / 1e6,
                                 "frac": bp / tpair / 1e6 / hbm}
    plan.check()
    plan.close()
    return res


def extra_adjoint(args, pos2, rcut2):
    """Adjoint timings: the field VJP (transposed apply) and the position VJP
    (through every moment-matrix solve) of the Laplacian at 256^2 (jitter
    0.1h, seed 4, f and g N(0,1)) and of Gradient + Laplacian at 128^3,
    against the oracle's reference adjoint on all host cores (all rows at
    256^2, the first 16384 rows at 128^3); FD and oracle parity are
    tests/test_gpu_adjoint.py's."""
    import torch

    import oracle
    from openfpm_numerics_gb300 import _capi as C
    from openfpm_numerics_gb300 import workloads as W
    from openfpm_numerics_gb300.plan import DcpsePlan

    stream = torch.cuda.current_stream()
    res = {"host_cores": host_cores()}
    cases = [("lap_256sq", W.config4(), [[(2, 0), (0, 2)]], None),
             ("grad_lap_128cube", {"pos": pos2, "rcut": rcut2}, W.grad_lap_outputs(3), 16384)]
    for name, cfg, outputs, host_rows in cases:
        pos_np = cfg["pos"]
        n, dim = pos_np.shape
        rng = np.random.default_rng(4)
        if "f" in cfg:
            f_np, g_np = cfg["f"], cfg["g"][None, :]
        else:
            f_np = rng.standard_normal(n)
            g_np = rng.standard_normal((len(outputs), n))
        pos = torch.tensor(pos_np, device="cuda")
        plan = DcpsePlan(dim, outputs, order=2, stream=stream)
        plan.build_neighbors(pos, cfg["rcut"])
        plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32)
        f = torch.tensor(f_np, device="cuda")
        g = torch.tensor(g_np, device="cuda")
        gout = torch.empty(n, dtype=torch.float64, device="cuda")
        r = {"particles": n, "nnz": plan.info()["nnz"]}
        r["vjp_field_fp64_ms"] = _events_ms(stream, lambda: plan.vjp_field(g, C.F64, gout), 10)
        r["vjp_field_fp32_ms"] = _events_ms(stream, lambda: plan.vjp_field(g, C.F32, gout), 10)
        r["vjp_positions_ms"] = _events_ms(stream, lambda: plan.vjp_positions(pos, f, g), 3, warm=1)
        grad = plan.vjp_positions(pos, f, g).cpu().numpy()
        rp, cols = (x.cpu().numpy() for x in plan.neighbors())
        rows = (0, n if host_rows is None else min(host_rows, n))
        t0 = time.perf_counter()
        ref = oracle.vjp_positions(pos_np, rp, cols, outputs, f_np, g_np, rows=rows, nthreads=host_cores())
        t_host = (time.perf_counter() - t0) * 1e3
        r["host_rows"] = rows[1] - rows[0]
        r["host_vjp_positions_ms"] = t_host
        r["vjp_positions_vs_host"] = (t_host / r["host_rows"]) / (r["vjp_positions_ms"] / n)
        if host_rows is None:
            r["vjp_positions_vs_oracle_normwise"] = float(np.abs(grad - ref).max() / np.abs(ref).max())
        plan.check()
        plan.close()
        del plan
        torch.cuda.empty_cache()
        res[name] = r
    res["definition"] = ("vjp_positions_vs_host: host ms per row / GPU ms per row (host: the oracle's reference "
                         "adjoint, same lists, all host cores)")
    return res


def extra_shuffled(args, pos_np, rcut, f_np, res32):
    """The benchmark set in a seeded random particle order (seed 11): the
    apply's sliced layout is renumbered (row-major order at the mean spacing,
    and the Z-order of the list's cells), so the field gathers stay local
    whatever the caller's order; outputs come back in the caller's order."""
    import torch

    from openfpm_numerics_gb300 import _capi as C
    from openfpm_numerics_gb300 import workloads as W
    from openfpm_numerics_gb300.plan import DcpsePlan

    N = pos_np.shape[0]
    perm = np.random.default_rng(11).permutation(N)
    sp = np.ascontiguousarray(pos_np[perm])
    stream = torch.cuda.current_stream()
    pos = torch.tensor(sp, device="cuda")
    f = torch.tensor(np.ascontiguousarray(f_np[perm]), device="cuda")
    out = torch.empty((NOUT, N), dtype=torch.float64, device="cuda")
    hbm, _ = peaks()
    res = {}
    for label, order, pol in (("row_major_order", 1, 0), ("cell_order", 0, 0), ("caller_order", 0, -1)):
        if label != "caller_order":
            if label != "row_major_order":
                plan.close()
            plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2, stream=stream)
            plan.set_timing(True)
            plan.set_reorder_order(order)
            plan.build_neighbors(pos, rcut)
            plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32)
            nnz = plan.info()["nnz"]
            res["reorder_" + label] = plan.reorder_info()
        plan.set_reorder(pol)
        for _ in range(5):
            plan.apply(f, C.F32, out)
        plan.reset_timing()
        for _ in range(50):
            plan.apply(f, C.F32, out)
        ms, kn = plan.timing(C.K_APPLY_BATCHED)
        sm, sn = plan.timing(C.K_SPLIT)
        t = ms / kn / 1e3
        b = W.apply_bytes(N, nnz, NOUT, 4)
        res[label] = {"kernel_ms": t * 1e3, "split_ms": sm / max(sn, 1), "achieved_gbs": b / t / 1e9,
                      "frac": b / t / 1e9 / hbm, "renumbered": plan.reorder_info()[0]}
        if label == "cell_order":
            o = out.cpu().numpy()
            res["fp32_vs_ordered_fp32_normwise"] = max(rel_err(o[k], res32[k][perm]) for k in range(NOUT))
    plan.check()
    plan.close()
    return res


def extra_cpp_dropin(args):
    """The C++ drop-in end to end (tests/cpp/bench_dcpse_api.cpp): the
    reference's user code getV<1>(parts) = Lap(getV<0>(parts)) and the
    Gradient on 128^3 host-resident particles, FP64 expression path and the
    opt-in batched FP32 paths; built here with the host compiler against the
    library."""
    import subprocess
    import tempfile

    from openfpm_numerics_gb300 import build as b

    lib = b.build()
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "bench_dcpse_api")
        cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
               os.path.join(ROOT, "tests", "cpp", "bench_dcpse_api.cpp"), "-L" + os.path.dirname(lib),
               "-ldcpse_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return {"error": "compile failed: " + r.stderr[-500:]}
        r = subprocess.run([exe, str(args.nside)], capture_output=True, text=True, timeout=900)
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
        if r.returncode != 0 or not lines:
            return {"error": "run failed (rc %d): %s" % (r.returncode, r.stderr[-500:])}
        res = json.loads(lines[-1])
    res["workload"] = ("128^3 jittered particles (std::mt19937_64 seed 2, +-0.15h), rCut 2.8h, order 2; "
                       "timings include the host property gather and scatter of each assignment")
    return res


def run_gray_scott(args):
    print(json.dumps(gray_scott_run(args)), flush=True)


def extra_gray_scott(args):
    return gray_scott_run(args)


def gray_scott_run(args):
    """3D Gray-Scott on 96^3 = 884,736 jittered particles in a periodic unit
    cube (jitter +-0.1h, seed 6), DC-PSE Laplacian order 2, rCut = 2.8h, two
    FP32 species, Du=2e-5, Dv=1e-5, F=0.04, k=0.06, dt = 0.2 h^2/Du,
    1000 RK4 steps replayed from CUDA graphs of 10 steps; then the gradient of
    sum(v_final) with respect to v 100 steps earlier by the checkpointed
    adjoint (checkpoints every 10 steps)."""
    import torch

    from openfpm_numerics_gb300 import _capi as C
    from openfpm_numerics_gb300 import workloads as W
    from openfpm_numerics_gb300.odeint import GrayScottRK4
    from openfpm_numerics_gb300.plan import DcpsePlan

    torch.cuda.set_device(0)
    nside = args.nside if args.nside != 128 else 96
    cfg = W.config5(nside)
    s = torch.cuda.Stream()
    plan = DcpsePlan(3, [[(2, 0, 0), (0, 2, 0), (0, 0, 2)]], box=cfg["box"], stream=s)
    pos = torch.tensor(cfg["pos"], device="cuda")
    with torch.cuda.stream(s):
        plan.build_neighbors(pos, cfg["rcut"])
        plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32)
        if args.lanes:
            plan.set_apply_config(args.lanes, 1)
        u0, v0 = W.gray_scott_initial(cfg["pos"])
        u = torch.tensor(u0, device="cuda", dtype=torch.float32)
        v = torch.tensor(v0, device="cuda", dtype=torch.float32)
    s.synchronize()
    Du, Dv, F, K = 2e-5, 1e-5, 0.04, 0.06
    dt = 0.2 * cfg["h"] ** 2 / Du
    gs = GrayScottRK4(plan, u, v, Du, Dv, F, K, dt)
    gs.capture(10, s)  # includes one eager warm-up step
    total, window, every = 1000, 100, 10
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(s):
        ev0.record(s)
        gs.run(total - 1 - window - 9)  # steps before the backward window (graph multiples)
        ev1.record(s)
    s.synchronize()
    t_fwd = ev0.elapsed_time(ev1) / (total - 1 - window - 9)
    with torch.cuda.stream(s):
        for _ in range(9):
            gs.step()
        ckpts = []
        for _ in range(window // every):
            ckpts.append((gs.u.clone(), gs.v.clone()))
            gs.run(every)
        s.synchronize()
        ybar = (torch.zeros_like(gs.u), torch.ones_like(gs.v))
        # warm-up call: the adjoint set-up, the kernels' first loads and the
        # graph capture happen once; the timed call repeats the same window
        gs.backward(ckpts, every, ybar, stream=s)
        s.synchronize()
        ev0.record(s)
        ub, vb = gs.backward(ckpts, every, ybar, stream=s)
        ev1.record(s)
    s.synchronize()
    t_bwd = ev0.elapsed_time(ev1)
    nnz = plan.info()["nnz"]
    n = pos.shape[0]
    # per stage: row offsets, columns and FP32 weights once, the stage input
    # (2 species, gathered from L2), the step's start state, the accumulator
    # (read and written), the stage output
    step_bytes = 4 * (8 * (n + 1) + 8 * nnz + 8 * n + 8 * n + 16 * n + 8 * n)
    hbm, peak_kind = peaks()
    res = {"workload": "96^3 periodic Gray-Scott, 1000 RK4 steps from 10-step CUDA graphs",
           "particles": n, "nnz": nnz, "steps": total,
           "ms_per_step_graph": t_fwd,
           "roofline": {"bound": "hbm", "algorithmic_bytes_per_step": step_bytes,
                        "achieved_gbs": step_bytes / t_fwd / 1e6, "peak_gbs": hbm,
                        "frac": step_bytes / t_fwd / 1e6 / hbm, "peak_source": peak_kind}, "backward_window_steps": window, "checkpoint_every": every,
           "backward_ms": t_bwd, "backward_ms_per_step": t_bwd / window,
           "v_final_mean": float(gs.v.mean()), "grad_v_norm": float(vb.norm()),
           "finite": bool(torch.isfinite(gs.v).all() and torch.isfinite(vb).all())}
    res["backward_over_forward"] = res["backward_ms_per_step"] / t_fwd
    plan.check()
    plan.close()
    return res


def run_interp(args):
    """Particle to particle interpolation (PPInterpolation::p2p): from a
    jittered copy of the 128^3 lattice (jitter U(+-0.3h), seed 7) onto the
    lattice (h = 1/127, jitter U(+-0.15h), seed 2), order 2, rCut = 2.8h,
    two-set lists (createVerletTwoPhase).  Times the assembly, the
    reference-order FP64 p2p (per-term kernels), and the batched p2p from
    the summed weights in FP64 and FP32 (field as an exact float pair)."""
    import torch

    from openfpm_numerics_gb300 import _capi as C
    from openfpm_numerics_gb300 import workloads as W
    from openfpm_numerics_gb300.plan import DcpsePlan

    torch.cuda.set_device(0)
    cfg = W.config2(args.nside)
    dom_np = cfg["pos"]
    h = cfg["h"]
    sup_np = dom_np + np.random.default_rng(7).uniform(-0.3 * h, 0.3 * h, dom_np.shape)
    N = dom_np.shape[0]
    dom = torch.tensor(dom_np, device="cuda")
    sup = torch.tensor(sup_np, device="cuda")
    f = torch.tensor(W.field2(sup_np)[0], device="cuda")
    stream = torch.cuda.current_stream()
    plan = DcpsePlan(3, [[(0, 0, 0)]], order=2, stream=stream)
    plan.set_timing(True)
    plan.set_support(sup)
    plan.build_neighbors(dom, cfg["rcut"])
    nnz = plan.info()["nnz"]
    plan.reset_timing()
    plan.assemble(dom, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    t_asm = plan.timing(C.K_ASSEMBLE)[0]
    nbad = plan.particle_status()[0]
    out = torch.empty(N, dtype=torch.float64, device="cuda")
    outb = torch.empty((1, N), dtype=torch.float64, device="cuda")
    res = {"only": "interp", "particles": N, "support_particles": N, "nnz": nnz, "mean_neighbors": nnz / N,
           "assembly_ms": t_asm, "failed_particles": nbad}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(3, min(args.steps, 50))

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        plan.reset_timing()
        ev0.record(stream)
        for _ in range(reps):
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / reps

    res["p2p_f64_reference_ms"] = timed(lambda: plan.p2p_f64(0, f, out))
    ref = out.clone()
    res["p2p_f64_batched_ms"] = timed(lambda: plan.p2p(f, C.F64, outb))
    b64 = outb[0].clone()
    sweep = []
    for lanes, mode in [(ln, md) for ln in (4, 8, 16) for md in (1, 3)] + [(0, 4)]:
        plan.set_apply_config(lanes, mode)
        sweep.append({"lanes": lanes, "mode": mode, "ms": timed(lambda: plan.p2p(f, C.F32, outb))})
    best = min(sweep, key=lambda r: r["ms"])
    res["p2p_f32_sweep"] = sweep
    plan.set_apply_config(0, 0)
    res["p2p_f32_auto_ms"] = timed(lambda: plan.p2p(f, C.F32, outb))
    plan.set_apply_config(best["lanes"], best["mode"])
    res["p2p_f32_ms"] = timed(lambda: plan.p2p(f, C.F32, outb))
    res["p2p_f32_schedule"] = {"lanes": best["lanes"], "mode": best["mode"]}
    k_ms, k_n = plan.timing(C.K_APPLY_BATCHED)
    b32 = outb[0].clone()
    fmax = f.abs().max().item()
    res["err_f64_batched_vs_reference"] = (b64 - ref).abs().max().item() / fmax
    res["err_f32_vs_reference"] = (b32 - ref).abs().max().item() / fmax
    exact = torch.tensor(W.field2(dom_np)[0], device="cuda")
    inner = torch.tensor(W.interior_mask(dom_np, cfg["rcut"]), device="cuda")
    res["err_reference_vs_analytic_interior"] = ((ref - exact)[inner]).abs().max().item() / fmax
    hbm, peak_kind = peaks()
    # row offsets, columns, FP32 weights, the split field gathered once, FP64 output
    bytes_f32 = 8 * (N + 1) + nnz * (4 + 4) + 8 * N + 8 * N
    kern_ms = k_ms / max(k_n, 1)
    res["p2p_f32_kernel_ms"] = kern_ms
    res["roofline_f32"] = {"bound": "hbm", "algorithmic_bytes": bytes_f32, "achieved_gbs": bytes_f32 / kern_ms / 1e6,
                           "peak_gbs": hbm, "frac": bytes_f32 / kern_ms / 1e6 / hbm, "peak_source": peak_kind}
    res["value_gparticles_s_f32"] = N / res["p2p_f32_ms"] / 1e6
    plan.check()
    plan.close()
    print(json.dumps(res), flush=True)


def run_graded(args):
    """Uneven 2D cloud: 1,000,000 particles, density growing 4x along x
    (inverse-CDF sampling, seed 3), per-particle cutoff 3.1 h_p, five
    operators Dx, Dy, Dxx, Dyy, Dxy assembled in one persistent launch
    (FP64; neighbour-count bins and CTA size autotuned) and applied in one
    FP32 pass (lanes and loading autotuned)."""
    import torch

    from openfpm_numerics_gb300 import _capi as C
    from openfpm_numerics_gb300 import autotune
    from openfpm_numerics_gb300 import workloads as W
    from openfpm_numerics_gb300.plan import DcpsePlan

    torch.cuda.set_device(0)
    cfg = W.config3()
    pos_np = cfg["pos"]
    N = pos_np.shape[0]
    pos = torch.tensor(pos_np, device="cuda")
    rpp = torch.tensor(cfg["rcut_pp"], device="cuda")
    plan = DcpsePlan(2, W.five_ops_2d(), order=2, stream=torch.cuda.current_stream())
    plan.set_timing(True)
    plan.build_neighbors(pos, 0.0, rpp)
    rp, _ = plan.neighbors()
    k = (rp[1:] - rp[:-1]).cpu().numpy()
    nnz = plan.info()["nnz"]
    flags = C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.STORE_OUT_F64 | C.STORE_OUT_F32_RESID | C.STORE_OUT_F32_CORR
    tuned_asm = autotune.tune_assembly(plan, pos, flags)
    nbad = plan.particle_status()[0]
    x, y = pos_np[:, 0], pos_np[:, 1]
    f_np = np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)
    f = torch.tensor(f_np, device="cuda")
    tuned_app = autotune.tune_apply(plan, f, C.F32, reps=20)
    out64 = plan.apply(f, C.F64).cpu().numpy()
    out32 = plan.apply(f, C.F32).cpu().numpy()
    plan.set_apply_config(0, 0)
    stream = torch.cuda.current_stream()
    t_pair = _events_ms(stream, lambda: plan.apply(f, C.F32_PAIR), 20)
    t_64 = _events_ms(stream, lambda: plan.apply(f, C.F64), 20)
    outp = plan.apply(f, C.F32_PAIR).cpu().numpy()
    plan.set_apply_config(0, 1)
    out32r = plan.apply(f, C.F32_RESID).cpu().numpy()
    tp = 2 * np.pi
    s, c = np.sin(tp * x), np.cos(tp * x)
    sy, cy = np.sin(tp * y), np.cos(tp * y)
    exact = [tp * c * cy, -tp * s * sy, -tp * tp * s * cy, -tp * tp * s * cy, -tp * tp * c * sy]
    margin = float(cfg["rcut_pp"].max())
    ok = plan.eps()[1].cpu().numpy() == 0  # particles that could be assembled
    inner = (x > margin) & (x < 1 - margin) & (y > margin) & (y < 1 - margin) & ok

    def pct(a, b, mask):
        e = np.abs(a[mask] - b[mask]) / np.abs(b[mask]).max()
        return {"p50": float(np.percentile(e, 50)), "p99": float(np.percentile(e, 99)), "max": float(e.max())}

    res = {"only": "graded", "particles": N, "nnz": nnz, "k_min": int(k.min()), "k_mean": float(k.mean()),
           "k_max": int(k.max()), "failed_particles": nbad,
           "assembly_ms": tuned_asm["ms"], "assembly_mparticles_s": N / tuned_asm["ms"] / 1e3,
           "assembly_autotune": tuned_asm,
           "apply_ms": tuned_app["ms"], "apply_gparticle_ops_s": N * 5 / tuned_app["ms"] / 1e6,
           "apply_autotune": {k2: v for k2, v in tuned_app.items() if k2 != "sweep"},
           "fp32_vs_fp64": [pct(out32[o], out64[o], ok) for o in range(5)],
           "fp32_resid_vs_fp64": [pct(out32r[o], out64[o], ok) for o in range(5)],
           "fp32_pair_ms": t_pair, "fp64_ms": t_64,
           "fp32_pair_vs_fp64": [pct(outp[o], out64[o], ok) for o in range(5)],
           "fp64_vs_analytic_interior": [pct(out64[o], exact[o], inner) for o in range(5)],
           "error_definition": "|a-b| / max|b| over assembled particles (status 0); percentiles and max"}
    plan.check()
    plan.close()
    print(json.dumps(res), flush=True)


def run_only(args):
    """One kernel family on the benchmark geometry, nothing else resident:
    --only apply keeps just the FP32 weights (fast assembly), --only apply64
    just the FP64 summed weights (batched FP64 apply), --only assemble runs
    the reference-order and fast assemblies, --only assemble-tc the fast
    assembly with the FP64 Gram and with the tensor-core Gram."""
    import torch

    from openfpm_numerics_gb300 import _capi as C
    from openfpm_numerics_gb300 import workloads as W
    from openfpm_numerics_gb300.plan import DcpsePlan

    if args.only == "gray-scott":
        run_gray_scott(args)
        return
    if args.only == "graded":
        run_graded(args)
        return
    if args.only == "interp":
        run_interp(args)
        return
    torch.cuda.set_device(0)
    cfg = W.config2(args.nside)
    pos = torch.tensor(cfg["pos"], device="cuda")
    f = torch.tensor(W.field2(cfg["pos"])[0], device="cuda")
    N = pos.shape[0]
    stream = torch.cuda.current_stream()
    plan = DcpsePlan(3, W.grad_lap_outputs(3), order=2, stream=stream)
    plan.set_timing(True)
    plan.build_neighbors(pos, cfg["rcut"])
    plan.reset_timing()
    plan.build_neighbors(pos, cfg["rcut"])  # timed on the second build (first one warms up)
    nnz = plan.info()["nnz"]
    res = {"only": args.only, "particles": N, "nnz": nnz, "neighbors_ms": plan.timing(C.K_NEIGHBORS)[0]}
    if args.only == "apply":
        plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32)
        plan.set_apply_config(args.lanes, args.mode)
        out = torch.empty((NOUT, N), dtype=torch.float64, device="cuda")
        for _ in range(args.warmup):
            plan.apply(f, C.F32, out)
        plan.reset_timing()
        for _ in range(args.steps):
            plan.apply(f, C.F32, out)
        ms, k = plan.timing(C.K_APPLY_BATCHED)
        res["apply_ms"] = ms / max(k, 1)
        res["achieved_gbs"] = W.apply_bytes(N, nnz, NOUT, 4) / (ms / max(k, 1) / 1e3) / 1e9
    elif args.only == "apply-pair":
        # the FP32 weight pairs (DCPSE_F32_PAIR): 8 bytes per entry and output
        plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.STORE_OUT_F32_CORR)
        plan.set_apply_config(args.lanes, args.mode)
        out = torch.empty((NOUT, N), dtype=torch.float64, device="cuda")
        for _ in range(args.warmup):
            plan.apply(f, C.F32_PAIR, out)
        plan.reset_timing()
        for _ in range(args.steps):
            plan.apply(f, C.F32_PAIR, out)
        ms, k = plan.timing(C.K_APPLY_BATCHED)
        res["apply_pair_ms"] = ms / max(k, 1)
        res["achieved_gbs"] = W.apply_bytes(N, nnz, NOUT, 8) / (ms / max(k, 1) / 1e3) / 1e9
    elif args.only == "vjp":
        # the position VJP (FP64, through eps, the moment systems and the
        # kernels) with N(0, 1) cotangents
        plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F64)
        g = torch.tensor(np.random.default_rng(4).standard_normal((NOUT, N)), device="cuda")
        for _ in range(args.warmup):
            plan.vjp_positions(pos, f, g)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            plan.vjp_positions(pos, f, g)
        e1.record(stream)
        torch.cuda.synchronize()
        res["vjp_positions_ms"] = e0.elapsed_time(e1) / max(args.steps, 1)
    elif args.only == "apply64":
        plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F64)
        out = torch.empty((NOUT, N), dtype=torch.float64, device="cuda")
        for _ in range(args.warmup):
            plan.apply(f, C.F64, out)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            plan.apply(f, C.F64, out)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / max(args.steps, 1)
        res["apply64_ms"] = t
        res["apply64_gbs"] = W.apply_bytes(N, nnz, NOUT, 8) / (t / 1e3) / 1e9
    elif args.only == "assemble-tc":
        plan.set_assembly_config(0, 4, args.qr_lanes)
        ts = {"fp64_gram_ms": [], "tc_gram_ms": []}
        for _ in range(max(1, args.steps)):
            for key, extra in (("fp64_gram_ms", 0), ("tc_gram_ms", C.ASSEMBLE_TC)):
                plan.reset_timing()
                plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32 | extra)
                ts[key].append(plan.timing(C.K_ASSEMBLE)[0])
        res.update(ts)
        res["tensor_cores_used"] = plan.gram_on_tensor_cores()
    else:
        plan.set_assembly_config(0, 4, args.qr_lanes)
        for _ in range(max(1, args.steps)):
            plan.reset_timing()
            plan.assemble(pos, C.STORE_TERMS_F64)
            t_ref = plan.timing(C.K_ASSEMBLE)[0]
            plan.reset_timing()
            plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32)
            t_fast = plan.timing(C.K_ASSEMBLE)[0]
        res["assemble_ref_ms"] = t_ref
        res["assemble_fast_ms"] = t_fast
    plan.check()
    plan.close()
    print(json.dumps(res), flush=True)


def main():
    args = parse()
    if args.only:
        run_only(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
