"""Parity of the CUDA path (through the C-ABI) with the CPU oracle.

Bars (FP64): neighbour lists, eps, eps^-|alpha|, per-term kernels, the
per-term apply and the reference-order output apply are bit-exact; the
batched FP64 apply and the fast (summed right-hand side) assembly are within
1e-12 normwise relative; the batched FP32 apply within 1e-6 normwise relative
(max |err| / max |ref|).
"""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu

GRAD_LAP_2D = [[(1, 0)], [(0, 1)], [(2, 0), (0, 2)], [(1, 1)]]
GRAD_LAP_3D = W.grad_lap_outputs(3)


def _case(name):
    if name == "2d":
        pos, h = W.lattice(24, 2, jitter=0.15, seed=11)
        return dict(pos=pos, rcut=3.1 * h, outputs=GRAD_LAP_2D, order=2)
    if name == "3d":
        pos, h = W.lattice(12, 3, jitter=0.15, seed=12)
        return dict(pos=pos, rcut=2.8 * h, outputs=GRAD_LAP_3D, order=2)
    if name == "3d_periodic":
        h = 1.0 / 10
        pos, _ = W.lattice(10, 3, h=h, jitter=0.1, seed=13)
        pos = np.mod(pos, 1.0)
        return dict(pos=pos, rcut=2.8 * h, outputs=[[(2, 0, 0), (0, 2, 0), (0, 0, 2)]], order=2,
                    box=((0.0,) * 3, (1.0,) * 3, (1, 1, 1)))
    if name == "2d_lattice":
        pos, h = W.lattice(16, 2)
        return dict(pos=pos, rcut=3.1 * h, outputs=[[(1, 0)], [(2, 0), (0, 2)]], order=2)
    if name == "2d_order3":
        pos, h = W.lattice(20, 2, jitter=0.1, seed=14)
        return dict(pos=pos, rcut=3.6 * h, outputs=[[(1, 0)], [(2, 0), (0, 2)]], order=3)
    if name == "2d_adaptive":
        pos, h = W.lattice(20, 2, jitter=0.1, seed=15)
        rpp = (2.9 + 0.6 * np.random.default_rng(15).random(pos.shape[0])) * h
        return dict(pos=pos, rcut=0.0, rcut_pp=rpp, outputs=[[(1, 0)], [(0, 1)], [(2, 0), (0, 2)]], order=2)
    if name == "2d_hoe05":
        pos, h = W.lattice(18, 2, jitter=0.1, seed=16)
        return dict(pos=pos, rcut=3.1 * h, outputs=[[(1, 0)], [(2, 0), (0, 2)]], order=2, hoe=0.5)
    if name == "2d_sparse":
        pos, h = W.lattice(14, 2, jitter=0.2, seed=17)
        return dict(pos=pos, rcut=2.05 * h, outputs=[[(1, 0)], [(2, 0), (0, 2)]], order=2)
    if name == "2d_lattice_tie":
        # candidates exactly on the cutoff (distance 5h = |(5, 0)h| = |(3, 4)h|
        # on an exact lattice): the FP32 pre-filter leaves them to the FP64
        # predicate
        pos, h = W.lattice(16, 2)
        return dict(pos=pos, rcut=5.0 * h, outputs=[[(1, 0)], [(2, 0), (0, 2)]], order=2)
    if name == "2d_periodic_2cells":
        # two cells per periodic axis: every candidate takes the FP64 test
        h = 1.0 / 8
        pos, _ = W.lattice(8, 2, h=h, jitter=0.1, seed=18)
        pos = np.mod(pos, 1.0)
        return dict(pos=pos, rcut=2.8 * h, outputs=[[(1, 0)], [(2, 0), (0, 2)]], order=2,
                    box=((0.0, 0.0), (1.0, 1.0), (1, 1)))
    raise KeyError(name)


CASES = ["2d", "3d", "3d_periodic", "2d_lattice", "2d_order3", "2d_adaptive", "2d_hoe05", "2d_sparse",
         "2d_lattice_tie", "2d_periodic_2cells"]


def _build(c, flags=C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32):
    dim = c["pos"].shape[1]
    plan = DcpsePlan(dim, c["outputs"], order=c["order"], h_over_eps=c.get("hoe", 0.9), box=c.get("box"))
    pos = torch.tensor(c["pos"], device="cuda")
    rpp = torch.tensor(c["rcut_pp"], device="cuda") if c.get("rcut_pp") is not None else None
    plan.build_neighbors(pos, c["rcut"], rpp)
    rc = plan.assemble(pos, flags)
    return plan, pos, rc


def _oracle_terms(orc, c, rp, cols):
    res = []
    for o, out in enumerate(c["outputs"]):
        for s in out:
            eps, eip, K, st = orc.assemble(c["pos"], rp, cols, s, c["order"], box=c.get("box"),
                                           h_over_eps=c.get("hoe", 0.9))
            res.append(dict(sig=s, out=o, eps=eps, eip=eip, K=K, st=st))
    return res


def _group_order(terms):
    keys = []
    for t in terms:
        k = sum(t["sig"])
        if k not in keys:
            keys.append(k)
    return keys


@pytest.mark.parametrize("name", CASES)
def test_neighbors_bitexact(cuda, orc, name):
    c = _case(name)
    plan, pos, _ = _build(c)
    rp_o, cols_o = orc.neighbors(c["pos"], c["rcut"], rcut_pp=c.get("rcut_pp"), box=c.get("box"))
    rp, cols = plan.neighbors()
    assert np.array_equal(rp.cpu().numpy(), rp_o)
    assert np.array_equal(cols.cpu().numpy(), cols_o)
    assert plan.info()["max_neighbors"] == int(np.diff(rp_o).max())


@pytest.mark.parametrize("name", CASES)
def test_assembly_bitexact(cuda, orc, name):
    c = _case(name)
    plan, pos, rc = _build(c)
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    terms = _oracle_terms(orc, c, rp, cols)
    eps, st = (x.cpu().numpy() for x in plan.eps())
    # eps is the same for every term
    assert np.array_equal(eps.view(np.int64), terms[0]["eps"].view(np.int64))
    for t, ref in enumerate(terms):
        K, eip = plan.term_kernels(t)
        K = K.cpu().numpy()
        eip = eip.cpu().numpy()
        assert np.array_equal(eip, ref["eip"]), "eps^-|alpha| of term %d" % t
        ok = ref["st"] == 0
        assert np.array_equal(K, ref["K"]), "kernels of term %d differ: max %g" % (t, np.abs(K - ref["K"]).max())
    # particle status = first failing basis in group order
    keys = _group_order(terms)
    expect = np.zeros_like(st)
    for k in keys:
        s_g = next(t["st"] for t in terms if sum(t["sig"]) == k)
        expect = np.where(expect == 0, s_g, expect)
    assert np.array_equal(st, expect)
    assert (rc == C.ERR_PARTICLES) == bool(np.any(expect != 0))


@pytest.mark.parametrize("name", CASES)
def test_apply_parity(cuda, orc, name):
    c = _case(name)
    plan, pos, _ = _build(c)
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    terms = _oracle_terms(orc, c, rp, cols)
    f = np.random.default_rng(5).standard_normal(c["pos"].shape[0])
    ft = torch.tensor(f, device="cuda")
    # per term, reference order: bit-exact
    for t, ref in enumerate(terms):
        got = plan.apply_term_f64(t, ft).cpu().numpy()
        exp = orc.apply(f, rp, cols, ref["K"], ref["eip"], sum(ref["sig"]))
        assert np.array_equal(got, exp), "term %d" % t
    # outputs composed as the reference does (VECT_DCPSE_V_SUM): bit-exact
    refs = []
    for o in range(len(c["outputs"])):
        ts = [t for t in terms if t["out"] == o]
        exp = orc.apply_sum(f, rp, cols, [t["K"] for t in ts], [t["eip"] for t in ts], [sum(t["sig"]) for t in ts])
        got = plan.apply_output_f64(o, ft).cpu().numpy()
        assert np.array_equal(got, exp), "output %d" % o
        refs.append(exp)
    refs = np.stack(refs)
    # batched FP64 (summed, eps-folded weights, difference form)
    b64 = plan.apply(ft, C.F64).cpu().numpy()
    for o in range(len(refs)):
        err = np.abs(b64[o] - refs[o]).max() / np.abs(refs[o]).max()
        assert err <= 1e-12, (o, err)
    # batched FP32
    b32 = plan.apply(ft, C.F32).cpu().numpy()
    for o in range(len(refs)):
        err = np.abs(b32[o] - refs[o]).max() / np.abs(refs[o]).max()
        assert err <= 1e-6, (o, err)
    # host-buffer entry point equals the device one
    h32 = plan.apply_host(f, precision=C.F32)
    assert np.array_equal(h32, b32)


@pytest.mark.parametrize("name", ["2d", "3d", "3d_periodic", "2d_order3"])
def test_fast_assembly_close(cuda, orc, name):
    c = _case(name)
    plan, pos, _ = _build(c, C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    terms = _oracle_terms(orc, c, rp, cols)
    _, st = plan.eps()
    ok = st.cpu().numpy() == 0
    for o in range(len(c["outputs"])):
        w_ref = np.zeros(rp[-1])
        for t in terms:
            if t["out"] == o:
                w_ref = w_ref + t["K"] * np.repeat(t["eip"], np.diff(rp))
        w64, w32 = plan.output_weights(o)
        w64 = w64.cpu().numpy()
        for p in np.where(ok)[0]:
            a, b = rp[p], rp[p + 1]
            scale = np.abs(w_ref[a:b]).max()
            assert np.abs(w64[a:b] - w_ref[a:b]).max() <= 1e-12 * scale, (o, p)
        assert np.array_equal(w32.cpu().numpy(), w64.astype(np.float32))


@pytest.mark.parametrize("name", ["2d", "3d", "2d_adaptive", "2d_sparse"])
def test_apply_schedules(cuda, orc, name):
    """Direct and TMA-staged loading give identical bits; every lane count
    and the bf16-residual correction stay within their bars."""
    c = _case(name)
    plan, pos, _ = _build(c, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32 | C.STORE_OUT_F32_RESID)
    f = torch.tensor(np.random.default_rng(8).standard_normal(c["pos"].shape[0]), device="cuda")
    refs = torch.stack([plan.apply_output_f64(o, f) for o in range(len(c["outputs"]))]).cpu().numpy()
    staged = 0
    for lanes in (4, 8, 16, 32):
        res = {}
        for mode in (1, 2, 3, 1 | 16):
            plan.set_apply_config(lanes, mode)
            try:
                res[mode] = plan.apply(f, C.F32).clone()
            except C.DcpseError as e:  # staged tiles larger than shared memory
                assert mode == 2 and e.code == C.ERR_CAPACITY
                continue
            plan.check()
        assert torch.equal(res[1], res[3]), lanes
        if 2 in res:
            staged += 1
            assert torch.equal(res[1], res[2]), lanes
        for m in (1, 1 | 16):
            got = res[m].cpu().numpy()
            for o in range(len(refs)):
                assert np.abs(got[o] - refs[o]).max() <= 1e-6 * np.abs(refs[o]).max()
        for mode in (1, 2) if 2 in res else (1,):
            plan.set_apply_config(lanes, mode)
            try:
                g = plan.apply(f, C.F32_RESID).cpu().numpy()
            except C.DcpseError as e:  # the residual streams make the tiles larger
                assert mode == 2 and e.code == C.ERR_CAPACITY
                continue
            for o in range(len(refs)):
                err = np.abs(g[o] - refs[o]).max() / np.abs(refs[o]).max()
                assert err <= 1e-9, (lanes, mode, o, err)
    assert staged >= 1  # the TMA-staged kernel ran for at least one lane count
    # sliced ELL layout (thread per row): within the FP32 bar, with and
    # without compensated sums for every output; the residual precision
    # falls back to the CSR kernels
    for mode in (4, 4 | 16):
        plan.set_apply_config(0, mode)
        got = plan.apply(f, C.F32).cpu().numpy()
        plan.check()
        for o in range(len(refs)):
            assert np.abs(got[o] - refs[o]).max() <= 1e-6 * np.abs(refs[o]).max(), (mode, o)
        g = plan.apply(f, C.F32_RESID).cpu().numpy()
        for o in range(len(refs)):
            assert np.abs(g[o] - refs[o]).max() <= 1e-9 * np.abs(refs[o]).max(), (mode, o)
    # batched FP64: CSR kernel (mode 1) and sliced layout (modes 0 and 4)
    if plan.output_weights(0)[0] is not None:
        for mode in (1, 4, 0):
            plan.set_apply_config(0, mode)
            g = plan.apply(f, C.F64).cpu().numpy()
            for o in range(len(refs)):
                assert np.abs(g[o] - refs[o]).max() <= 1e-12 * np.abs(refs[o]).max(), (mode, o)
    plan.set_apply_config(0, 0)


@pytest.mark.parametrize("name", ["2d_adaptive", "3d"])
def test_assembly_schedules_bitexact(cuda, orc, name):
    """Neighbour-count binning, CTA size and QR lane grouping change the
    schedule only."""
    c = _case(name)
    plan, pos, _ = _build(c)
    ref = [plan.term_kernels(t)[0].clone() for t in range(plan.n_terms)]
    for bw, wp, ql in ((4, 2, 0), (16, 8, 1), (1, 4, 2), (0, 4, 4), (0, 4, 8), (0, 2, 16), (0, 8, 32)):
        plan.set_assembly_config(bw, wp, ql)
        try:
            plan.assemble(pos, C.STORE_TERMS_F64 | C.STORE_OUT_F64 | C.STORE_OUT_F32)
        except C.DcpseError as e:  # QR work space larger than shared memory
            assert ql in (1, 2) and e.code == C.ERR_CAPACITY
            continue
        for t in range(plan.n_terms):
            assert torch.equal(plan.term_kernels(t)[0], ref[t]), (bw, wp, ql, t)
    from openfpm_numerics_gb300 import autotune

    best = autotune.tune_assembly(plan, pos, C.ASSEMBLE_FAST | C.STORE_OUT_F32)
    assert len(best["sweep"]) >= 11 and best["warps"] in (2, 4, 8) and best["qr_lanes"] in (0, 2, 4, 8, 16)


def test_autotune(cuda):
    from openfpm_numerics_gb300 import autotune

    c = _case("3d")
    plan, pos, _ = _build(c, C.STORE_OUT_F32)
    f = torch.tensor(np.random.default_rng(9).standard_normal(c["pos"].shape[0]), device="cuda")
    ref = plan.apply(f, C.F32).clone()
    best = autotune.tune_apply(plan, f, reps=2, warmup=1)
    # 3 lane counts x 3 CSR kernels + the sliced ELL kernel (lanes do not apply: 0)
    assert len(best["sweep"]) == 10 and best["lanes"] in (0, 4, 8, 16)
    assert any(e["mode"] == "sliced-ell" and e["ms"] is not None for e in best["sweep"])
    got = plan.apply(f, C.F32)
    assert torch.allclose(got, ref, rtol=0, atol=1e-6 * ref.abs().max().item())


def test_analytic_config1_laplacian(cuda):
    cfg = W.config1()
    c = dict(pos=cfg["pos"], rcut=cfg["rcut"], outputs=[[(2, 0), (0, 2)]], order=2)
    plan, pos, _ = _build(c)
    f, lf = W.field1(cfg["pos"])
    ft = torch.tensor(f, device="cuda")
    inner = W.interior_mask(cfg["pos"], cfg["rcut"])
    for prec in (C.F64, C.F32):
        lap = plan.apply(ft, prec)[0].cpu().numpy()
        rel = np.abs(lap - lf)[inner].max() / np.abs(lf).max()
        assert rel < 2e-2


def test_edge_cases(cuda):
    # empty particle set
    plan = DcpsePlan(2, [[(1, 0)]])
    pos = torch.zeros((0, 2), dtype=torch.float64, device="cuda")
    plan.build_neighbors(pos, 0.1)
    assert plan.info()["nnz"] == 0
    assert plan.assemble(pos) == C.OK
    out = plan.apply(torch.zeros(0, dtype=torch.float64, device="cuda"))
    assert out.shape == (1, 0)
    # isolated particle and a NaN position: flagged, weights zero, others fine
    p, h = W.lattice(10, 2, jitter=0.1, seed=3)
    p = np.concatenate([p, [[5.0, 5.0]], [[np.nan, 0.5]]])
    plan = DcpsePlan(2, [[(1, 0)]], box=((0, 0), (6, 6), (0, 0)))
    pt = torch.tensor(p, device="cuda")
    plan.build_neighbors(pt, 3.1 * h)
    rc = plan.assemble(pt)
    assert rc == C.ERR_PARTICLES
    nb, first, code = plan.particle_status()
    eps, st = plan.eps()
    st = st.cpu().numpy()
    assert st[-1] != 0 and st[-2] == C.PART_TOO_FEW and first <= len(p) - 2
    w64, _ = plan.output_weights(0)
    assert torch.isfinite(w64).all()
    # state errors
    plan2 = DcpsePlan(2, [[(1, 0)]])
    with pytest.raises(C.DcpseError) as ei:
        plan2.apply(torch.zeros(4, dtype=torch.float64, device="cuda"))
    assert ei.value.code == C.ERR_STATE


def test_term_basis_matches_oracle(cuda, orc):
    plan = DcpsePlan(3, GRAD_LAP_3D, order=2)
    t = 0
    for out in GRAD_LAP_3D:
        for s in out:
            e, _ = orc.basis(3, s, 2)
            assert np.array_equal(plan.term_basis(t), e)
            t += 1


def test_host_apply_chunked_equals_device(cuda):
    """Host buffers above the chunking threshold: the outputs come back in row
    chunks overlapped with the apply (pageable outputs) or are stored by the
    apply itself (pinned outputs); both equal the device apply bit for bit
    (also with the bf16 residual stream)."""
    pos, h = W.lattice(48, 3, jitter=0.15, seed=19)
    plan = DcpsePlan(3, GRAD_LAP_3D, order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 2.8 * h)
    plan.assemble(pt, C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.STORE_OUT_F32_RESID)
    f = np.cos(5 * pos[:, 0]) * pos[:, 2] + pos[:, 1]
    # pinned outputs are written by the kernels directly (mapped host memory)
    pinned = torch.empty((plan.n_outputs, pos.shape[0]), dtype=torch.float64, pin_memory=True)
    pinned_f = torch.tensor(f).pin_memory()
    for prec in (C.F32, C.F32_RESID):
        dev = plan.apply(torch.tensor(f, device="cuda"), prec).cpu().numpy()
        for _ in range(2):
            host = plan.apply_host(f, precision=prec)
            assert np.array_equal(host, dev)
            pinned.fill_(np.nan)
            plan.apply_host(f, pinned.numpy(), precision=prec)
            assert np.array_equal(pinned.numpy(), dev)
            # pinned field as well: split in place from host memory
            pinned.fill_(np.nan)
            plan.apply_host(pinned_f.numpy(), pinned.numpy(), precision=prec)
            assert np.array_equal(pinned.numpy(), dev)
    plan.close()


def test_host_apply_after_particle_count_grows(cuda):
    """A new neighbour list with more particles than the last host-buffer
    call saw: the device staging of pageable buffers is re-sized (copy
    pipeline and the single-copy FP64 path)."""
    plan = DcpsePlan(3, GRAD_LAP_3D, order=2)
    for nside in (44, 52):
        pos, h = W.lattice(nside, 3, jitter=0.15, seed=nside)
        pt = torch.tensor(pos, device="cuda")
        plan.build_neighbors(pt, 2.8 * h)
        plan.assemble(pt, C.ASSEMBLE_FAST | C.STORE_OUT_F32 | C.STORE_OUT_F64)
        f = np.sin(3 * pos[:, 0]) + pos[:, 1] * pos[:, 2]
        for prec in (C.F32, C.F64):
            dev = plan.apply(torch.tensor(f, device="cuda"), prec).cpu().numpy()
            assert np.array_equal(plan.apply_host(f, precision=prec), dev)
    plan.close()


def test_lengths_checked_before_the_device(cuda):
    """Arrays whose length does not match the plan's particle set are refused
    on the host (the C-ABI takes bare pointers sized by the plan)."""
    pos, h = W.lattice(12, 2, jitter=0.1, seed=20)
    plan = DcpsePlan(2, [[(1, 0)], [(2, 0), (0, 2)]], order=2)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 3.1 * h)
    plan.assemble(pt)
    n = pos.shape[0]
    short = torch.zeros(n - 1, dtype=torch.float64, device="cuda")
    good = torch.zeros(n, dtype=torch.float64, device="cuda")
    for call in (lambda: plan.apply(short), lambda: plan.apply_term_f64(0, short),
                 lambda: plan.apply_output_f64(0, short), lambda: plan.apply_host(np.zeros(n + 1)),
                 lambda: plan.assemble(pt[:-1]), lambda: plan.vjp_field(torch.zeros((2, n - 1), device="cuda")),
                 lambda: plan.apply(good, C.F32, torch.empty((2, n - 1), dtype=torch.float64, device="cuda")),
                 lambda: plan.apply_host(np.zeros(n), np.empty((2, n), dtype=np.float32))):
        with pytest.raises(ValueError):
            call()
    # the plan is untouched
    assert plan.apply(good).shape == (2, n)
    plan.close()
