"""RK4 reaction-diffusion (configuration 5 pattern) on a periodic box: the
fused stage kernels against a generic RK4 written with the plan's apply, CUDA
graph replay against eager stepping, and the checkpointed adjoint against a
directional central difference (FP64), then the same in FP32."""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.odeint import GrayScottRK4, runge_kutta4
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu

P = dict(Du=2e-5, Dv=1e-5, F=0.04, k=0.06)


def _setup(nside, dtype):
    cfg = W.config5(nside)
    plan = DcpsePlan(3, [[(2, 0, 0), (0, 2, 0), (0, 0, 2)]], box=cfg["box"])
    pos = torch.tensor(cfg["pos"], device="cuda")
    plan.build_neighbors(pos, cfg["rcut"])
    plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    u0, v0 = W.gray_scott_initial(cfg["pos"], radius=0.15)
    u = torch.tensor(u0, device="cuda", dtype=dtype)
    v = torch.tensor(v0, device="cuda", dtype=dtype)
    # the step of the 96^3 configuration (0.2 h^2 / Du at h = 1/96); on this
    # coarser set 0.2 h^2 / Du would take the reaction terms past RK4's
    # stability limit ((F + k) dt = 3.9)
    dt = 0.2 * (1.0 / 96) ** 2 / P["Du"]
    return plan, u, v, dt


def test_fused_rk4_matches_generic(cuda):
    plan, u, v, dt = _setup(16, torch.float64)
    gs = GrayScottRK4(plan, u, v, P["Du"], P["Dv"], P["F"], P["k"], dt)

    def rhs(y, t):
        uu, vv = y
        L = lambda f: plan.apply(f, C.F64)[0]  # noqa: E731
        uvv = uu * vv * vv
        return (P["Du"] * L(uu) - uvv + P["F"] * (1 - uu), P["Dv"] * L(vv) + uvv - (P["F"] + P["k"]) * vv)

    y = (u.clone(), v.clone())
    for _ in range(5):
        gs.step()
        y = runge_kutta4(rhs, y, 0.0, dt)
    for a, b in ((gs.u, y[0]), (gs.v, y[1])):
        assert (a - b).abs().max().item() <= 1e-12 * b.abs().max().item()


def test_graph_replay_equals_eager(cuda):
    plan, u, v, dt = _setup(16, torch.float32)
    s = torch.cuda.Stream()
    plan.set_stream(s)
    eager = GrayScottRK4(plan, u, v, P["Du"], P["Dv"], P["F"], P["k"], dt)
    graph = GrayScottRK4(plan, u, v, P["Du"], P["Dv"], P["F"], P["k"], dt)
    with torch.cuda.stream(s):
        for _ in range(11):  # the capture below runs one warm-up step first
            eager.step()
    graph.capture(5, s)
    with torch.cuda.stream(s):
        graph.run(10)
    s.synchronize()
    assert torch.equal(eager.u, graph.u) and torch.equal(eager.v, graph.v)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-7), (torch.float32, 2e-2)])
def test_checkpointed_adjoint(cuda, dtype, tol):
    plan, u, v, dt = _setup(16, dtype)
    gs = GrayScottRK4(plan, u, v, P["Du"], P["Dv"], P["F"], P["k"], dt)
    gs.run(10)
    every, nseg = 5, 2
    start = (gs.u.clone(), gs.v.clone())
    wgt = torch.tensor(np.random.default_rng(7).standard_normal(u.numel()), device="cuda", dtype=dtype)

    def J(state):
        g2 = GrayScottRK4(plan, state[0], state[1], P["Du"], P["Dv"], P["F"], P["k"], dt)
        g2.run(every * nseg)
        return float((g2.v.double() * wgt.double()).sum())

    ckpts = []
    for sgm in range(nseg):
        ckpts.append((gs.u.clone(), gs.v.clone()))
        gs.run(every)
    ybar = (torch.zeros_like(gs.u), wgt.clone())
    ub, vb = gs.backward(ckpts, every, ybar)
    delta = torch.tensor(np.random.default_rng(8).standard_normal(u.numel()), device="cuda", dtype=dtype)
    h = 1e-6 if dtype == torch.float64 else 1e-2
    jp = J((start[0], start[1] + h * delta))
    jm = J((start[0], start[1] - h * delta))
    fd = (jp - jm) / (2 * h)
    ad = float((vb.double() * delta.double()).sum())
    assert abs(fd - ad) <= tol * abs(fd), (fd, ad)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 2e-5)])
def test_adjoint_stage_equals_transposed_jacobian(cuda, dtype, tol):
    """One adjoint stage against J(Y)^T kbar written with the Laplacian as a
    sparse matrix L = W - diag(row sums of W): ubar = Du L^T kbar_u
    - (v^2 + F) kbar_u + v^2 kbar_v, vbar = Dv L^T kbar_v - 2 u v kbar_u
    + (2 u v - F - k) kbar_v; accumulated into acc, and the next stage's kbar
    = cy ybar + cY Ybar."""
    import scipy.sparse as sp

    plan, u, v, dt = _setup(16, dtype)
    gs = GrayScottRK4(plan, u, v, P["Du"], P["Dv"], P["F"], P["k"], dt)
    gs.prepare_adjoint()
    n = u.numel()
    rng = np.random.default_rng(9)
    Y = tuple(torch.tensor(rng.uniform(0.2, 1.0, n), device="cuda", dtype=dtype) for _ in range(2))
    kb = tuple(torch.tensor(rng.standard_normal(n), device="cuda", dtype=dtype) for _ in range(2))
    yb = tuple(torch.tensor(rng.standard_normal(n), device="cuda", dtype=dtype) for _ in range(2))
    acc0 = tuple(torch.tensor(rng.standard_normal(n), device="cuda", dtype=dtype) for _ in range(2))
    acc = tuple(a.clone() for a in acc0)
    nxt = (torch.empty_like(u), torch.empty_like(u))
    cy, cY = dt / 3.0, dt / 2.0
    gs._adj_stage(Y, kb, yb, acc, nxt, cy, cY)
    torch.cuda.synchronize()
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    w = plan.output_weights(0)[0 if dtype == torch.float64 else 1].double().cpu().numpy()
    W_ = sp.csr_matrix((w, cols, rp), shape=(n, n))
    L = W_ - sp.diags(np.asarray(W_.sum(axis=1)).ravel())
    Yu, Yv, ku, kv, bu, bv = (t.double().cpu().numpy() for t in (*Y, *kb, *yb))
    Ybu = P["Du"] * (L.T @ ku) - (Yv ** 2 + P["F"]) * ku + Yv ** 2 * kv
    Ybv = P["Dv"] * (L.T @ kv) - 2 * Yu * Yv * ku + (2 * Yu * Yv - P["F"] - P["k"]) * kv
    for got, ref in ((acc[0].double().cpu().numpy() - acc0[0].double().cpu().numpy(), Ybu),
                     (acc[1].double().cpu().numpy() - acc0[1].double().cpu().numpy(), Ybv),
                     (nxt[0].double().cpu().numpy(), cy * bu + cY * Ybu),
                     (nxt[1].double().cpu().numpy(), cy * bv + cY * Ybv)):
        scale = np.abs(ref).max() + np.abs(acc0[0].double().cpu().numpy()).max()
        assert np.abs(got - ref).max() <= tol * scale


@pytest.mark.parametrize("dtype,bar", [(torch.float64, 1e-10), (torch.float32, 2e-5)])
def test_rk4_matches_oracle_rk4(cuda, orc, dtype, bar):
    """Five fused RK4 steps against a classic RK4 whose Laplacian is the
    oracle's (the reference's three Dcpse terms 2e_i, assembled and applied
    in the reference's order on the periodic set); src/OdeIntegrators/tests/
    OdeIntegratores_base_tests.cpp:33-72 defines the stepping."""
    cfg = W.config5(12)
    plan, u, v, dt = _setup(12, dtype)
    pos = cfg["pos"]
    rp, cols = orc.neighbors(pos, cfg["rcut"], box=cfg["box"])
    terms = [orc.assemble(pos, rp, cols, s, 2, box=cfg["box"]) for s in [(2, 0, 0), (0, 2, 0), (0, 0, 2)]]

    def L(fld):
        return orc.apply_sum(fld, rp, cols, [t[2] for t in terms], [t[1] for t in terms], [2, 2, 2])

    def rhs(y, t):
        uu, vv = y
        uvv = uu * vv * vv
        return (P["Du"] * L(uu) - uvv + P["F"] * (1 - uu), P["Dv"] * L(vv) + uvv - (P["F"] + P["k"]) * vv)

    gs = GrayScottRK4(plan, u, v, P["Du"], P["Dv"], P["F"], P["k"], dt)
    y = (u.double().cpu().numpy(), v.double().cpu().numpy())
    for _ in range(5):
        gs.step()
        y = runge_kutta4(rhs, y, 0.0, dt)
    for a, b in ((gs.u, y[0]), (gs.v, y[1])):
        a = a.double().cpu().numpy()
        assert np.abs(a - b).max() <= bar * np.abs(b).max()


def test_graph_backward_equals_eager(cuda):
    """The checkpointed backward with its segments replayed from a CUDA graph
    gives the eager backward's gradient bit for bit (FP32 state)."""
    plan, u, v, dt = _setup(16, torch.float32)
    s = torch.cuda.Stream()
    plan.set_stream(s)
    with torch.cuda.stream(s):
        gs = GrayScottRK4(plan, u, v, P["Du"], P["Dv"], P["F"], P["k"], dt)
        gs.run(6)
        ckpts = []
        for _ in range(3):
            ckpts.append((gs.u.clone(), gs.v.clone()))
            gs.run(4)
        ybar = (torch.zeros_like(gs.u), torch.ones_like(gs.v))
        eager = gs.backward(ckpts, 4, ybar)
        graph = gs.backward(ckpts, 4, ybar, stream=s)
    s.synchronize()
    assert torch.equal(eager[0], graph[0]) and torch.equal(eager[1], graph[1])


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_fused_reverse_step_equals_stages(cuda, dtype):
    """dcpse_rk4_gs_reverse_step (the four adjoint stages in five kernels,
    kbar kept as pairs) gives the separate stages' ybar bit for bit."""
    plan, u, v, dt = _setup(16, dtype)
    gs = GrayScottRK4(plan, u, v, P["Du"], P["Dv"], P["F"], P["k"], dt)
    gs.run(3)
    gs.prepare_adjoint()
    hist = [(torch.empty_like(gs.u), torch.empty_like(gs.v)) for _ in range(4)]
    gs.step(record=hist)
    g = torch.Generator(device="cuda").manual_seed(7)
    yb0 = (torch.rand(gs.u.shape, generator=g, device="cuda", dtype=dtype),
           torch.rand(gs.v.shape, generator=g, device="cuda", dtype=dtype))
    bufs = [(torch.empty_like(gs.u), torch.empty_like(gs.v)) for _ in range(3)]
    ref = (yb0[0].clone(), yb0[1].clone())
    gs._reverse_step_stages(hist, ref, *bufs)
    got = (yb0[0].clone(), yb0[1].clone())
    gs._reverse_step_into(hist, got, bufs[0])
    torch.cuda.synchronize()
    assert torch.equal(got[0], ref[0]) and torch.equal(got[1], ref[1])
