"""Adjoint of the DC-PSE apply (configuration 4 pattern): field and position
gradients of the hand-written backward (torch.autograd.Function over the
C-ABI) against central finite differences and the oracle's FP64 reference
adjoint.  Neighbour lists are held fixed."""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import _capi as C
from openfpm_numerics_gb300 import workloads as W
from openfpm_numerics_gb300.autograd import dcpse_apply
from openfpm_numerics_gb300.plan import DcpsePlan

pytestmark = pytest.mark.gpu


def _dense_L(rp, cols, w, n):
    L = np.zeros((n, n))
    for p in range(n):
        for j in range(rp[p], rp[p + 1]):
            L[p, cols[j]] += w[j]
            L[p, p] -= w[j]
    return L


def test_vjp_field_matches_transpose(cuda):
    pos, h = W.lattice(16, 2, jitter=0.15, seed=31)
    outputs = [[(2, 0), (0, 2)], [(1, 0)], [(1, 1)]]
    plan = DcpsePlan(2, outputs)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 3.1 * h)
    plan.assemble(pt, C.ASSEMBLE_FAST | C.STORE_OUT_F64 | C.STORE_OUT_F32)
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    n = pos.shape[0]
    g = np.random.default_rng(2).standard_normal((3, n))
    exp = np.zeros(n)
    for o in range(3):
        w64, _ = plan.output_weights(o)
        exp += _dense_L(rp, cols, w64.cpu().numpy(), n).T @ g[o]
    got = plan.vjp_field(torch.tensor(g, device="cuda"), C.F64).cpu().numpy()
    assert np.abs(got - exp).max() <= 1e-12 * np.abs(exp).max()
    got32 = plan.vjp_field(torch.tensor(g, device="cuda"), C.F32).cpu().numpy()
    assert np.abs(got32 - exp).max() <= 1e-6 * np.abs(exp).max()
    # <L f, g> == <f, L^T g>
    f = torch.tensor(np.random.default_rng(3).standard_normal(n), device="cuda")
    lhs = float((plan.apply(f, C.F64) * torch.tensor(g, device="cuda")).sum())
    rhs = float((f * torch.tensor(got, device="cuda")).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("outputs", [[[(2, 0), (0, 2)]], [[(2, 0), (0, 2)], [(1, 0)], [(0, 1)]]])
def test_vjp_positions_vs_reference_adjoint(cuda, orc, outputs):
    pos, h = W.lattice(20, 2, jitter=0.1, seed=32)
    n = pos.shape[0]
    plan = DcpsePlan(2, outputs)
    pt = torch.tensor(pos, device="cuda")
    plan.build_neighbors(pt, 3.1 * h)
    plan.assemble(pt, C.ASSEMBLE_FAST | C.STORE_OUT_F64)
    rp, cols = (x.cpu().numpy() for x in plan.neighbors())
    rng = np.random.default_rng(4)
    f = rng.standard_normal(n)
    g = rng.standard_normal((len(outputs), n))
    got = plan.vjp_positions(pt, torch.tensor(f, device="cuda"), torch.tensor(g, device="cuda")).cpu().numpy()
    ref = orc.vjp_positions(pos, rp, cols, outputs, f, g)
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_config4_adjoint_fd(cuda, orc):
    """256^2 jittered particles, Laplacian, loss = ||L f - g||^2: autograd
    gradients vs central differences (step 1e-6 h) on 200 random coordinates
    and vs the FP64 reference adjoint."""
    cfg = W.config4()
    pos_np, h, f_np, g_np = cfg["pos"], cfg["h"], cfg["f"], cfg["g"]
    n = pos_np.shape[0]
    outputs = [[(2, 0), (0, 2)]]
    plan = DcpsePlan(2, outputs)
    pos0 = torch.tensor(pos_np, device="cuda")
    plan.build_neighbors(pos0, cfg["rcut"])
    rp, cols = plan.neighbors()
    rp, cols = rp.clone(), cols.clone()  # the list held fixed from here on
    g = torch.tensor(g_np, device="cuda")
    f = torch.tensor(f_np, device="cuda", requires_grad=True)
    pos = pos0.clone().requires_grad_(True)
    y = dcpse_apply(f, pos, plan)[0]
    loss = ((y - g) ** 2).sum()
    loss.backward()
    gf = f.grad.detach().cpu().numpy()
    gp = pos.grad.detach().cpu().numpy()

    def yfun(P, F):
        plan.set_neighbors(rp, cols)
        plan.assemble(P, C.ASSEMBLE_FAST | C.STORE_OUT_F64)
        return plan.apply(F, C.F64)[0]

    rng = np.random.default_rng(5)
    coords = rng.choice(n * 2, 200, replace=False)
    step = 1e-6 * h
    fd, ad = [], []
    y0 = y.detach()
    fz = f.detach()
    for c in coords:
        i, d = divmod(int(c), 2)
        P = pos0.clone()
        P[i, d] += step
        yp = yfun(P, fz)
        P[i, d] -= 2 * step
        ym = yfun(P, fz)
        # loss(+) - loss(-) summed row by row (unaffected rows cancel exactly)
        dl = float(((yp - ym) * (yp + ym - 2 * g)).sum())
        fd.append(dl / (2 * step))
        ad.append(gp[i, d])
    fd, ad = np.array(fd), np.array(ad)
    err = np.abs(fd - ad).max() / np.abs(fd).max()
    assert err < 1e-5, err
    # field gradient: the loss is quadratic in f
    idx = rng.choice(n, 200, replace=False)
    fdf = []
    sf = 1e-3
    for i in idx:
        F = fz.clone()
        F[i] += sf
        yp = yfun(pos0, F)
        F[i] -= 2 * sf
        ym = yfun(pos0, F)
        fdf.append(float(((yp - ym) * (yp + ym - 2 * g)).sum()) / (2 * sf))
    fdf = np.array(fdf)
    assert np.abs(fdf - gf[idx]).max() <= 1e-8 * np.abs(fdf).max()
    # FP64 reference adjoint (oracle) with the same cotangent
    cot = (2 * (y0 - g)).cpu().numpy()[None, :]
    ref = orc.vjp_positions(pos_np, rp.cpu().numpy(), cols.cpu().numpy(), outputs, f_np, cot)
    assert np.abs(gp - ref).max() <= 1e-9 * np.abs(ref).max()


def test_backward_reassembles_only_when_the_plan_changed(cuda):
    """The backward skips the re-assembly when the plan still holds the
    forward's weights (same generation), and re-assembles when another
    assembly ran in between: the gradients are the same either way."""
    pos_np, h = W.lattice(40, 2, jitter=0.1, seed=21)
    plan = DcpsePlan(2, [[(2, 0), (0, 2)]])
    pos0 = torch.tensor(pos_np, device="cuda")
    plan.build_neighbors(pos0, 3.1 * h)
    g = torch.tensor(np.random.default_rng(22).standard_normal(pos_np.shape[0]), device="cuda")
    f0 = torch.tensor(np.sin(3 * pos_np[:, 0]) * pos_np[:, 1], device="cuda")

    def grads(between=None):
        f = f0.clone().requires_grad_(True)
        pos = pos0.clone().requires_grad_(True)
        y = dcpse_apply(f, pos, plan)[0]
        gen = plan.generation
        if between is not None:
            between()
        ((y - g) ** 2).sum().backward()
        return f.grad.clone(), pos.grad.clone(), plan.generation - gen

    gf, gp, bumps = grads()
    assert bumps == 0  # no re-assembly in backward
    # an assembly at other positions between forward and backward
    moved = pos0 + 0.05 * h
    gf2, gp2, bumps2 = grads(lambda: plan.assemble(moved, C.ASSEMBLE_FAST | C.STORE_OUT_F64))
    assert bumps2 == 2  # the intervening assembly and the backward's own
    assert torch.equal(gf, gf2) and torch.equal(gp, gp2)
    plan.close()
