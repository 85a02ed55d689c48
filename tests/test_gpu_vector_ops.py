"""Divergence, Advection and Curl2D (DCPSE_op.hpp:1226-1781) on the GPU:
reference-order results equal the oracle's composition bit for bit, and the
reference's scenarios keep their bars (DCPSE_op_test_base_tests.cpp:469-660)."""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import operators as O
from openfpm_numerics_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _grid(nside, h):
    pos, _ = W.lattice(nside, 2, h=h)
    return pos


def test_divergence(cuda, orc):
    h = 10.0 / 62
    pos = _grid(63, h)
    parts = O.ParticleSet(pos)
    vl = parts.getVerlet(3.1 * h)
    Div = O.Divergence(parts, vl, 2, 3.1 * h)
    x, y = pos[:, 0], pos[:, 1]
    v = np.stack([np.sin(x) + np.sin(y), np.cos(x) + np.cos(y)], 1)
    vt = torch.tensor(v, device="cuda")
    div = Div(vt).cpu().numpy()
    assert np.abs(div - (np.cos(x) - np.sin(y))).max() < 0.05
    rp, cols = vl.rowptr.cpu().numpy(), vl.cols.cpu().numpy()
    ref = np.zeros(len(pos))
    for i, name in enumerate(("x", "y")):
        o = orc.operator(pos, rp, cols, name)[0]
        ref = ref + orc.apply(v[:, i], rp, cols, o[3], o[2], 1)
    assert np.array_equal(div, ref)
    d32 = Div(vt, precision="f32").cpu().numpy()
    assert np.abs(d32 - ref).max() <= 1e-6 * np.abs(ref).max() * 4
    # the FP32 weight pairs: the FP64 bar
    dp = Div(vt, precision="f32-pair").cpu().numpy()
    assert np.abs(dp - ref).max() <= 1e-12 * np.abs(ref).max()
    Div.deallocate()


def test_advection(cuda, orc):
    h = 10.0 / 320
    pos = _grid(321, h)
    parts = O.ParticleSet(pos)
    vl = parts.getVerlet(3.1 * h)
    Adv = O.Advection(parts, vl, 2, 3.1 * h)
    x, y = pos[:, 0], pos[:, 1]
    P = np.sin(x) + np.sin(y)
    v = np.stack([np.sin(x) + np.sin(y), np.cos(x) + np.cos(y)], 1)
    vt = torch.tensor(v, device="cuda")
    dP = Adv(vt, torch.tensor(P, device="cuda")).cpu().numpy()
    exact = np.cos(x) * (np.sin(x) + np.sin(y)) + np.cos(y) * (np.cos(x) + np.cos(y))
    assert np.abs(dP - exact).max() < 0.03
    dv = Adv(vt, vt).cpu().numpy()
    exact_v1 = -np.sin(x) * (np.sin(x) + np.sin(y)) - np.sin(y) * (np.cos(x) + np.cos(y))
    assert np.abs(dv[:, 1] - exact_v1).max() < 0.03
    Adv.deallocate()


def test_advection_and_curl_bitexact(cuda, orc):
    pos, h = W.lattice(30, 2, jitter=0.1, seed=61)
    parts = O.ParticleSet(pos)
    vl = parts.getVerlet(3.1 * h)
    rp, cols = vl.rowptr.cpu().numpy(), vl.cols.cpu().numpy()
    dx = orc.operator(pos, rp, cols, "x")[0]
    dy = orc.operator(pos, rp, cols, "y")[0]
    f = np.sin(4 * pos[:, 0]) * np.cos(pos[:, 1])
    v = np.stack([pos[:, 1], -pos[:, 0] + 0.5], 1)
    Adv = O.Advection(parts, vl, 2, 3.1 * h)
    got = Adv(torch.tensor(v, device="cuda"), torch.tensor(f, device="cuda")).cpu().numpy()
    ref = (0.0 + v[:, 0] * orc.apply(f, rp, cols, dx[3], dx[2], 1)) + v[:, 1] * orc.apply(f, rp, cols, dy[3], dy[2], 1)
    assert np.array_equal(got, ref)
    Curl = O.Curl2D(parts, vl, 2, 3.1 * h)
    c = Curl(torch.tensor(f, device="cuda")).cpu().numpy()
    assert np.array_equal(c[0], orc.apply(f, rp, cols, dy[3], dy[2], 1))
    assert np.array_equal(c[1], -orc.apply(f, rp, cols, dx[3], dx[2], 1))
    Adv.deallocate()
    Curl.deallocate()
