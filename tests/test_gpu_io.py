"""Operator save / load (Dcpse::save / load byte layout) through the Python
operators on the GPU: a loaded operator applies bit for bit like the saved
one; the files hold the plan's eps, eps^-|alpha|, kernels and kernel offsets."""
import numpy as np
import pytest
import torch

from openfpm_numerics_gb300 import kernel_file
from openfpm_numerics_gb300 import operators as O
from openfpm_numerics_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["Derivative_x", "Laplacian"])
def test_save_load_round_trip(cuda, tmp_path, kind):
    pos, h = W.lattice(32, 2, jitter=0.1, seed=51)
    parts = O.ParticleSet(pos)
    vl = parts.getVerlet(3.1 * h)
    op = getattr(O, kind)(parts, vl, 2, 3.1 * h)
    f = torch.tensor(np.sin(4 * pos[:, 0]) * pos[:, 1], device="cuda")
    ref = op(f)
    base = str(tmp_path / "op")
    op.save(parts, base)
    files = [base + "_0"] if kind == "Derivative_x" else [base + "_term0_0", base + "_term1_0"]
    eps = op.plan.eps()[0].cpu().numpy()
    for t, path in enumerate(files):
        e, eip, K, off = kernel_file.read(path)
        Kp, eipp = op.plan.term_kernels(t)
        assert np.array_equal(e, eps) and np.array_equal(eip, eipp.cpu().numpy())
        assert np.array_equal(K, Kp.cpu().numpy())
        assert np.array_equal(off, vl.rowptr[:-1].cpu().numpy().astype(np.uint64))
    op2 = getattr(O, kind)(parts, vl, 2, 3.1 * h, O.support_options.LOAD)
    with pytest.raises(RuntimeError):
        op2(f)
    op2.load(parts, base)
    assert torch.equal(op2(f), ref)
    # a file of another neighbour list is refused
    vl3 = parts.getVerlet(2.9 * h)
    op3 = getattr(O, kind)(parts, vl3, 2, 2.9 * h, O.support_options.LOAD)
    with pytest.raises(ValueError):
        op3.load(parts, base)
    for o in (op, op2, op3):
        o.deallocate()
