"""The weight-pair apply's difference split (fixed_pair in
openfpm_numerics_gb300/csrc/dcpse_f32_row.cuh) restated with numpy float32
operations, against exact rational arithmetic: for |d| < 2^63 the three
pieces x + y + z equal d 2^-64 exactly, and the float pair dh + dl is within
2^-47 |d| 2^-64 of it; zero gives an exact zero.  The kernel's results are
checked against the oracle on the GPU (tests/test_gpu_pair.py)."""
from fractions import Fraction

import numpy as np

f32 = np.float32


def _bits(u):
    return np.asarray(u, dtype=np.uint32).view(f32)


def fixed_pair(d):
    """The device function's operations, elementwise on int64 d."""
    a = d >> 42
    b = (d >> 21) & 0x1FFFFF
    c = d & 0x1FFFFF
    x = _bits((0x40400000 + a).astype(np.uint32)) - f32(3.0)
    y = _bits((0x35800000 | b).astype(np.uint32)) - f32(2.0 ** -20)
    z = _bits((0x2B000000 | c).astype(np.uint32)) - f32(2.0 ** -41)
    s = x + y
    t = (y - (s - x)) + z
    dh = s + t
    dl = t - (dh - s)
    return x, y, z, dh, dl, a, b, c


def test_pieces_exact_and_pair_bound():
    rng = np.random.default_rng(7)
    ds = [np.array([0, 1, -1, (1 << 42) - 1, -(1 << 42), (1 << 63) - 1, -(1 << 63) + 1], dtype=np.int64)]
    for lim in (2 ** 21, 2 ** 42, 2 ** 45, 2 ** 53, 2 ** 62, 2 ** 63 - 1):
        ds.append(rng.integers(-lim, lim, size=3000, dtype=np.int64))
    d = np.concatenate(ds)
    x, y, z, dh, dl, a, b, c = fixed_pair(d)
    assert np.all((a >= -(1 << 21)) & (a < (1 << 21)))
    # the three pieces are exact (scaled by 2^-64)
    assert np.array_equal(x.astype(np.float64), a * 2.0 ** -22)
    assert np.array_equal(y.astype(np.float64), b * 2.0 ** -43)
    assert np.array_equal(z.astype(np.float64), c * 2.0 ** -64)
    worst = Fraction(0)
    for i in range(0, d.size, 7):
        exact = Fraction(int(d[i]), 1 << 64)
        got = Fraction(float(dh[i])) + Fraction(float(dl[i]))
        if d[i] == 0:
            assert got == 0
        else:
            worst = max(worst, abs(got - exact) / abs(exact))
    assert worst <= Fraction(1, 1 << 47), float(worst)
