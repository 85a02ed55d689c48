"""Seeded synthetic particle sets and analytic fields for the DC-PSE configs.

No public dataset is involved: the reference's own tests and the benchmark
configurations use lattices with seeded jitter, which these functions
generate (numpy PCG64 streams; seeds fixed per configuration).
"""
from __future__ import annotations

import math

import numpy as np


def lattice(nside, dim, h=None, jitter=0.0, seed=0, origin=0.0):
    """Lattice of nside^dim points with spacing h (default 1/(nside-1)),
    index = i0 + nside*(i1 + nside*i2) (x fastest), each coordinate jittered
    by U(-jitter*h, +jitter*h)."""
    if h is None:
        h = 1.0 / (nside - 1)
    ax = origin + np.arange(nside, dtype=np.float64) * h
    grids = np.meshgrid(*([ax] * dim), indexing="ij")
    # flattened in C order the last grid axis varies fastest: use it for x
    pos = np.stack([grids[dim - 1 - d].reshape(-1) for d in range(dim)], axis=1)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        pos = pos + rng.uniform(-jitter * h, jitter * h, size=pos.shape)
    return np.ascontiguousarray(pos), h


def interior_mask(pos, margin, lo=0.0, hi=1.0):
    return np.all((pos > lo + margin) & (pos < hi - margin), axis=1)


# -- configuration 1: 2D Laplacian, 64x64, jitter 0.1h, rCut = 3.1h ------------
def config1():
    pos, h = lattice(64, 2, jitter=0.1, seed=1)
    return dict(pos=pos, h=h, rcut=3.1 * h, order=2, dim=2)


def field1(pos):
    x, y = pos[:, 0], pos[:, 1]
    f = np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)
    return f, -8 * np.pi ** 2 * f


# -- configuration 2: 3D Gradient + Laplacian, 128^3, jitter 0.15h, rCut 2.8h --
def config2(nside=128):
    h = 1.0 / 127.0
    pos, _ = lattice(nside, 3, h=h, jitter=0.15, seed=2)
    return dict(pos=pos, h=h, rcut=2.8 * h, order=2, dim=3)


def field2(pos):
    """f = exp(-10|x-0.5|^2) sin(3 pi x_1) (x_1 = first coordinate) with its
    analytic gradient (3 components) and Laplacian."""
    c = pos - 0.5
    r2 = np.sum(c * c, axis=1)
    g = np.exp(-10.0 * r2)
    k = 3.0 * np.pi
    s = np.sin(k * pos[:, 0])
    cs = np.cos(k * pos[:, 0])
    f = g * s
    grad = np.empty_like(pos)
    for d in range(3):
        grad[:, d] = -20.0 * c[:, d] * g * s
    grad[:, 0] += g * k * cs
    lap_g = g * (400.0 * r2 - 60.0)
    lap = s * lap_g + 2.0 * (-20.0 * c[:, 0] * g) * (k * cs) - g * k * k * s
    return f, grad, lap


# -- configuration 3: graded 2D cloud, density growing 4x along x ---------------
def config3(n=1_000_000, seed=3):
    """x from inverse-CDF sampling of a density rho(x) = 1 + 3x on [0,1]
    (4x from x=0 to x=1), y uniform; local spacing h = rho_n^(-1/2) with
    rho_n = n rho(x) / 2.5, rCut_p = 3.1 h_p."""
    rng = np.random.default_rng(seed)
    u = rng.random(n)
    # CDF(x) = (x + 1.5 x^2) / 2.5  ->  1.5 x^2 + x - 2.5 u = 0
    x = (-1.0 + np.sqrt(1.0 + 15.0 * u)) / 3.0
    y = rng.random(n)
    pos = np.ascontiguousarray(np.stack([x, y], axis=1))
    dens = n * (1.0 + 3.0 * x) / 2.5
    h = 1.0 / np.sqrt(dens)
    return dict(pos=pos, h=h, rcut_pp=3.1 * h, order=2, dim=2)


# -- configuration 4: adjoint check, 256^2, jitter 0.1h, Laplacian ----------------
def config4(nside=256):
    pos, h = lattice(nside, 2, jitter=0.1, seed=4)
    rng = np.random.default_rng(4)
    f = rng.standard_normal(pos.shape[0])
    g = rng.standard_normal(pos.shape[0])
    return dict(pos=pos, h=h, rcut=3.1 * h, order=2, dim=2, f=f, g=g)


# -- configuration 5: periodic 3D Gray-Scott --------------------------------------
def config5(nside=96):
    h = 1.0 / nside
    pos, _ = lattice(nside, 3, h=h, jitter=0.1, seed=6)
    pos = np.mod(pos, 1.0)
    return dict(pos=pos, h=h, rcut=2.8 * h, order=2, dim=3, box=((0.0,) * 3, (1.0,) * 3, (1, 1, 1)))


def gray_scott_initial(pos, nspheres=20, radius=0.05, seed=6):
    rng = np.random.default_rng(seed)
    centers = rng.random((nspheres, 3))
    u = np.ones(pos.shape[0])
    v = np.zeros(pos.shape[0])
    for c in centers:
        d = pos - c
        d -= np.round(d)  # periodic minimum image
        inside = np.sum(d * d, axis=1) < radius * radius
        u[inside] = 0.5
        v[inside] = 0.25
    return u, v


def grad_lap_outputs(dim):
    """Outputs of a Gradient + Laplacian plan: dim single-term outputs, then
    the Laplacian as the sum of the dim terms 2e_i."""
    outs = [[tuple(1 if d == i else 0 for d in range(dim))] for i in range(dim)]
    outs.append([tuple(2 if d == i else 0 for d in range(dim)) for i in range(dim)])
    return outs


def five_ops_2d():
    """Dx, Dy, Dxx, Dyy, Dxy."""
    return [[(1, 0)], [(0, 1)], [(2, 0)], [(0, 2)], [(1, 1)]]


def apply_bytes(n, nnz, nout, wbytes, fbytes=8, obytes=8):
    """Algorithmic bytes of one batched apply: row offsets (8 B), column
    index (4 B) and nout weights per entry, each f read once, nout outputs."""
    return n * 8 + nnz * (4 + nout * wbytes) + n * fbytes + nout * n * obytes


def assembly_flops(n_particles, kbar, groups):
    """FP64 flops per assembly: for each basis (n functions, R right-hand
    sides): Gram k n (n+1) (symmetric), QR (4/3) n^3, solves 2 n^2 R and
    weight evaluation 2 k n R.  groups = [(n, R), ...].  Gram entries shared
    between bases are counted once per basis (upper bound)."""
    f = 0.0
    for n, R in groups:
        f += kbar * n * (n + 1) + (4.0 / 3.0) * n ** 3 + 2.0 * n * n * R + 2.0 * kbar * n * R
    return n_particles * f
