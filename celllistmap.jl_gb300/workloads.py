"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is involved; every generator is deterministic for a given seed (numpy PCG64).
  cfg1  uniform points in an orthorhombic periodic box (Float64)
  cfg2  fcc lattice mapped through a triclinic cell, Gaussian jitter (Float32)
  cfg3  many independent uniform systems of log-uniform size at one density (Float64)
  cfg4  two-type LJ mixture on a jittered fcc lattice in a cubic box (Float32)
  cfg5  two uniform sets with Gaussian velocities in a periodic cube (Float64)
"""
from __future__ import annotations

import numpy as np


def fcc_fractional(ncell: int) -> np.ndarray:
    g = np.stack(np.meshgrid(np.arange(ncell), np.arange(ncell), np.arange(ncell), indexing="ij"), -1).reshape(-1, 3)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    return ((g[:, None, :] + basis[None, :, :]).reshape(-1, 3)) / ncell


def cfg1(n=100_000, side=100.0, seed=1):
    rng = np.random.default_rng(seed)
    return rng.random((n, 3)) * side, np.array([side, side, side])


def cfg2(ncell=64, rho=0.8, jitter=0.05, seed=2):
    """fcc (ncell^3 x 4 sites) at density rho in the cell a=(L,0,0), b=(0.2L,L,0), c=(0.1L,0.15L,L)."""
    n = 4 * ncell ** 3
    L = (n / rho) ** (1.0 / 3.0)
    M = np.array([[L, 0.2 * L, 0.1 * L], [0.0, L, 0.15 * L], [0.0, 0.0, L]])  # columns a, b, c
    rng = np.random.default_rng(seed)
    x = fcc_fractional(ncell) @ M.T + rng.normal(0.0, jitter, (n, 3))
    return x.astype(np.float32), M


def cfg3(nsys=4096, nmin=64, nmax=20_000, rho=0.1, seed=3):
    """Independent systems: sizes log-uniform in [nmin, nmax], each uniform in its own cube at density rho.
    Returns (positions concatenated, offsets[nsys+1], sides[nsys])."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), nsys)).astype(np.int64)
    sides = (sizes / rho) ** (1.0 / 3.0)
    off = np.zeros(nsys + 1, np.int64)
    off[1:] = np.cumsum(sizes)
    x = np.empty((off[-1], 3))
    for s in range(nsys):
        x[off[s]:off[s + 1]] = rng.random((sizes[s], 3)) * sides[s]
    return x, off, sides


def cfg4(n=200_000, rho=1.2, jitter=0.05, frac_a=0.8, seed=4):
    """Kob-Andersen-like 80:20 mixture on a jittered fcc lattice (m=37 cells, first n sites of a seeded
    permutation).  Returns (positions float32, side L, types int32, eps table, sigma table)."""
    m = int(np.ceil((n / 4) ** (1.0 / 3.0)))
    L = (n / rho) ** (1.0 / 3.0)
    rng = np.random.default_rng(seed)
    sites = fcc_fractional(m)[rng.permutation(4 * m ** 3)[:n]] * L
    x = sites + rng.normal(0.0, jitter, sites.shape)
    types = (rng.random(n) >= frac_a).astype(np.int32)  # 0 = A (80 %), 1 = B (20 %)
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    return x.astype(np.float32), L, types, eps, sig


def cfg5(n=2_000_000, side=250.0, vsigma=300.0, dim=3, seed=5):
    rng = np.random.default_rng(seed)
    x = rng.random((n, dim)) * side
    y = rng.random((n, dim)) * side
    vx = rng.normal(0.0, vsigma, (n, dim))
    vy = rng.normal(0.0, vsigma, (n, dim))
    return x, y, vx, vy, np.full(dim, side)


def cfg5_bins(rmin=0.1, rmax=25.0, nbins=50):
    return 10.0 ** np.linspace(np.log10(rmin), np.log10(rmax), nbins + 1)
