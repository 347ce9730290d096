"""Seeded synthetic initial fields for the benchmark and test workloads.

No public dataset exists for this path; every workload is synthetic.  Shapes
are ``[batch, Nz, Ny, Nx]`` (x fastest, the reference's ijk order).
"""
from __future__ import annotations

import numpy as np


def _coords(nx, ny, nz, lx, ly, lz):
    z, y, x = np.meshgrid(np.arange(nz) * (lz / nz), np.arange(ny) * (ly / ny),
                          np.arange(nx) * (lx / nx), indexing="ij")
    return x, y, z


def lamellar(nx, ny, nz, lx, ly, lz, chiN, seed, batch=1, amp=0.1, noise=0.01):
    """wA/wB = +-chiN*amp*cos(2 pi x / Lx) + N(0, noise)."""
    rng = np.random.default_rng(seed)
    x, _, _ = _coords(nx, ny, nz, lx, ly, lz)
    base = chiN * amp * np.cos(2 * np.pi * x / lx)
    wa = base[None] + rng.normal(0.0, noise, (batch, nz, ny, nx))
    wb = -base[None] + rng.normal(0.0, noise, (batch, nz, ny, nx))
    return wa, wb


def gyroid(nx, ny, nz, lx, ly, lz, chiN, seed, batch=1, amp=0.2, noise=0.02):
    """chiN*amp*g(r) + N(0, noise), g = sin X cos Y + sin Y cos Z + sin Z cos X."""
    rng = np.random.default_rng(seed)
    x, y, z = _coords(nx, ny, nz, lx, ly, lz)
    X, Y, Z = 2 * np.pi * x / lx, 2 * np.pi * y / ly, 2 * np.pi * z / lz
    g = np.sin(X) * np.cos(Y) + np.sin(Y) * np.cos(Z) + np.sin(Z) * np.cos(X)
    base = chiN * amp * g
    wa = base[None] + rng.normal(0.0, noise, (batch, nz, ny, nx))
    wb = -base[None] + rng.normal(0.0, noise, (batch, nz, ny, nx))
    return wa, wb


def hexagonal(nx, ny, nz, lx, ly, lz, chiN, seed, batch=1, amp=0.2, noise=0.02):
    """A-rich cylinders along z on a hexagonal lattice in the rectangular cell
    Lx = a, Ly = a*sqrt(3) (two cylinders per cell, at (0, 0) and
    (a/2, Ly/2)): h sums the three shortest reciprocal vectors (0, 2)*2pi/L
    and (1, +-1)*2pi/L of that cell, and wA is lowest (A richest) at its
    maxima."""
    rng = np.random.default_rng(seed)
    x, y, _ = _coords(nx, ny, nz, lx, ly, lz)
    X, Y = 2 * np.pi * x / lx, 2 * np.pi * y / ly
    h = (np.cos(2 * Y) + np.cos(X + Y) + np.cos(X - Y)) / 3.0
    base = -chiN * amp * h
    wa = base[None] + rng.normal(0.0, noise, (batch, nz, ny, nx))
    wb = -base[None] + rng.normal(0.0, noise, (batch, nz, ny, nx))
    return wa, wb


def mixture(nx, ny, nz, lx, ly, lz, chiN, seed, batch=1, amp=0.1, noise=0.02, periods=1):
    """Lamellar + gyroid mixture: chiN*amp*(cos(X) + g(r)) + N(0, noise) with
    X = 2 pi periods x / Lx (likewise Y, Z): `periods` unit cells per box."""
    rng = np.random.default_rng(seed)
    x, y, z = _coords(nx, ny, nz, lx, ly, lz)
    k = 2 * np.pi * periods
    X, Y, Z = k * x / lx, k * y / ly, k * z / lz
    g = np.sin(X) * np.cos(Y) + np.sin(Y) * np.cos(Z) + np.sin(Z) * np.cos(X)
    base = chiN * amp * (np.cos(X) + g)
    wa = base[None] + rng.normal(0.0, noise, (batch, nz, ny, nx))
    wb = -base[None] + rng.normal(0.0, noise, (batch, nz, ny, nx))
    return wa, wb


def random_fields(nx, ny, nz, seed, batch=1, scale=1.0):
    rng = np.random.default_rng(seed)
    wa = rng.normal(0.0, scale, (batch, nz, ny, nx))
    wb = rng.normal(0.0, scale, (batch, nz, ny, nx))
    return wa, wb
