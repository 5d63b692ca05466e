"""Seeded synthetic workload of the benchmark and of the pressure-guess
training runs: a periodic 2*pi x 2*pi MAC grid, a unit stream u = 1 with a
divergence-free random perturbation, and 1-8 fixed disks (radii 0.02-0.08 of
the height) coupled through the direct-forcing mask.  The reference is
periodic only, so the "channel" is this periodic stream past obstacles.
"""
from __future__ import annotations

import math

import numpy as np


def make_workload(n: int = 2048, seed: int = 5):
    """Seeded initial velocity (f64 MAC faces) and disks.

    The perturbation is the discrete curl of a corner streamfunction built from
    random Fourier modes with 4 <= |k| <= 8, so it is exactly divergence-free
    on the MAC grid; the disks make every projection non-trivial."""
    rng = np.random.default_rng(seed)
    L = 2 * math.pi
    h = L / n
    x = np.arange(n) * h
    X, Y = np.meshgrid(x, x)  # corners (i h, j h), [j, i]
    psi = np.zeros((n, n))
    for _ in range(24):
        while True:
            kx, ky = rng.integers(-8, 9, size=2)
            if 4 <= math.hypot(kx, ky) <= 8:
                break
        psi += rng.normal() * np.sin(kx * X + ky * Y + rng.uniform(0, 2 * math.pi)) / (kx * kx + ky * ky)
    du = (np.roll(psi, -1, axis=0) - psi) / h    # (psi[j+1, i] - psi[j, i]) / dy
    dv = -(np.roll(psi, -1, axis=1) - psi) / h   # -(psi[j, i+1] - psi[j, i]) / dx
    scale = 0.1 / max(np.abs(du).max(), np.abs(dv).max())
    u = 1.0 + scale * du
    v = scale * dv
    ndisk = int(rng.integers(1, 9))
    disks = []
    while len(disks) < ndisk:
        r = float(rng.uniform(0.02, 0.08)) * L
        cx, cy = float(rng.uniform(0, L)), float(rng.uniform(0, L))
        if all(math.hypot(cx - d[0], cy - d[1]) > r + d[2] + 0.3 for d in disks):
            disks.append((cx, cy, r))
    umax = float(max(np.abs(u).max(), np.abs(v).max()))
    dt = 0.5 * h / umax
    return np.ascontiguousarray(u.ravel()), np.ascontiguousarray(v.ravel()), disks, dt
