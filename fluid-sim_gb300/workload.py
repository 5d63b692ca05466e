"""Seeded synthetic workloads on a periodic 2*pi x 2*pi MAC grid.

* channel_workload: the benchmark's and the pressure-guess training runs'
  channel flow -- uniform inflow u = 1 through a fringe strip, no-slip walls
  (an immersed slab), 1-8 fixed disks of radius 0.02-0.08 of the channel
  height, a divergence-free random perturbation;
* make_workload: the periodic stream past disks (no walls, no fringe);
* vortex_blobs, decaying_turbulence, batch_sides: the batched and the
  mixed-precision configurations.
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


def channel_geometry(L: float = 2 * math.pi) -> dict:
    """The channel of the learned-guess workload on the periodic [0, L)^2
    grid: a no-slip wall slab of thickness L/16 centred on y = 0 (its edges
    y = L/32 and y = L - L/32 are the two walls, height H = 15 L / 16), and an
    inflow fringe of width L/12 centred at x = 11 L / 12 with a ramp of L/256
    (its core sets u = 1 to within 1e-9), which turns the outflow back into
    the uniform inflow u = 1."""
    return {"wall_y": 0.0, "wall_half": L / 32, "fringe_x": L * 11 / 12, "fringe_half": L / 24,
            "fringe_ramp": L / 256, "inflow_u": 1.0}


def channel_workload(n: int = 2048, seed: int = 5):
    """Seeded channel flow past immersed disks (the learned-guess workload:
    inflow u = 1, 1-8 fixed disks of radius 0.02-0.08 of the channel height,
    no-slip walls).  Returns (u, v, disks, dt, channel): the initial velocity
    is the uniform inflow with the divergence-free perturbation of
    make_workload (amplitude 0.1) inside the channel and zero in the walls;
    the disks sit between the fringe's exit and its entry, clear of the
    walls and of each other; dt is CFL 0.5 of the initial field."""
    rng = np.random.default_rng(seed)
    L = 2 * math.pi
    h = L / n
    ch = channel_geometry(L)
    x = np.arange(n) * h
    X, Y = np.meshgrid(x, x)  # corners (i h, j h), [j, i]
    psi = np.zeros((n, n))
    for _ in range(24):
        while True:
            kx, ky = rng.integers(-8, 9, size=2)
            if 4 <= math.hypot(kx, ky) <= 8:
                break
        psi += rng.normal() * np.sin(kx * X + ky * Y + rng.uniform(0, 2 * math.pi)) / (kx * kx + ky * ky)
    du = (np.roll(psi, -1, axis=0) - psi) / h
    dv = -(np.roll(psi, -1, axis=1) - psi) / h
    scale = 0.1 / max(np.abs(du).max(), np.abs(dv).max())
    yu = (np.arange(n) + 0.5) * h  # u faces at (i h, (j + 1/2) h)
    fluid = np.abs((yu + L / 2) % L - L / 2) > ch["wall_half"]
    u = (1.0 + scale * du) * fluid[:, None]
    v = scale * dv
    H = L - 2 * ch["wall_half"]
    x_lo, x_hi = ch["fringe_x"] + ch["fringe_half"] - L + 0.1 * L, ch["fringe_x"] - ch["fringe_half"] - 0.1 * L
    ndisk = int(rng.integers(1, 9))
    disks = []
    while len(disks) < ndisk:
        r = float(rng.uniform(0.02, 0.08)) * H
        cx = float(rng.uniform(max(x_lo, 0.0) + r, x_hi - r))
        cy = float(rng.uniform(ch["wall_half"] + r + 0.05 * H, L - ch["wall_half"] - r - 0.05 * H))
        if all(math.hypot(cx - d[0], cy - d[1]) > r + d[2] + 0.1 * H for d in disks):
            disks.append((cx, cy, r))
    umax = float(max(np.abs(u).max(), np.abs(v).max()))
    dt = 0.5 * h / umax
    return np.ascontiguousarray(u.ravel()), np.ascontiguousarray(v.ravel()), disks, dt, ch


def vortex_blobs(n: int, seed: int, L: float = 2 * math.pi):
    """Seeded decaying-vortex initial state: 4-16 Gaussian blobs of radius
    0.05-0.15 L with circulation ~ N(0, 1), periodic images included; the
    streamfunction comes from the spectral inversion of the vorticity at the
    cell corners and the MAC velocity from its differences, so the field is
    exactly divergence-free on the grid.  Returns (u, v, dt) with dt at CFL 0.5."""
    rng = np.random.default_rng(seed)
    h = L / n
    x = np.arange(n) * h
    X, Y = np.meshgrid(x, x)  # corners (i h, j h), [j, i]
    w = np.zeros((n, n))
    for _ in range(int(rng.integers(4, 17))):
        r = float(rng.uniform(0.05, 0.15)) * L
        cx, cy = rng.uniform(0, L, size=2)
        gam = float(rng.normal())
        dx = X - cx
        dy = Y - cy
        dx -= L * np.round(dx / L)
        dy -= L * np.round(dy / L)
        w += gam / (2 * math.pi * r * r) * np.exp(-(dx * dx + dy * dy) / (2 * r * r))
    w -= w.mean()
    k = np.fft.fftfreq(n, d=h) * 2 * math.pi
    KX, KY = np.meshgrid(k, k)
    k2 = KX * KX + KY * KY
    k2[0, 0] = 1.0
    psi_hat = np.fft.fft2(w) / k2
    psi_hat[0, 0] = 0.0
    psi = np.real(np.fft.ifft2(psi_hat))
    u = (np.roll(psi, -1, axis=0) - psi) / h   # (psi[j+1, i] - psi[j, i]) / dy on the left face
    v = -(np.roll(psi, -1, axis=1) - psi) / h  # -(psi[j, i+1] - psi[j, i]) / dx on the bottom face
    umax = float(max(np.abs(u).max(), np.abs(v).max(), 1e-12))
    return np.ascontiguousarray(u.ravel()), np.ascontiguousarray(v.ravel()), 0.5 * h / umax


BATCH_SIDES = (64, 128, 192, 256, 384, 512)


def batch_sides(count: int, seed: int):
    """Domain sides of a seeded batch of uneven simulations."""
    rng = np.random.default_rng(seed)
    return [int(rng.choice(BATCH_SIDES)) for _ in range(count)]


def decaying_turbulence(n: int, seed: int, L: float = 2 * math.pi, k0: float = 16.0):
    """Seeded decaying-turbulence state: random-phase streamfunction whose
    shell spectrum is E(k) ~ k^4 exp(-(k/k0)^2) (|psi_k|^2 ~ k exp(-(k/k0)^2)
    since E ~ k^3 |psi_k|^2 in 2-D), sampled at the cell corners so the MAC
    velocity from its differences is exactly divergence-free, normalised to
    kinetic energy 1/2 <u^2 + v^2> = 1.  Returns (u, v, dt) with dt at CFL 0.5."""
    rng = np.random.default_rng(seed)
    h = L / n
    kk = np.fft.fftfreq(n, d=1.0 / n)
    KX, KY = np.meshgrid(kk, kk)
    k = np.hypot(KX, KY)
    amp = np.sqrt(k * np.exp(-(k / k0) ** 2))
    amp[0, 0] = 0.0
    psi_hat = amp * np.exp(2j * math.pi * rng.random((n, n)))
    psi = np.real(np.fft.ifft2(psi_hat)) * n * n
    u = (np.roll(psi, -1, axis=0) - psi) / h
    v = -(np.roll(psi, -1, axis=1) - psi) / h
    ke = 0.5 * np.mean(u * u + v * v)
    s = 1.0 / math.sqrt(ke)
    u *= s
    v *= s
    umax = float(max(np.abs(u).max(), np.abs(v).max()))
    return np.ascontiguousarray(u.ravel()), np.ascontiguousarray(v.ravel()), 0.5 * h / umax
