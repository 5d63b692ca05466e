"""fs_render: the reference's RENDER arithmetic (src/gpu/shaders.js:677-768)
into a buffer, checked against a float64 numpy restatement of the same
formulas on the read-back state (tolerance 1e-4 absolute on colours of order 1:
the device evaluates in f32)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAGENTA = np.array([1.00, 0.10, 0.62]); CYAN = np.array([0.10, 0.92, 1.00])
VIOLET = np.array([0.16, 0.03, 0.42]); VOID = np.array([0.004, 0.003, 0.016])


def smooth(e0, e1, x):
    t = np.clip((x - e0) / (e1 - e0), 0, 1)
    return t * t * (3 - 2 * t)


def mix(a, b, t):
    return a * (1 - t[..., None]) + b * t[..., None]


def render_ref(u, v, dye, dx, dy, exposure, mode):
    curl = (v - np.roll(v, 1, axis=1)) / dx - (u - np.roll(u, 1, axis=0)) / dy  # corner (i, j)
    w = 0.25 * (curl + np.roll(curl, -1, axis=1) + np.roll(curl, -1, axis=0) + np.roll(np.roll(curl, -1, 0), -1, 1))
    speed = np.hypot(u, v)
    if mode == 0:
        sig = np.tanh(np.clip(w * exposure, -12, 12))
        mag = np.abs(sig)
        hue = np.where((sig >= 0)[..., None], MAGENTA, CYAN)
        ramp = mix(mix(np.broadcast_to(VOID, hue.shape), np.broadcast_to(VIOLET, hue.shape), smooth(0, 0.22, mag)),
                   hue, smooth(0.12, 0.62, mag))
        col = ramp * (0.30 + 4.6 * mag * mag)[..., None]
    else:
        t = np.tanh(np.clip(speed * exposure, -12, 12))
        hue = mix(np.broadcast_to(VIOLET, t.shape + (3,)), np.broadcast_to(CYAN, t.shape + (3,)), smooth(0.15, 0.95, t))
        col = mix(np.broadcast_to(VOID, hue.shape), hue, smooth(0, 0.6, t)) * (0.35 + 2.9 * t * t)[..., None]
    sp = np.tanh(np.clip(speed * exposure * 0.45, 0, 12))
    col = col + np.array([0.55, 0.78, 1.0]) * (sp ** 5 * 0.85)[..., None]
    if dye is not None:
        lum = dye[..., 0] * 0.2126 + dye[..., 1] * 0.7152 + dye[..., 2] * 0.0722
        col = col + col * (lum * 1.5)[..., None] + dye[..., :3] * 0.20
    return col


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("with_dye", [False, True])
def test_render_matches_formula(fs, O, mode, with_dye):
    n = 64
    g = O.grid(n)
    u, v = O.tg_init(g)
    s = fs.GPUFluidSolver(n=n, precision="mixed", pressure_solver="multigrid", pressure_iterations=1)
    s.upload_velocity(u, v)
    dye = None
    if with_dye:
        rng = np.random.default_rng(2)
        dye = rng.random((n, n, 4)).astype(np.float32)
        s.upload_dye(dye)
    out = s.render("vorticity" if mode == 0 else "speed", exposure=0.7)
    ref = render_ref(u.reshape(n, n), v.reshape(n, n), None if dye is None else dye.astype(np.float64),
                     s.dx, s.dy, 0.7, mode)
    np.testing.assert_allclose(out[..., :3], ref, atol=1e-4)
    assert np.all(out[..., 3] == 1.0)
    s.destroy()


def test_render_ppm(fs, O, tmp_path):
    n = 32
    g = O.grid(n)
    u, v = O.tg_init(g)
    s = fs.GPUFluidSolver(n=n, pressure_solver="multigrid", pressure_iterations=1)
    s.upload_velocity(u, v)
    path = tmp_path / "w.ppm"
    s.save_ppm(path, s.render())
    b = path.read_bytes()
    assert b.startswith(b"P6 32 32 255\n") and len(b) == len(b"P6 32 32 255\n") + 32 * 32 * 3
    s.destroy()
