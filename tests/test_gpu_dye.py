"""Dye (fs_upload_dye / fs_read_dye, ADVECT_SCALAR of src/gpu/shaders.js:234-266):
advected after the projection through the new velocity, faded, clamped.

Parity: each channel of one step against the oracle's f64 semi-Lagrangian
scalar advection (src/cpu/advect.js) through the velocity the step produced,
relL2 <= 1e-5 (f32 traces); fade and clamp exactly.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg(fs):
    fs._lib.load()
    return fs


def _dye(n, seed):
    rng = np.random.default_rng(seed)
    x = np.arange(n) / n * 2 * np.pi
    X, Y = np.meshgrid(x, x)
    d = np.empty((n, n, 4), np.float32)
    for c in range(4):
        kx, ky = rng.integers(1, 4, size=2)
        d[..., c] = 0.5 + 0.4 * np.sin(kx * X + rng.uniform(0, 6)) * np.cos(ky * Y + rng.uniform(0, 6))
    return d


@pytest.mark.parametrize("solver", ["multigrid", "jacobi"])
def test_dye_matches_oracle_advection(pkg, O, solver):
    n = 64
    g = O.grid(n)
    u, v = O.tg_init(g)
    dye = _dye(n, 1)
    # fixed iteration counts: the dye is compared through whatever velocity the step produced
    kw = dict(pressure_solver=solver, pressure_iterations=2 if solver == "multigrid" else 40)
    s = pkg.GPUFluidSolver(n=n, precision="mixed", **kw)
    s.upload_velocity(u, v)
    s.upload_dye(dye)
    dt = 0.02
    s.step(dt)
    un, vn = s.read_velocity()
    got = s.read_dye()
    for c in range(4):
        ref = O.advect_scalar(g, un, vn, dye[..., c].astype(np.float64).ravel(), dt, "semi-lagrangian")
        assert O.rel_l2(got[..., c].ravel(), ref) <= 1e-5, c
    s.destroy()


def test_dye_fade_and_clamp(pkg):
    n = 32
    s = pkg.GPUFluidSolver(n=n, pressure_solver="multigrid", pressure_iterations=1, dye_fade=0.1)
    s.upload_velocity(np.zeros(n * n), np.zeros(n * n))
    d = np.full((n, n, 4), 0.5, np.float32)
    d[..., 3] = 2.0
    s.upload_dye(d)
    s.step(0.01)
    out = s.read_dye()
    np.testing.assert_allclose(out[..., :3], 0.45, rtol=1e-6)
    np.testing.assert_allclose(out[..., 3], 1.0, rtol=0)  # 2.0 * 0.9 clamped to 1
    s.step(0.01)
    np.testing.assert_allclose(s.read_dye()[..., 3], 0.9, rtol=1e-6)
    s.destroy()


def test_dye_rejections(pkg):
    s = pkg.GPUFluidSolver(n=32, pressure_solver="multigrid", pressure_iterations=1)
    with pytest.raises(pkg.FluidError):
        s.read_dye()
    with pytest.raises(ValueError):
        s.upload_dye(np.zeros(10, np.float32))
    s.destroy()
    with pytest.raises(pkg.FluidError):
        pkg.GPUFluidSolver(n=32, dye_fade=1.5)
