"""Device diagnostics (fs_diagnose, fs_energy_spectrum) against the oracle's
restatement of the reference's CPU diagnostics (src/core/grid.js:280-327,
src/core/fft.js:196-254).

Per-cell values are f32 on the device and sums are double, so the scalars
match to ~1e-6 relative; the spectrum uses an f32 FFT, compared on shells
holding at least 1e-8 of the peak to 1e-4 relative, mode counts exactly.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module")
def pkg(fs):
    fs._lib.load()
    return fs


@pytest.mark.parametrize("precision", ["f32", "mixed"])
def test_scalars_match_oracle(pkg, O, precision):
    n = 64
    g = O.grid(n)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(n * n)
    v = rng.standard_normal(n * n)
    s = pkg.GPUFluidSolver(n=n, precision=precision, pressure_solver="multigrid", pressure_iterations=1)
    s.upload_velocity(u, v)
    if precision == "f32":
        u, v = u.astype(np.float32).astype(np.float64), v.astype(np.float32).astype(np.float64)
    d = s.diagnostics()
    assert _rel(d["kinetic_energy"], O.kinetic_energy(g, u, v)) < 1e-6
    assert _rel(d["enstrophy"], O.enstrophy(g, u, v)) < 1e-5
    div = O.divergence(g, u, v)
    assert _rel(d["max_divergence"], np.abs(div).max()) < 1e-5
    assert _rel(d["l2_divergence"], math.sqrt(np.mean(div * div))) < 1e-5
    s.destroy()


def test_taylor_green_invariants(pkg, O):
    """Taylor-Green u = sin x cos y, v = -cos x sin y: KE 1/4, enstrophy 1/2
    (src/core/analytic.js:58-61) up to the grid's O(h^2) averaging."""
    n = 128
    g = O.grid(n)
    u, v = O.tg_init(g)
    s = pkg.GPUFluidSolver(n=n, precision="mixed", pressure_solver="multigrid", pressure_iterations=1)
    s.upload_velocity(u, v)
    d = s.diagnostics()
    assert _rel(d["kinetic_energy"], O.kinetic_energy(g, u, v)) < 1e-6
    assert _rel(d["enstrophy"], O.enstrophy(g, u, v)) < 1e-6
    assert abs(d["kinetic_energy"] - 0.25) < 1e-3 and abs(d["enstrophy"] - 0.5) < 2e-3
    # per-cell f32 evaluation: the exactly divergence-free field reads at f32
    # rounding (fs_max_divergence is the double-float-exact measure)
    assert d["max_divergence"] < 1e-6
    assert s.max_divergence() < 1e-12
    s.destroy()


@pytest.mark.parametrize("n", [64, 256])
def test_energy_spectrum_matches_oracle(pkg, O, n):
    g = O.grid(n)
    u, v, _ = pkg.workload.vortex_blobs(n, 9)
    s = pkg.GPUFluidSolver(n=n, precision="mixed", pressure_solver="multigrid", pressure_iterations=1)
    s.upload_velocity(u, v)
    k, E, cnt, (tot, ke) = s.energy_spectrum()
    cu, cv = O.velocity_at_centers(g, u, v)
    E_ref, cnt_ref = O.energy_spectrum(cu, cv, n, n)[:2]
    assert np.array_equal(cnt, cnt_ref)
    big = E_ref > 1e-8 * E_ref.max()
    np.testing.assert_allclose(E[big], E_ref[big], rtol=1e-4)
    assert _rel(ke, O.kinetic_energy(g, u, v)) < 1e-6
    assert _rel(tot, E_ref.sum()) < 1e-5
    s.destroy()


def test_spectrum_rejects_unsupported_grids(pkg):
    s = pkg.GPUFluidSolver(n=96, pressure_solver="multigrid", pressure_iterations=1)
    with pytest.raises(pkg.FluidError):
        s.energy_spectrum()
    s.destroy()
