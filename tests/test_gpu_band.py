"""Band-limited random forcing renewed every step (fs_set_band_forcing)
against the oracle.

* The forcing stage alone, from rest, two calls in a row (the second must use
  the next step's draws): the reference's own bandForcing (24 LCG modes,
  seed + step; src/cpu/solver.js:179-217) and the Philox Gaussian lattice
  band, each against the oracle's f64 restatement; relative L2 <= 1e-6 (the
  GPU sums f32 plane-wave tables).
* Drag: (u + F) exp(-drag dt), as linearDrag after the force
  (src/cpu/solver.js:232-237, applied in that order by step, :353-358).
* The forced-turbulence configuration scaled down: 256^2 from rest, the
  Gaussian band 8 <= |k| <= 10, nu = 1e-4, drag 0.1, MacCormack, the
  mixed-precision multigrid to a relative residual of 1e-6, 20 captured
  steps, against the oracle's f64 solver (FFT projection) given the same
  draws each step: u, v relative L2 <= 1e-5, and every projection met its
  relative tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg(fs):
    fs._lib.load()
    return fs


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("kind,kf,width,amp,seed", [
    ("reference", 28.0, 2.0, 0.4, 7),
    ("gaussian", 9.0, 1.0, 3.0, (1 << 40) + 5),
])
def test_forcing_stage_matches_oracle_two_steps(pkg, O, kind, kf, width, amp, seed):
    n, dt = 128, 0.01
    s = pkg.GPUFluidSolver(n=n)
    s.upload_velocity(np.zeros(n * n), np.zeros(n * n))
    s.set_band_forcing(kind, kf=kf, width=width, amplitude=amp, seed=seed)
    g = O.grid(n)
    cu = np.zeros(n * n)
    cv = np.zeros(n * n)
    for step in range(2):
        s.run_stage("forcing", dt)
        if kind == "reference":
            O.band_forcing(g, cu, cv, kf, width, amp, (seed + step) & 0xFFFFFFFF, dt)
        else:
            O.gauss_band_forcing(g, cu, cv, kf, width, amp, seed, step, dt)
        u, v = s.read_velocity()
        assert np.abs(cu).max() > 0
        assert _rel(u, cu) <= 1e-6 and _rel(v, cv) <= 1e-6, (_rel(u, cu), _rel(v, cv))
    s.destroy()


def test_band_forcing_drag(pkg, O):
    n, dt, drag = 64, 0.02, 0.5
    a, b = O.lcg_uv(31, n * n)
    s = pkg.GPUFluidSolver(n=n)
    s.upload_velocity(a, b)
    s.set_band_forcing("gaussian", kf=6.0, width=1.5, amplitude=2.0, seed=9, drag=drag)
    s.run_stage("forcing", dt)
    u, v = s.read_velocity()
    s.destroy()
    g = O.grid(n)
    cu = np.asarray(a, dtype=np.float32).astype(np.float64)
    cv = np.asarray(b, dtype=np.float32).astype(np.float64)
    O.gauss_band_forcing(g, cu, cv, 6.0, 1.5, 2.0, 9, 0, dt)
    f = np.exp(-drag * dt)
    assert _rel(u, cu * f) <= 1e-6 and _rel(v, cv * f) <= 1e-6


def test_band_forcing_rejects_bad_arguments(pkg):
    s = pkg.GPUFluidSolver(n=64)
    with pytest.raises(pkg.FluidError):
        s.set_band_forcing("gaussian", kf=-1.0)
    with pytest.raises(pkg.FluidError):
        s.set_band_forcing("gaussian", kf=9.0, width=1.0, drag=-0.1)
    with pytest.raises(pkg.FluidError):
        s.set_band_forcing("gaussian", kf=0.2, width=0.1)  # no lattice mode in the band
    s.set_band_forcing(None)
    s.destroy()


def test_forced_turbulence_steps_match_oracle(pkg, O):
    n, nu, drag, dt, seed = 256, 1e-4, 0.1, 0.004, 2024
    s = pkg.GPUFluidSolver(n=n, nu=nu, advection="maccormack", pressure_solver="multigrid", pressure_iterations=1,
                           precision="mixed", pressure_tol=1e-6, pressure_tol_relative=True, max_cycles=60)
    s.upload_velocity(np.zeros(n * n), np.zeros(n * n))
    s.set_band_forcing("gaussian", kf=9.0, width=1.0, amplitude=3.0, seed=seed, drag=drag)
    O.set_threads(8)
    cpu = O.CpuSolver(n=n, nu=nu, advection="maccormack", explicit_diffusion=True, projection="fft")
    for k in range(20):
        s.step(dt)
        st = s.last_stats()
        assert st["converged"] and st["residual_max"] <= 1e-6 * st["residual_initial"], st
        cpu.step(dt, advect_dye=False, drag=drag, gauss_band=(9.0, 1.0, 3.0, seed, k))
    rec = s.convergence_record()
    assert rec["steps"] == 20 and rec["failed_steps"] == 0, rec
    u, v = s.read_velocity()
    s.destroy()
    assert np.abs(np.asarray(cpu.u)).max() > 1e-3
    assert _rel(u, np.asarray(cpu.u)) <= 1e-5 and _rel(v, np.asarray(cpu.v)) <= 1e-5


def test_reference_forced_turbulence_study_matches_oracle(pkg, O):
    """The reference's own forced-turbulence study configuration
    (validate/longrun-spectrum.js: 256^2 from rest, bandForcing with kf 24,
    width 1.5, amp 3 and seed 1000 + step, linear drag 0.05, nu 1e-5,
    dt 0.004, MacCormack), 20 steps on the GPU (mixed-precision multigrid to a
    relative residual of 1e-6) against the oracle's f64 solver with the
    reference's FFT projection and the same draws: u, v relative L2 <= 1e-5;
    the device spectrum's Parseval sum equals the kinetic energy."""
    n, nu, dt, drag, seed = 256, 1e-5, 0.004, 0.05, 1000
    s = pkg.GPUFluidSolver(n=n, nu=nu, advection="maccormack", pressure_solver="multigrid", pressure_iterations=1,
                           precision="mixed", pressure_tol=1e-6, pressure_tol_relative=True, max_cycles=60)
    s.upload_velocity(np.zeros(n * n), np.zeros(n * n))
    s.set_band_forcing("reference", kf=24.0, width=1.5, amplitude=3.0, seed=seed, drag=drag)
    O.set_threads(8)
    cpu = O.CpuSolver(n=n, nu=nu, advection="maccormack", explicit_diffusion=True, projection="fft")
    for k in range(20):
        s.step(dt)
        cpu.step(dt, advect_dye=False, drag=drag, band=(24.0, 1.5, 3.0, seed + k))
    rec = s.convergence_record()
    assert rec["steps"] == 20 and rec["failed_steps"] == 0, rec
    u, v = s.read_velocity()
    _, E, _, (esum, ke) = s.energy_spectrum()
    s.destroy()
    assert _rel(u, np.asarray(cpu.u)) <= 1e-5 and _rel(v, np.asarray(cpu.v)) <= 1e-5
    assert abs(esum - ke) <= 1e-6 * ke
