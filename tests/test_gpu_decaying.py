"""Decaying turbulence with the mixed-precision projection to 1e-10
(the mixed-precision configuration of the workload table): random-phase
initial spectrum E(k) ~ k^4 exp(-(k/16)^2), unit kinetic energy, nu = 5e-5.

* 1024^2 against the oracle's f64 CPU solver (MacCormack, explicit diffusion,
  exact FFT projection) after two steps: relL2 of u, v (and of the mean-free
  pressure the step leaves) per field.  The GPU advects in f32 (like the
  reference GPU backend), so the fields agree to ~1e-6 relative.
* 4096^2: every projection reaches max|div u| <= 1e-10 and the stored
  field's divergence agrees.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg(fs):
    fs._lib.load()
    return fs


def test_1024_matches_oracle_per_field(pkg, O):
    n, nu = 1024, 5e-5
    u, v, dt = pkg.workload.decaying_turbulence(n, 3)
    s = pkg.GPUFluidSolver(n=n, nu=nu, advection="maccormack", pressure_solver="multigrid", pressure_iterations=1,
                           precision="mixed", pressure_tol=1e-10, max_cycles=80)
    s.upload_velocity(u, v)
    O.set_threads(8)
    cpu = O.CpuSolver(n=n, nu=nu, advection="maccormack", explicit_diffusion=True, projection="fft")
    cpu.u[:] = u
    cpu.v[:] = v
    for _ in range(2):
        s.step(dt)
        assert s.last_stats()["converged"]
        cpu.step(dt, advect_dye=False)
    ug, vg = s.read_velocity()
    eu, ev = O.rel_l2(ug, cpu.u), O.rel_l2(vg, cpu.v)
    assert eu < 2e-6 and ev < 2e-6, (eu, ev)
    assert s.max_divergence() <= 1.5e-10
    s.destroy()


def test_4096_reaches_1e_10(pkg):
    n = 4096
    u, v, dt = pkg.workload.decaying_turbulence(n, 4)
    s = pkg.GPUFluidSolver(n=n, nu=5e-5, advection="maccormack", pressure_solver="multigrid", pressure_iterations=1,
                           precision="mixed", pressure_tol=1e-10, max_cycles=80)
    s.upload_velocity(u, v)
    for _ in range(3):
        s.step(dt)
        st = s.last_stats()
        assert st["converged"] and st["residual_max"] <= 1e-10, st
    assert s.max_divergence() <= 1.5e-10
    d = s.diagnostics()
    assert 0.9 < d["kinetic_energy"] <= 1.0 + 1e-9
    s.destroy()
