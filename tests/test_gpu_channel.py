"""The channel (inflow fringe + no-slip wall slab, fs_set_channel) against
the oracle's f64 restatement of the same forcing.

* the forcing alone on a random field (the solid stage with only the
  channel set), relative L2 <= 1e-6;
* its effect: after the stage the wall slab holds u = v = 0 and the fringe
  core holds (inflow_u, 0);
* the channel workload at 256^2 (uniform inflow, walls, seeded disks),
  mixed-precision multigrid to 1e-6 with relaxation 1.2, 10 captured steps
  against the oracle's f64 solver with the same channel and disks (FFT
  projection): u, v relative L2 <= 1e-5, every projection converged.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg(fs):
    fs._lib.load()
    return fs


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_channel_forcing_matches_oracle(pkg, O):
    n = 512
    ch = pkg.workload.channel_geometry()
    a, b = O.lcg_uv(77, n * n)
    s = pkg.GPUFluidSolver(n=n)
    s.upload_velocity(a, b)
    s.set_channel(ch)
    s.run_stage("solid", 0.01)
    u, v = s.read_velocity()
    s.destroy()
    g = O.grid(n)
    cu = np.asarray(a, np.float32).astype(np.float64)
    cv = np.asarray(b, np.float32).astype(np.float64)
    O.channel_forcing(g, cu, cv, ch, 1.5)
    assert _rel(u, cu) <= 1e-6 and _rel(v, cv) <= 1e-6, (_rel(u, cu), _rel(v, cv))
    # walls at rest, fringe core at the inflow velocity
    h = 2 * math.pi / n
    U = u.reshape(n, n)
    V = v.reshape(n, n)
    yu = (np.arange(n) + 0.5) * h
    dist = np.abs((yu + math.pi) % (2 * math.pi) - math.pi)  # of the u faces from the slab centre
    wall_rows = dist < ch["wall_half"] - 7.5 * 1.5 * h
    fluid_rows = dist > ch["wall_half"] + 8.5 * 1.5 * h + h
    assert wall_rows.sum() >= 4
    assert np.abs(U[wall_rows]).max() < 1e-5
    core = np.abs(np.arange(n) * h - ch["fringe_x"]) < ch["fringe_half"] - 7.5 * ch["fringe_ramp"]
    assert core.sum() >= 4
    assert np.abs(U[fluid_rows][:, core] - 1.0).max() < 1e-5
    assert np.abs(V[fluid_rows][:, core]).max() < 1e-5


def test_channel_steps_match_oracle(pkg, O):
    n, steps, nu = 256, 10, 1e-4
    u0, v0, disks, dt, ch = pkg.workload.channel_workload(n, 11)
    s = pkg.GPUFluidSolver(n=n, nu=nu, advection="maccormack", pressure_solver="multigrid", pressure_iterations=1,
                           precision="mixed", pressure_tol=1e-6, max_cycles=60, relax=1.2)
    s.upload_velocity(u0, v0)
    s.set_channel(ch)
    s.set_solids(disks)
    for _ in range(steps):
        s.step(dt)
    rec = s.convergence_record()
    u, v = s.read_velocity()
    s.destroy()
    assert rec["steps"] == steps and rec["failed_steps"] == 0, rec
    O.set_threads(8)
    cpu = O.CpuSolver(n=n, nu=nu, advection="maccormack", explicit_diffusion=True, projection="fft",
                      coupling_passes=1)
    cpu.u[:] = u0
    cpu.v[:] = v0
    cpu.set_channel(ch)
    for d in disks:
        cpu.add_solid(O.disk(d[0], d[1], d[2], density=8, fixed=True))
    for _ in range(steps):
        cpu.step(dt, advect_dye=False)
    assert _rel(u, np.asarray(cpu.u)) <= 1e-5 and _rel(v, np.asarray(cpu.v)) <= 1e-5, (
        _rel(u, np.asarray(cpu.u)), _rel(v, np.asarray(cpu.v)))
