"""fs_autotune / fs_set_mg_sweeps: the sweep counts of the fused multigrid
step picked by timing, with the state restored afterwards."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_restores_state_and_picks_a_valid_pair(fs):
    n = 256
    u, v, disks, dt = fs.workload.make_workload(n, 7)
    s = fs.GPUFluidSolver(n=n, nu=1e-4, pressure_solver="multigrid", pressure_iterations=1, precision="mixed",
                          pressure_tol=1e-8, max_cycles=60)
    s.upload_velocity(u, v)
    s.set_solids(disks)
    s.step(dt)
    before = s.read_velocity()
    t0, k0 = s.t, s.steps
    r = s.autotune(dt, 3)
    assert 1 <= r["pre"] <= 3 and 1 <= r["post"] <= 3 and r["ms_per_step"] > 0
    after = s.read_velocity()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    assert s.t == t0 and s.steps == k0
    # the tuned solver steps on to the same tolerance
    s.step(dt)
    st = s.last_stats()
    assert st["converged"] and st["residual_max"] <= 1e-8
    s.destroy()


def test_set_mg_sweeps(fs):
    s = fs.GPUFluidSolver(n=64, pressure_solver="multigrid", pressure_iterations=1)
    s.set_mg_sweeps(3, 1)
    with pytest.raises(fs.FluidError):
        s.set_mg_sweeps(4, 2)  # the fused kernels take 1..3
    with pytest.raises(fs.FluidError):
        s.set_mg_sweeps(0, 2)
    s.destroy()
    j = fs.GPUFluidSolver(n=64, pressure_solver="jacobi", pressure_iterations=4)
    with pytest.raises(fs.FluidError):
        j.autotune(0.01)
    j.destroy()
