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


def _mixed(fs, n, **kw):
    return fs.GPUFluidSolver(n=n, nu=1e-3, advection="maccormack", pressure_solver="multigrid",
                             pressure_iterations=1, precision="mixed", pressure_tol=1e-8, max_cycles=60, **kw)


def test_tile_sides_do_not_change_results(fs, O):
    """The fused tiles give the same values whatever their size: three steps at
    1024^2 with every tile level at 16, 32 or 64 cells, or mixed, equal the
    built-in choice bit for bit (fields and cycle counts)."""
    n = 1024
    u0, v0 = O.lcg_uv(73, n * n)
    out = []
    for tiles in (None, [16, 16, 16, 16], [64, 64, 64, 64], [32, 64, 16, 32]):
        s = _mixed(fs, n)
        if tiles is not None:
            s.set_mg_tiles(tiles)
            assert s.mg_tiles() == tiles
        s.upload_velocity(u0, v0)
        cyc = []
        for _ in range(3):
            s.step(0.002)
            cyc.append(s.last_stats()["cycles"])
        u, v = s.read_velocity()
        out.append((u, v, s.read_field("pressure"), cyc))
        s.destroy()
    for o in out[1:]:
        assert all(np.array_equal(a, b) for a, b in zip(o[:3], out[0][:3])) and o[3] == out[0][3]


def test_autotune_tiles_restores_state(fs, O):
    n = 512
    u0, v0 = O.lcg_uv(74, n * n)
    s = _mixed(fs, n)
    s.upload_velocity(u0, v0)
    s.step(0.002)
    before = s.read_velocity()
    t0, k0 = s.t, s.steps
    r = s.autotune_tiles(0.002, 2)
    assert len(r["tiles"]) == 3 and all(t in (16, 32, 64) for t in r["tiles"]) and r["ms_per_step"] > 0
    after = s.read_velocity()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    assert s.t == t0 and s.steps == k0
    # the tuned solver steps on exactly like one that was never tuned
    ref = _mixed(fs, n)
    ref.upload_velocity(u0, v0)
    ref.step(0.002)
    ref.step(0.002)
    s.step(0.002)
    assert np.array_equal(s.read_velocity()[0], ref.read_velocity()[0])
    with pytest.raises(fs.FluidError):
        s.set_mg_tiles([48])
    s.destroy()
    ref.destroy()


def test_tile_side_larger_than_half_a_level_falls_back(fs, O):
    """A tile side serves a level only if it is at most half the level: at
    132^2 (tile levels 132 and 66) a 64-cell override on level 1 gives way to
    the built-in 16, and the step equals the built-in choice bit for bit."""
    n = 132
    u0, v0 = O.lcg_uv(75, n * n)
    out = []
    for tiles in (None, [64, 64]):
        s = _mixed(fs, n)
        if tiles is not None:
            s.set_mg_tiles(tiles)
            assert s.mg_tiles() == [64, 16]
        s.upload_velocity(u0, v0)
        for _ in range(2):
            s.step(0.002)
        out.append(s.read_velocity())
        s.destroy()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_batch_class_of_small_levels_keeps_tiles_within_half(fs, O):
    """The class rule counts the tiles of all members (64 members of 132^2
    would ask for 64-cell tiles on the 66-cell level); the side stays within
    half the level and every member equals a solver stepped alone."""
    fs._lib.load()
    n, count = 132, 64
    cfg = dict(nu=1e-3, advection="maccormack", pressure_solver="multigrid", pressure_iterations=1,
               precision="mixed", pressure_tol=1e-8, max_cycles=60)
    b = fs.GPUFluidBatch([dict(n=n, **cfg) for _ in range(count)])
    states = [O.lcg_uv(200 + i, n * n) for i in range(count)]
    for m, (u, v) in zip(b.members, states):
        m.upload_velocity(u, v)
    for _ in range(2):
        b.step([0.002] * count)
    b.sync()
    for i in (0, count - 1):
        s = _mixed(fs, n)
        s.upload_velocity(*states[i])
        for _ in range(2):
            s.step(0.002)
        ua, va = b.members[i].read_velocity()
        ub, vb = s.read_velocity()
        assert np.array_equal(ua, ub) and np.array_equal(va, vb)
        s.destroy()
    b.destroy()
