"""Batches of uneven simulations (fs_batch_*): one graph launch per step.

Each member's step is the same captured kernel sequence as a solver stepped
alone (same kernels, same deterministic reductions), so after K batch steps
every member must equal an independently stepped solver bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CFG = dict(nu=1e-3, advection="maccormack", pressure_solver="multigrid", pressure_iterations=1,
           precision="mixed", pressure_tol=1e-8, max_cycles=60)


@pytest.fixture(scope="module")
def pkg(fs):
    fs._lib.load()
    return fs


def _members(pkg, sides, seed0=20):
    states = [pkg.workload.vortex_blobs(n, seed0 + i) for i, n in enumerate(sides)]
    return states


def test_batch_equals_independent_solvers(pkg):
    sides = [64, 96, 128, 64]
    states = _members(pkg, sides)
    b = pkg.GPUFluidBatch([dict(n=n, **CFG) for n in sides])
    _, _, disks, _ = pkg.workload.make_workload(64, 3)
    for m, (u, v, _) in zip(b.members, states):
        m.upload_velocity(u, v)
    b.members[1].set_solids([(1.0, 2.0, 0.4)])
    dts = [dt for _, _, dt in states]
    for _ in range(4):
        b.step(dts)
    b.sync()
    for i, (n, (u, v, dt)) in enumerate(zip(sides, states)):
        s = pkg.GPUFluidSolver(n=n, **CFG)
        s.upload_velocity(u, v)
        if i == 1:
            s.set_solids([(1.0, 2.0, 0.4)])
        for _ in range(4):
            s.step(dt)
        ua, va = b.members[i].read_velocity()
        ub, vb = s.read_velocity()
        assert np.array_equal(ua, ub) and np.array_equal(va, vb), f"member {i} (n={n})"
        st = b.members[i].last_stats()
        assert st["converged"] and st["residual_max"] <= 1e-8
        assert b.members[i].steps == 4
        s.destroy()
    assert b.launch_count() > 4 * len(sides) * 10
    b.destroy()


def test_batch_recaptures_on_change(pkg):
    sides = [64, 128]
    states = _members(pkg, sides, 40)
    b = pkg.GPUFluidBatch([dict(n=n, **CFG) for n in sides])
    for m, (u, v, _) in zip(b.members, states):
        m.upload_velocity(u, v)
    dts = [dt for _, _, dt in states]
    b.step(dts)
    b.members[0].set_solids([(3.0, 3.0, 0.5)])  # invalidates the captured branch
    b.step(dts)
    b.step([0.5 * d for d in dts])  # new dt: another capture
    s = pkg.GPUFluidSolver(n=64, **CFG)
    s.upload_velocity(states[0][0], states[0][1])
    s.step(dts[0])
    s.set_solids([(3.0, 3.0, 0.5)])
    s.step(dts[0])
    s.step(0.5 * dts[0])
    ua, _ = b.members[0].read_velocity()
    ub, _ = s.read_velocity()
    assert np.array_equal(ua, ub)
    s.destroy()
    b.destroy()


def test_batch_rejects_unfused_members(pkg):
    with pytest.raises(pkg.FluidError):
        pkg.GPUFluidBatch([dict(n=64, **CFG), dict(n=64, pressure_solver="jacobi", pressure_iterations=10)])


def test_batch_of_uneven_sides_times(pkg):
    sides = pkg.workload.batch_sides(24, 1)
    b = pkg.GPUFluidBatch([dict(n=n, **CFG) for n in sides])
    dts = []
    for i, (m, n) in enumerate(zip(b.members, sides)):
        u, v, dt = pkg.workload.vortex_blobs(n, 100 + i)
        m.upload_velocity(u, v)
        dts.append(dt)
    ms = b.time_steps(dts, 5)
    assert ms > 0
    for m in b.members:
        assert m.last_stats()["converged"]
    b.destroy()


def test_batch_mixed_paths_equal_independent_solvers(pkg):
    """Three ways a member steps inside a batch, each bit for bit equal to the
    same solver stepped alone: two 64^2 members in one size class of which one
    has forcing (the class loop is batched, their other kernels run as member
    branches), an F32 member with a tolerance (outside every class: its own
    captured step), and a plain 128^2 class (its whole step batched)."""
    f32 = dict(CFG, precision="f32", pressure_tol=1e-4)
    cfgs = [dict(n=64, **CFG), dict(n=64, **CFG), dict(n=64, **f32), dict(n=128, **CFG)]
    states = _members(pkg, [c["n"] for c in cfgs], 60)
    modes = [(3.0, 1.0, 0.2), (0.0, 4.0, 1.0)]

    def setup(s, i, u, v):
        s.upload_velocity(u, v)
        if i == 1:
            s.set_forcing(modes, amplitude=0.5, drag=0.1)

    b = pkg.GPUFluidBatch(cfgs)
    for i, (m, (u, v, _)) in enumerate(zip(b.members, states)):
        setup(m, i, u, v)
    dts = [dt for _, _, dt in states]
    for _ in range(3):
        b.step(dts)
    b.sync()
    for i, (cfg, (u, v, dt)) in enumerate(zip(cfgs, states)):
        s = pkg.GPUFluidSolver(**cfg)
        setup(s, i, u, v)
        for _ in range(3):
            s.step(dt)
        ua, va = b.members[i].read_velocity()
        ub, vb = s.read_velocity()
        assert np.array_equal(ua, ub) and np.array_equal(va, vb), f"member {i}"
        assert b.members[i].last_stats()["cycles"] == s.last_stats()["cycles"]
        s.destroy()
    b.destroy()


def test_batch_tile_autotune_keeps_results(pkg):
    """fs_batch_autotune_tiles times tile sides per class and level from one
    saved state, restores it, and the tuned batch still equals the members
    stepped alone bit for bit (the tiles give the same values whatever their size)."""
    sides = [128, 128, 256, 64]
    states = _members(pkg, sides, 80)
    b = pkg.GPUFluidBatch([dict(n=n, **CFG) for n in sides])
    for m, (u, v, _) in zip(b.members, states):
        m.upload_velocity(u, v)
    dts = [dt for _, _, dt in states]
    b.step(dts)
    b.sync()
    before = [m.read_velocity()[0] for m in b.members]
    r = b.autotune_tiles(dts, 1)
    assert r["ms_per_step"] > 0 and set(r["tiles"]) == {(128, 128), (256, 256), (64, 64)}
    assert all(np.array_equal(x, m.read_velocity()[0]) for x, m in zip(before, b.members))
    for _ in range(2):
        b.step(dts)
    b.sync()
    for i, (n, (u, v, dt)) in enumerate(zip(sides, states)):
        s = pkg.GPUFluidSolver(n=n, **CFG)
        s.upload_velocity(u, v)
        for _ in range(3):
            s.step(dt)
        assert np.array_equal(b.members[i].read_velocity()[0], s.read_velocity()[0]), f"member {i}"
        assert b.members[i].steps == 3
        s.destroy()
    assert b.launch_count() > 0
    b.destroy()


def test_batch_members_with_channel_and_band_forcing(pkg):
    """Members with the channel (walls and inflow fringe) or the renewed band
    forcing leave the batched launches of their class and run their own
    captured step; they still equal independently stepped solvers bit for
    bit, and the band forcing's draws advance per member."""
    sides = [128, 128, 128]
    ch = pkg.workload.channel_geometry()
    states = _members(pkg, sides, seed0=40)
    b = pkg.GPUFluidBatch([dict(n=n, **CFG) for n in sides])
    for m, (u, v, _) in zip(b.members, states):
        m.upload_velocity(u, v)
    b.members[0].set_channel(ch)
    b.members[1].set_band_forcing("gaussian", kf=6.0, width=1.0, amplitude=2.0, seed=5, drag=0.1)
    dts = [dt for _, _, dt in states]
    for _ in range(3):
        b.step(dts)
    b.sync()
    for i, (n, (u, v, dt)) in enumerate(zip(sides, states)):
        s = pkg.GPUFluidSolver(n=n, **CFG)
        s.upload_velocity(u, v)
        if i == 0:
            s.set_channel(ch)
        if i == 1:
            s.set_band_forcing("gaussian", kf=6.0, width=1.0, amplitude=2.0, seed=5, drag=0.1)
        for _ in range(3):
            s.step(dt)
        ua, va = b.members[i].read_velocity()
        ub, vb = s.read_velocity()
        assert np.array_equal(ua, ub) and np.array_equal(va, vb), f"member {i}"
        s.destroy()
    b.destroy()
