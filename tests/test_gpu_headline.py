"""The benchmark's own configuration against the f64 oracle.

The bench step is the channel flow past seeded disks (fluid-sim_gb300/
workload.py channel_workload, seed 5: inflow u = 1 through the fringe,
no-slip walls, five disks), MacCormack advection, explicit diffusion
nu = 1e-4, dt at CFL 0.5, the mixed-precision multigrid projection with
red-black relaxation 1.2 and 8 sweeps on the coarsest level iterated to
max|div u| <= 1e-6 after every step.
The oracle is the f64 CPU solver (restatement of src/cpu/solver.js:336-398:
MacCormack, explicit diffusion, exact FFT projection, the same channel
forcing, one direct-forcing pass per disk) from the same initial state.  Per field, relative L2 <= 1e-5 (the
tolerance of the f32 advection paths) and relative L-inf <= 1e-4; every
projection of the run met the tolerance (the device-side convergence record,
not just the last step's flag).

* 1024^2 with 64-cell level-0 tiles forced (the 2048^2 level-0 kernels' tile
  side; the built-in rule picks 32 at 1024^2), 10 steps;
* 2048^2 itself, the bench's tiles and first-cycle setting, 5 steps;
* the first V-cycle of each projection without the finest level's sweeps
  (fs_params mg_first_pre / mg_first_post).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NU, TOL, RELAX, COARSE = 1e-4, 1e-6, 1.2, 8


@pytest.fixture(scope="module")
def pkg(fs):
    fs._lib.load()
    return fs


def _gpu(pkg, n, first=(-1, -1)):
    return pkg.GPUFluidSolver(n=n, nu=NU, advection="maccormack", pressure_solver="multigrid", pressure_iterations=1,
                              precision="mixed", pressure_tol=TOL, max_cycles=60, relax=RELAX,
                              mg_coarse_sweeps=COARSE, mg_first_pre=first[0], mg_first_post=first[1])


def _run(pkg, O, n, steps, tiles=None, first=(-1, -1)):
    u0, v0, disks, dt, ch = pkg.workload.channel_workload(n, 5)
    assert len(disks) == 5
    s = _gpu(pkg, n, first)
    if tiles is not None:
        s.set_mg_tiles(tiles)
        assert s.mg_tiles()[0] == tiles[0]
    s.upload_velocity(u0, v0)
    s.set_channel(ch)
    s.set_solids(disks)
    for _ in range(steps):
        s.step(dt)
    rec = s.convergence_record()
    ug, vg = s.read_velocity()
    md = s.max_divergence()
    s.destroy()

    O.set_threads(16)
    cpu = O.CpuSolver(n=n, nu=NU, advection="maccormack", explicit_diffusion=True, projection="fft",
                      coupling_passes=1)
    cpu.u[:] = u0
    cpu.v[:] = v0
    cpu.set_channel(ch)
    for d in disks:
        cpu.add_solid(O.disk(d[0], d[1], d[2], density=8, fixed=True))
    for _ in range(steps):
        cpu.step(dt, advect_dye=False)
    cu, cv = np.asarray(cpu.u), np.asarray(cpu.v)

    assert rec["steps"] == steps and rec["failed_steps"] == 0, rec
    assert rec["worst_max_div"] <= TOL and md <= TOL, (rec, md)
    for a, b in ((ug, cu), (vg, cv)):
        rl2 = np.linalg.norm(a - b) / np.linalg.norm(b)
        linf = np.abs(a - b).max() / np.abs(b).max()
        assert rl2 <= 1e-5, rl2
        assert linf <= 1e-4, linf


def test_bench_config_1024_tile64_matches_oracle(pkg, O):
    _run(pkg, O, 1024, 10, tiles=[64, 0, 0, 0])


def test_bench_config_2048_matches_oracle(pkg, O):
    """the bench's settings, the first V-cycle of each projection without the
    finest level's sweeps included"""
    _run(pkg, O, 2048, 5, first=(0, 0))


def test_first_cycle_without_finest_sweeps_matches_oracle(pkg, O):
    """mg_first_pre = mg_first_post = 0: the first V-cycle of each projection
    runs no sweeps on the finest level (restriction of the divergence, the
    coarse levels' V(2,2), prolongation into the pressure); every projection
    still meets 1e-6 and the fields match the oracle."""
    _run(pkg, O, 1024, 10, tiles=[64, 0, 0, 0], first=(0, 0))


def test_first_cycle_sweeps_of_the_cycle_change_nothing(pkg):
    """mg_first_pre / mg_first_post equal to the cycle's sweeps (2, 2) give the
    default (-1, -1) bit for bit; (0, 0) meets the tolerance every step."""
    n, steps = 512, 6
    u0, v0, disks, dt, ch = pkg.workload.channel_workload(n, 5)
    out = []
    for first in ((-1, -1), (2, 2), (0, 0)):
        s = _gpu(pkg, n, first)
        s.upload_velocity(u0, v0)
        s.set_channel(ch)
        s.set_solids(disks)
        c0 = s.total_cycles()
        for _ in range(steps):
            s.step(dt)
        out.append((s.read_velocity(), s.total_cycles() - c0, s.convergence_record()))
        s.destroy()
    (a, ca, _), (b, cb, _), (_, cz, rz) = out
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and ca == cb
    assert rz["failed_steps"] == 0 and rz["steps"] == steps, rz
    assert cz <= ca + steps, (cz, ca)


def test_first_cycle_setting_in_eager_and_captured_steps_agree(pkg):
    """The eager step (the host knows which cycle it enqueues) and the captured
    step (the kernels read the loop's cycle count on the device) run the same
    cycles with mg_first_pre = mg_first_post = 0: equal fields, bit for bit; the
    eager profile names the first cycle's finest-level launches apart."""
    n, steps = 512, 3
    u0, v0, disks, dt, ch = pkg.workload.channel_workload(n, 5)
    res = []
    for eager in (False, True):
        s = _gpu(pkg, n, (0, 0))
        s.upload_velocity(u0, v0)
        s.set_channel(ch)
        s.set_solids(disks)
        if eager:
            prof = s.profile_step(dt, steps)
            names = {k["name"]: k["launches"] for k in prof}
            assert names.get("mg_up_acc_first") == steps and names.get("mg_down_l0_first") == steps, names
            assert names.get("mg_up_acc", 0) >= steps, names
        else:
            for _ in range(steps):
                s.step(dt)
        res.append(s.read_velocity())
        s.destroy()
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


@pytest.mark.parametrize("n,first", [(512, (0, 0)), (512, (1, 0)), (512, (0, 1)), (512, (1, 1)), (200, (0, 0)),
                                     (264, (0, 0))])
def test_first_cycle_settings_converge_to_the_same_flow(pkg, n, first):
    """Every mix of finest-level sweeps in the first cycle -- the short paths
    of (0, 0) included, and (1, 0), whose up kernel must add the prolongation
    to a smoothed iterate -- meets the tolerance every step, and the velocity
    agrees with the default cycle's to far below the tolerance's effect; n =
    200 and 264 have partial level-0 tiles (16- and 32-cell)."""
    steps = 6
    u0, v0, disks, dt, ch = pkg.workload.channel_workload(n, 5)
    out = []
    for f in ((-1, -1), first):
        s = _gpu(pkg, n, f)
        s.upload_velocity(u0, v0)
        s.set_channel(ch)
        s.set_solids(disks)
        for _ in range(steps):
            s.step(dt)
        out.append((s.read_velocity(), s.convergence_record(), s.max_divergence()))
        s.destroy()
    (a, _, _), (b, rec, md) = out
    assert rec["failed_steps"] == 0 and rec["steps"] == steps and md <= TOL, (rec, md)
    for x, y in zip(a, b):
        assert np.linalg.norm(x - y) / np.linalg.norm(x) <= 1e-5
