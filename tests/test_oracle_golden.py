"""Pin the oracle against the reference's own committed run outputs.

The reference is JavaScript and does not run here; ``tests/golden/
reference_results.json`` holds numbers extracted (by ``extract_golden.py``)
from its ``results/validation.json`` (Node 24, f64 CPU solver) and
``results/gpu-verify.json`` (WebGPU, f32).  Reproducing them shows the C
restatements compute what the reference computes before they are trusted as
the checker of the CUDA path.
"""
from __future__ import annotations

import math

import numpy as np
import pytest


def jsround(x: float) -> int:
    """JavaScript Math.round: halves round toward +infinity (Python rounds to even)."""
    return math.floor(x + 0.5)


def _decay_fit(ts, kes):
    """validate/studies.js:150-166: least-squares slope of log KE against t."""
    ts = np.asarray(ts)
    les = np.log(np.asarray(kes))
    mt, ml = ts.mean(), les.mean()
    stl = np.sum((ts - mt) * (les - ml))
    stt = np.sum((ts - mt) ** 2)
    sll = np.sum((les - ml) ** 2)
    rate = -stl / stt
    return rate, stl * stl / (stt * sll)


@pytest.mark.parametrize("scheme", ["semi-lagrangian", "maccormack"])
def test_taylor_green_trace_matches_reference_run(O, golden, scheme):
    """validate/studies.js:121-177 at n=64, nu=0.02, dt=0.005, T=1, CG tol 1e-11,
    implicit diffusion: KE, enstrophy, error vs exact, and CG iteration counts
    at every recorded time agree with the reference's own f64 run."""
    tg = golden["taylorGreen"]
    n, nu, dt, T = tg["n"], tg["nu"], tg["dt"], tg["T"]
    s = O.CpuSolver(n=n, nu=nu, advection=scheme, proj_tol=1e-11).init_tg(nu)
    steps = jsround(T / dt)
    every = max(1, jsround(steps / 40))
    rec = [(s.t, s.kinetic_energy(), s.enstrophy(), O.tg_error(s.g, s.u, s.v, s.t, nu), 0)]
    for k in range(steps):
        s.step(dt, advect_dye=False)
        if (k + 1) % every == 0:
            rec.append((s.t, s.kinetic_energy(), s.enstrophy(), O.tg_error(s.g, s.u, s.v, s.t, nu),
                        s.last_iterations))
    ref = tg["schemes"][scheme]["trace"]
    assert len(rec) == len(ref)
    for (t, ke, ens, rel, it), r in zip(rec, ref):
        assert t == pytest.approx(r["t"], rel=1e-15)
        assert ke == pytest.approx(r["ke"], rel=1e-12)
        assert ens == pytest.approx(r["enstrophy"], rel=1e-12)
        if r["relL2"] > 0:
            assert rel == pytest.approx(r["relL2"], rel=1e-10)
        # libm and V8 may differ in the last ulp of sin/cos in the initial field,
        # which can move the CG stopping point by one iteration.
        assert abs(it - r["cgIterations"]) <= 1
    rate, r2 = _decay_fit([x[0] for x in rec], [x[1] for x in rec])
    nu_num = rate / 4 - nu
    assert nu_num == pytest.approx(tg["schemes"][scheme]["nuNumerical"], rel=1e-9)
    assert r2 == pytest.approx(tg["schemes"][scheme]["decayFitR2"], rel=1e-9)


def test_numerical_viscosity_golden_values(golden):
    """README.md:27 -- nu_num: MacCormack 5.79e-4, semi-Lagrangian 2.10e-2."""
    s = golden["taylorGreen"]["schemes"]
    assert s["maccormack"]["nuNumerical"] == pytest.approx(5.79e-4, rel=2e-3)
    assert s["semi-lagrangian"]["nuNumerical"] == pytest.approx(2.10e-2, rel=5e-3)


@pytest.mark.parametrize("scheme", ["semi-lagrangian", "maccormack"])
def test_translating_gaussian_matches_reference_run(O, golden, scheme):
    """validate/studies.js:48-97: blob advected by (1, 0.6), n=64, dt=0.02."""
    a = golden["advection"]
    n, dt, steps, sigma = a["n"], a["dt"], a["steps"], a["sigma0"]
    g = O.grid(n)
    opts = dict(sigma=sigma, ax=1.0, ay=0.6, cx=math.pi, cy=math.pi)
    gauss = lambda t: (lambda X, Y: np.vectorize(lambda x, y: O.lib().fso_gaussian_scalar(
        x, y, t, opts["sigma"], opts["ax"], opts["ay"], opts["cx"], opts["cy"]))(X, Y))
    q = O.fill(g, gauss(0.0))
    u = np.full(n * n, 1.0)
    v = np.full(n * n, 0.6)
    ref = {p["step"]: p for p in a["schemes"][scheme]["trace"]}
    assert q.max() == pytest.approx(a["schemes"][scheme]["peakInitial"], rel=1e-14)
    for k in range(steps):
        q = O.advect_scalar(g, u, v, q, dt, scheme)
        if (k + 1) in ref:
            exact = O.fill(g, gauss((k + 1) * dt))
            assert O.rel_l2(q, exact) == pytest.approx(ref[k + 1]["relL2"], rel=1e-11)
            assert q.max() == pytest.approx(ref[k + 1]["peak"], rel=1e-13)


def test_convergence_table_matches_reference_run(O, golden):
    """validate/studies.js:191-230: MacCormack TG error over dt x N."""
    c = golden["convergence"]
    nu, T = c["nu"], c["T"]
    for row in c["table"]:
        n = row["n"]
        if n > 32:
            continue  # n = 64 rows take ~10 s and add nothing the n = 16, 32 rows do not pin
        for e in row["errors"]:
            dt = e["dt"]
            s = O.CpuSolver(n=n, nu=nu, advection="maccormack", proj_tol=1e-12).init_tg(nu)
            for _ in range(jsround(T / dt)):
                s.step(dt, advect_dye=False)
            assert O.tg_error(s.g, s.u, s.v, s.t, nu) == pytest.approx(e["relL2"], rel=1e-8)


def test_explicit_diffusion_amplification_matches_reference_run(O, golden):
    """validate/studies.js:275-300: the checkerboard grows by exactly |1 - 8d|."""
    ed = golden["explicitDiffusion"]
    n, nu = ed["n"], ed["nu"]
    g = O.grid(n)
    i, j = np.meshgrid(np.arange(n), np.arange(n))
    for p in ed["isolated"]:
        q = np.where((i + j) % 2 == 0, 1.0, -1.0).ravel()
        amps = []
        for _ in range(10):
            q, _ = O.diffuse(g, q, nu, p["dt"], explicit=True)
            amps.append(np.abs(q).max())
        np.testing.assert_allclose(amps, p["amplitudes"], rtol=1e-12)
        growth = amps[-1] / amps[-2]
        assert abs(growth - p["predictedAmplification"]) < 1e-6
        assert (growth > 1 + 1e-9) == p["unstable"]
    assert ed["measuredBoundary"]["isolated"] == {"lastStable": 0.25, "firstUnstable": 0.26}


def test_projection_iteration_sweep_matches_reference_run(O, golden):
    """validate/studies.js:437-454: TG with CG capped at maxIter iterations."""
    pi = golden["projectionIterations"]
    n, nu = pi["n"], pi["nu"]
    for p in pi["points"]:
        s = O.CpuSolver(n=n, nu=nu, advection="semi-lagrangian", proj_tol=1e-14,
                        proj_max_iter=p["maxIter"]).init_tg(nu)
        for _ in range(50):
            s.step(0.01, advect_dye=False)
        md = s.max_divergence()
        # A CG truncated after 2-20 iterations is chaotic at the ulp level: one
        # ulp changed in one input value moves max|div| after 50 steps by 1e-6
        # (2 iterations) to 1.4% (10 iterations).  libm and V8 differ by an ulp
        # in sin/cos, so those points are pinned to 3%; 1 iteration and the
        # converged runs are pinned tightly.
        tight = p["maxIter"] == 1
        if p["maxDivergence"] > 1e-12:
            assert md == pytest.approx(p["maxDivergence"], rel=1e-8 if tight else 3e-2)
        else:
            assert md < 1e-14
        err = O.tg_error(s.g, s.u, s.v, s.t, nu)
        assert err == pytest.approx(p["relL2"], rel=1e-12 if tight or p["maxIter"] >= 50 else 1e-4)


@pytest.mark.parametrize("solver", ["jacobi", "red-black", "multigrid"])
def test_reference_gpu_poisson_curves_reproduced(O, golden, solver):
    """tools/gputest.html:188-228: residual after k sweeps / V-cycles at 64^2
    from the seed-777 field, as the reference WebGPU backend measured it.

    The f32 restatement matches to ~1e-6 wherever the curve is above the f32
    floor (~1e-7); the multigrid plateau is round-off and only its level is
    checked."""
    n = 64
    u0, v0 = O.lcg_uv(777, n * n)
    s = O.RefGpuSolver(n=n, nu=0.0, pressure_solver=solver, precision="f32")
    s.upload_velocity(u0, v0)
    for p in golden["gpu"]["poissonCurves"][solver]:
        r = s.poisson_residual_after(p["iterations"])
        ref = p["residual"]
        if ref > 1e-4:
            assert r == pytest.approx(ref, rel=1e-5)
        elif ref > 1e-6:
            assert r == pytest.approx(ref, rel=1e-2)
        else:
            assert 3e-8 < r < 3e-7  # the f32 plateau the reference shows (~9e-8)


def test_reference_gpu_multigrid_converges_in_f64(O, golden):
    """The same V-cycle in f64 has no plateau: residual falls ~15x per cycle."""
    n = 64
    u0, v0 = O.lcg_uv(777, n * n)
    s = O.RefGpuSolver(n=n, nu=0.0, pressure_solver="multigrid", precision="f64")
    s.upload_velocity(u0, v0)
    curve = golden["gpu"]["poissonCurves"]["multigrid"]
    for p in curve[:4]:
        assert s.poisson_residual_after(p["iterations"]) == pytest.approx(p["residual"], rel=1e-5)
    assert s.poisson_residual_after(12) < 1e-13


def test_reference_gpu_ten_step_agreement_reproduced(O, golden):
    """tools/gputest.html:233-263: 10 steps, SL, RBGS-400 against the f64 CPU
    solver with FFT projection; the reference measured relL2 3.31e-6 and
    GPU max|div| 1.76e-5."""
    n, dt = 64, 0.01
    g = O.grid(n)
    u0, v0 = O.tg_init(g)
    cpu = O.CpuSolver(n=n, nu=0.0, projection="fft")
    cpu.u[:], cpu.v[:] = u0, v0
    gpu = O.RefGpuSolver(n=n, nu=0.0, pressure_solver="red-black", pressure_iterations=400,
                         advection="semi-lagrangian", precision="f32")
    gpu.upload_velocity(u0, v0)
    for _ in range(10):
        cpu.step(dt, advect_dye=False)
        gpu.step(dt)
    u, v = gpu.read_velocity()
    ref = golden["gpu"]["fullStep"]
    du, dv = O.rel_l2(u, cpu.u), O.rel_l2(v, cpu.v)
    assert max(du, dv) < 5e-3  # the reference's own gate
    assert max(du, dv) == pytest.approx(ref["du"], rel=0.5)
    assert gpu.max_divergence() == pytest.approx(ref["gpuMaxDiv"], rel=0.5)


def test_reference_gpu_scheme_energy_reproduced(O, golden):
    """tools/gputest.html:300-327: KE after 200 steps at nu=0, MG-3, 64^2."""
    n = 64
    g = O.grid(n)
    ke = {}
    for scheme in ("semi-lagrangian", "maccormack"):
        u0, v0 = O.tg_init(g)
        s = O.RefGpuSolver(n=n, nu=0.0, pressure_solver="multigrid", pressure_iterations=3,
                           advection=scheme, precision="f32")
        s.upload_velocity(u0, v0)
        for _ in range(200):
            s.step(0.01)
        u, v = s.read_velocity()
        ke[scheme] = 0.5 * float(np.sum(u * u + v * v)) / u.size
    ref = golden["gpu"]["schemeEnergy"]
    assert ke["semi-lagrangian"] == pytest.approx(ref["semi-lagrangian"], rel=1e-4)
    assert ke["maccormack"] == pytest.approx(ref["maccormack"], rel=1e-4)


def test_cpu_solid_force_matches_reference_run(O, golden):
    """tools/gputest.html:372-409: pinned disk in a unit stream, one coupling
    pass; the CPU force on the body was 1.1449815477540885e2."""
    n, dt = 128, 0.01
    cpu = O.CpuSolver(n=n, nu=0.0, projection="fft", advection="maccormack", coupling_passes=1)
    cpu.u[:] = 1.0
    cpu.v[:] = 0.0
    cpu.add_solid(O.disk(math.pi, math.pi, 0.6, density=8, fixed=True))
    cpu.step(dt, advect_dye=False)
    f = cpu.solid(0).force[0]
    assert f == pytest.approx(golden["gpu"]["gpuSolidAgreement"]["fCpu"], rel=1e-12)
