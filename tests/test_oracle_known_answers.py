"""Known-answer tests of the oracle, restated from the reference's test suite
(test/core.test.js, test/solver.test.js, test/validation.test.js).

These are the identities the reference asserts about its own CPU solver; the
oracle must satisfy every one of them before it is trusted as the checker.
"""
from __future__ import annotations

import math

import numpy as np
import pytest


def test_wrap(O):
    """test/core.test.js:35-42"""
    w = O.lib().fso_wrap
    assert [w(0, 8), w(7, 8), w(8, 8), w(-1, 8), w(-9, 8), w(17, 8)] == [0, 7, 0, 7, 7, 1]


def test_bilerp_exact_and_periodic(O):
    """test/core.test.js:44-64"""
    a = np.tile(np.arange(4, dtype=np.float64), 4)
    b = lambda gx, gy: O.lib().fso_bilerp(O._p(a), 4, 4, gx, gy)
    assert b(1, 1) == 1 and b(2, 0) == 2
    assert abs(b(1.5, 0) - 1.5) < 1e-15 and abs(b(1.25, 0) - 1.25) < 1e-15
    assert b(4, 0) == b(0, 0) and b(-1, 0) == b(3, 0)


def test_mac_samplers_round_trip(O):
    """test/core.test.js:66-83 -- the half-cell-offset check."""
    g = O.grid(16)
    u = O.fill(g, lambda x, y: np.sin(x) * np.cos(y), "u")
    v = O.fill(g, lambda x, y: np.cos(x) * np.sin(y), "v")
    p = O.fill(g, lambda x, y: np.sin(x + y), "p")
    L = O.lib()
    for i, j in [(0, 0), (3, 5), (15, 15), (8, 2)]:
        k = j * 16 + i
        assert abs(L.fso_sample_u(g, O._p(u), i * g.dx, (j + 0.5) * g.dy) - u[k]) < 1e-12
        assert abs(L.fso_sample_v(g, O._p(v), (i + 0.5) * g.dx, j * g.dy) - v[k]) < 1e-12
        assert abs(L.fso_sample_p(g, O._p(p), (i + 0.5) * g.dx, (j + 0.5) * g.dy) - p[k]) < 1e-12


def test_divergence_gradient_negative_adjoint(O):
    """test/core.test.js:85-120: <div w, q> = -<w, grad q> to 1e-12."""
    g = O.grid(16)
    r = O.lcg(12345, 3 * 256)
    wu, wv, q = r[:256].copy(), r[256:512].copy(), r[512:].copy()
    lhs = float(np.dot(O.divergence(g, wu, wv), q))
    gu, gv = O.zeros(g), O.zeros(g)
    O.subtract_gradient(g, gu, gv, q, -1.0)
    rhs = float(np.dot(wu, gu) + np.dot(wv, gv))
    assert abs(lhs + rhs) / max(abs(lhs), abs(rhs), 1e-30) < 1e-12


def test_constant_field_divergence_free(O):
    """test/core.test.js:122-126"""
    g = O.grid(32)
    assert O.max_divergence(g, np.full(1024, 1.3), np.full(1024, -0.7)) < 1e-14


@pytest.mark.parametrize("n", [16, 32, 64])
def test_taylor_green_discretely_divergence_free(O, n):
    """test/core.test.js:138-149 (phase-0 gate): max|div| < 1e-14."""
    g = O.grid(n)
    u, v = O.tg_init(g, 0.0, 0.01)
    assert O.max_divergence(g, u, v) < 1e-14


def test_taylor_green_kinetic_energy(O):
    """test/core.test.js:160-173"""
    g = O.grid(128)
    u, v = O.tg_init(g, 0.7, 0.03)
    exact = 0.25 * math.exp(-4 * 0.03 * 0.7)
    assert abs(O.kinetic_energy(g, u, v) - exact) / exact < 2e-3


def test_fft_matches_naive_dft_and_round_trips(O):
    """test/core.test.js:256-273 (FFT vs DFT) and the ifft round trip."""
    n = 64
    x = O.lcg(4242, 2 * n)
    re, im = x[:n].copy(), x[n:].copy()
    fr, fi = re.copy(), im.copy()
    O.lib().fso_fft_inplace(O._p(fr), O._p(fi), n, -1)
    dr, di = np.zeros(n), np.zeros(n)
    O.lib().fso_dft_naive(O._p(re), O._p(im), O._p(dr), O._p(di), n, -1)
    assert np.max(np.abs(fr - dr)) < 1e-12 and np.max(np.abs(fi - di)) < 1e-12
    O.lib().fso_fft_inplace(O._p(fr), O._p(fi), n, +1)
    assert np.max(np.abs(fr / n - re)) < 1e-14


def test_parseval(O):
    """test/core.test.js:318-345: sum E(k) equals the physical KE for a field
    with no corner modes."""
    g = O.grid(64)
    u, v = O.tg_init(g)
    cu, cv = O.velocity_at_centers(g, u, v)
    E, counts = O.energy_spectrum(cu, cv, 64, 64)
    phys = 0.5 * float(np.sum(cu * cu + cv * cv)) / cu.size
    assert abs(E.sum() - phys) / phys < 1e-12
    assert counts.sum() <= 64 * 64


def test_laplacian_symmetric_null_space_second_order(O):
    """test/solver.test.js:31-72"""
    g = O.grid(16)
    r = O.lcg(4242, 512)
    x, y = r[0::2].copy(), r[1::2].copy()
    lhs, rhs = np.dot(O.laplacian(g, x), y), np.dot(x, O.laplacian(g, y))
    assert abs(lhs - rhs) / max(abs(lhs), 1e-30) < 1e-12
    assert np.max(np.abs(O.laplacian(g, np.full(256, 3.7)))) < 1e-12
    hs, errs = [], []
    for n in (16, 32, 64, 128):
        g = O.grid(n)
        p = O.fill(g, lambda x, y: np.sin(x) * np.sin(y))
        ex = O.fill(g, lambda x, y: -2 * np.sin(x) * np.sin(y))
        hs.append(g.dx)
        errs.append(O.rel_l2(O.laplacian(g, p), ex))
    order = np.polyfit(np.log(hs), np.log(errs), 1)[0]
    assert 1.9 < order < 2.1


def test_cg_tolerance_and_versus_jacobi(O):
    """test/solver.test.js:76-129"""
    g = O.grid(32)
    rhs = O.fill(g, lambda x, y: -2 * np.sin(x) * np.sin(y))
    p, it, res = O.poisson_cg(g, rhs, tol=1e-12, max_iter=500)
    assert res < 1e-12
    assert O.rel_l2(p, O.fill(g, lambda x, y: np.sin(x) * np.sin(y))) < 5e-3
    rhs = O.fill(g, lambda x, y: np.sin(3 * x) * np.cos(2 * y))
    _, it, res_cg = O.poisson_cg(g, rhs, tol=1e-10, max_iter=2000)
    _, res_j, _ = O.poisson_jacobi(g, rhs, 200)
    assert res_cg <= 1e-10 and it < 60 and res_j > res_cg
    _, _, hist = O.poisson_jacobi(g, O.fill(g, lambda x, y: np.sin(2 * x) * np.sin(y)), 40)
    assert np.all(np.diff(hist) <= 1e-14)
    _, _, res = O.poisson_cg(O.grid(16), O.fill(O.grid(16), lambda x, y: np.sin(x) * np.sin(y) + 5), 1e-11, 500)
    assert res <= 1e-11


def test_projection_divergence_free_and_idempotent(O):
    """test/solver.test.js:133-181"""
    g = O.grid(32)
    u, v = O.lcg_uv(777, 1024)
    assert O.max_divergence(g, u, v) > 0.1
    O.project(g, u, v, tol=1e-12)
    assert O.max_divergence(g, u, v) < 1e-10
    u, v = O.tg_init(g, 0.0, 0.01)
    u0, v0 = u.copy(), v.copy()
    O.project(g, u, v, tol=1e-13)
    assert max(np.abs(u - u0).max(), np.abs(v - v0).max()) < 1e-11
    g = O.grid(16)
    u, v = O.lcg_uv(31337, 256)
    O.project(g, u, v, tol=1e-13)
    u1, v1 = u.copy(), v.copy()
    O.project(g, u, v, tol=1e-13)
    assert max(np.abs(u - u1).max(), np.abs(v - v1).max()) < 1e-11


def test_fft_and_cg_projection_agree(O):
    """test/validation.test.js:201-222"""
    def run(proj):
        s = O.CpuSolver(n=32, nu=0.02, projection=proj, proj_tol=1e-14, proj_max_iter=5000)
        g = s.g
        s.u[:] = O.fill(g, lambda x, y: np.sin(x) * np.cos(y) + 0.1 * np.sin(3 * x + y), "u")
        s.v[:] = O.fill(g, lambda x, y: -np.cos(x) * np.sin(y) + 0.1 * np.cos(x - 2 * y), "v")
        for _ in range(5):
            s.step(0.01, advect_dye=False)
        return s
    a, b = run("cg"), run("fft")
    m = max(np.abs(a.u - b.u).max(), np.abs(a.v - b.v).max())
    scale = max(np.abs(b.u).max(), np.abs(b.v).max())
    assert m / scale < 1e-9


def test_implicit_diffusion_amplitude_and_mean(O):
    """test/solver.test.js:185-223"""
    g = O.grid(64)
    q = O.fill(g, lambda x, y: np.sin(x) * np.sin(y))
    out, _ = O.diffuse(g, q, 0.05, 0.01)
    amp = np.dot(out, q) / np.dot(q, q)
    assert abs(amp - 1 / (1 + 2 * 0.05 * 0.01)) / (1 / 1.001) < 2e-3
    g = O.grid(32)
    q = O.fill(g, lambda x, y: 2 + np.sin(x) * np.cos(y))
    out, _ = O.diffuse(g, q, 0.1, 0.05)
    assert abs(out.sum() - q.sum()) / abs(q.sum()) < 1e-9


def test_advection_constant_and_limiter(O):
    """test/solver.test.js:227-295"""
    g = O.grid(32)
    u, v, q = np.full(1024, 0.7), np.full(1024, -0.4), np.full(1024, 2.5)
    for scheme in ("semi-lagrangian", "maccormack"):
        assert np.abs(O.advect_scalar(g, u, v, q, 0.05, scheme) - 2.5).max() < 1e-12
    g = O.grid(64)
    u, v = np.full(4096, 1.0), np.full(4096, 0.5)
    q = O.fill(g, lambda x, y: ((x > 2) & (x < 4) & (y > 2) & (y < 4)).astype(float))
    for _ in range(40):
        q = O.advect_scalar(g, u, v, q, 0.02, "maccormack")
    assert q.min() > -1e-9 and q.max() < 1 + 1e-9


def test_solver_div_free_every_step_and_uniform_flow(O):
    """test/solver.test.js:299-322"""
    s = O.CpuSolver(n=32, nu=0.01, proj_tol=1e-11).init_tg(0.01)
    for _ in range(20):
        s.step(0.02)
        assert s.max_divergence() < 1e-9
    s = O.CpuSolver(n=32, nu=0.05)
    s.u[:], s.v[:] = 1.3, -0.7
    for _ in range(10):
        s.step(0.05)
    assert max(np.abs(s.u - 1.3).max(), np.abs(s.v + 0.7).max()) < 1e-9


def test_taylor_green_tracks_analytic(O):
    """test/solver.test.js:339-361"""
    nu, dt = 0.05, 0.01
    s = O.CpuSolver(n=64, nu=nu, advection="maccormack").init_tg(nu)
    for _ in range(50):
        s.step(dt)
    assert O.tg_error(s.g, s.u, s.v, s.t, nu) < 0.05
    ke = s.kinetic_energy()
    assert ke < 0.25 and ke < 0.25 * math.exp(-4 * nu * s.t) * 1.02


def test_first_order_in_time(O):
    """test/solver.test.js:363-398: Lie splitting caps the step at first order."""
    nu, T, n = 0.05, 0.25, 32
    dts = [0.02, 0.01, 0.005, 0.0025]
    errs = []
    for dt in dts:
        s = O.CpuSolver(n=n, nu=nu, advection="maccormack", proj_tol=1e-12).init_tg(nu)
        for _ in range(math.floor(T / dt + 0.5)):
            s.step(dt, advect_dye=False)
        errs.append(O.tg_error(s.g, s.u, s.v, s.t, nu))
    assert all(errs[i] < errs[i - 1] for i in range(1, len(errs)))
    order = np.polyfit(np.log(dts), np.log(errs), 1)[0]
    assert 0.85 < order < 1.35


def test_blow_up_detection(O):
    """test/solver.test.js:428-438"""
    s = O.CpuSolver(n=16, nu=0.01)
    s.u[:] = 1.0
    assert not s.is_blown_up()
    s.u[5] = np.nan
    assert s.is_blown_up()
    s.u[5] = np.inf
    assert s.is_blown_up()


def test_rejects_unknown_scheme_and_non_pow2_fft(O):
    """src/cpu/solver.js:265-297 guards."""
    with pytest.raises(ValueError):
        O.CpuSolver(n=16, advection="quicK")
    with pytest.raises(ValueError):
        O.CpuSolver(n=24, projection="fft")


def test_lcg_matches_reference_fixture(O):
    """The JS LCG evaluated in doubles: the first values of seed 12345 depend on
    the >2^53 product being rounded before the ToInt32 wrap."""
    x = O.lcg(12345, 4)
    s = 12345
    exp = []
    for _ in range(4):
        t = float(s) * 1103515245.0 + 12345.0
        s = int(math.fmod(t, 4294967296.0)) & 0x7FFFFFFF
        exp.append(s / 0x7FFFFFFF - 0.5)
    assert list(x) == exp


def test_relaxation_factor_in_reference_gpu_restatement(O):
    """param_a of RED_BLACK_GS (shaders.js:368): 1.0 set explicitly gives the
    reference's curve bit for bit; 1.2 on every multigrid sweep lowers the
    residual after the same V-cycles (64^2, seed 777)."""
    n = 64
    u0, v0 = O.lcg_uv(777, n * n)
    res = {}
    for relax in (None, 1.0, 1.2):
        r = O.RefGpuSolver(n=n, nu=0.0, pressure_solver="multigrid", precision="f64")
        if relax is not None:
            r.set_relax(relax)
        r.upload_velocity(u0, v0)
        res[relax] = [r.poisson_residual_after(k) for k in (1, 2, 3)]
    assert res[None] == res[1.0]
    assert all(a < b for a, b in zip(res[1.2], res[1.0]))
