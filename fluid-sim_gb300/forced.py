"""Forced two-dimensional turbulence on the GPU: the long-run spectrum driver.

The reference runs this study on its f64 CPU solver
(validate/longrun-spectrum.js: band forcing renewed every step with seed++,
linear drag, MacCormack, FFT projection, from rest, spectra of the centre
velocity as it goes).  Here every step is one captured graph of the GPU
solver -- the band forcing's draws are made on the device from (seed, step)
-- and the spectrum is the device FFT (fs_energy_spectrum), so the run never
reads the velocity back.

The default configuration is the forced-turbulence workload: a periodic
1024^2 grid from rest, Gaussian complex amplitudes on every integer wave
vector with 8 <= |k| <= 10 renewed each step (Philox), nu = 1e-4, linear drag
0.1, MacCormack advection, red-black multigrid V-cycles to a relative
residual of 1e-6, 5000 steps, the spectrum every 100 steps.
"""
from __future__ import annotations

import math
import time

import numpy as np

from .solver import GPUFluidSolver


def fit_slope(k, E, k_lo, k_hi):
    """Least-squares slope of log E against log k over k_lo <= k <= k_hi
    (fitSlope, src/core/fft.js:286-310): slope, intercept, r^2, points."""
    sel = [(math.log(a), math.log(b)) for a, b in zip(k, E) if k_lo <= a <= k_hi and b > 0 and a > 0]
    n = len(sel)
    if n < 3:
        return {"slope": float("nan"), "intercept": float("nan"), "r2": float("nan"), "n": n}
    xs = np.array([p[0] for p in sel])
    ys = np.array([p[1] for p in sel])
    mx, my = xs.mean(), ys.mean()
    dx, dy = xs - mx, ys - my
    sxy, sxx, syy = float((dx * dy).sum()), float((dx * dx).sum()), float((dy * dy).sum())
    slope = sxy / sxx
    return {"slope": slope, "intercept": my - slope * mx, "r2": sxy * sxy / (sxx * syy) if syy > 0 else float("nan"),
            "n": n}


def run_forced_turbulence(n: int = 1024, steps: int = 5000, every: int = 100, dt: float = 2e-3, nu: float = 1e-4,
                          drag: float = 0.1, kf: float = 9.0, width: float = 1.0, amplitude: float = 3.0,
                          seed: int = 1, tol: float = 1e-6, device: int = 0, relax: float = 1.2):
    """Run the forced-turbulence study on the GPU.  Returns the record: the
    energy spectrum and kinetic energy every `every` steps, the averaged
    spectrum over the last 40% of the snapshots with its two slope fits
    (windows fixed from kf before the run, as the reference fixes them), the
    device time of the steps and the convergence record of the projections."""
    s = GPUFluidSolver(n=n, nu=nu, advection="maccormack", pressure_solver="multigrid", pressure_iterations=1,
                       precision="mixed", pressure_tol=tol, pressure_tol_relative=True, max_cycles=60,
                       device=device, relax=relax)
    try:
        s.upload_velocity(np.zeros(n * n), np.zeros(n * n))
        s.set_band_forcing("gaussian", kf=kf, width=width, amplitude=amplitude, seed=seed, drag=drag)
        snaps = []
        step_ms = 0.0
        t0 = time.perf_counter()
        done = 0
        while done < steps:
            chunk = min(every, steps - done)
            step_ms += s.time_steps(dt, chunk)
            done += chunk
            k, E, cnt, (esum, ke) = s.energy_spectrum()
            snaps.append({"step": done, "ke": ke, "parseval": esum, "E": E})
        wall = time.perf_counter() - t0
        rec = s.convergence_record()
        cycles = s.total_cycles()
    finally:
        s.destroy()
    kmax = n // 2
    windows = {"inverse": (4, math.floor(kf * 0.62)) if kf * 0.62 >= 6 else (2, max(3, math.floor(kf * 0.8))),
               "enstrophy": (math.ceil(kf * 1.5), math.floor(kmax * 0.7))}
    tail = snaps[int(len(snaps) * 0.6):] or snaps[-1:]
    E_avg = np.mean([sn["E"] for sn in tail], axis=0)
    kk = np.arange(kmax + 1)
    return {"n": n, "steps": steps, "every": every, "dt": dt, "nu": nu, "drag": drag, "band": [kf - width, kf + width],
            "amplitude": amplitude, "seed": seed, "tol_relative": tol,
            "ms_per_step": step_ms / steps, "cell_steps_per_s": float(n) * n * steps / (step_ms / 1e3),
            "wall_s": wall, "cycles_per_step": cycles / steps, "failed_steps": rec["failed_steps"],
            "projections": rec["steps"], "ke": [sn["ke"] for sn in snaps],
            "parseval_max_rel_err": max(abs(sn["parseval"] - sn["ke"]) / max(sn["ke"], 1e-300) for sn in snaps),
            "spectrum_avg": E_avg, "averaged_snapshots": len(tail), "windows": windows,
            "fits": {"inverse": fit_slope(kk, E_avg, *windows["inverse"]),
                     "enstrophy": fit_slope(kk, E_avg, *windows["enstrophy"])}}
