"""The numpy V-cycle model (fluid-sim_gb300/vcycle_model.py) against the
oracle's f64 restatement of the reference multigrid (src/gpu/multigrid.js
:277-330 with the RED_BLACK_GS, RESIDUAL, RESTRICT and PROLONG shaders): one
V(2,2) cycle from a zero iterate, 40 coarse sweeps, on the divergence of a
random velocity, equal to round-off -- so the cycle counts the model gives
for relaxation schedules and initial pressures are the reference cycle's.
"""
from __future__ import annotations

import importlib.util

import numpy as np
import pytest

from conftest import ROOT


def _model():
    spec = importlib.util.spec_from_file_location("vcycle_model", ROOT / "fluid-sim_gb300" / "vcycle_model.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("n,relax", [(64, 1.0), (64, 1.2), (128, 1.2)])
def test_model_vcycle_equals_reference_restatement(O, n, relax):
    M = _model()
    rng = np.random.default_rng(n)
    u, v = rng.standard_normal(n * n), rng.standard_normal(n * n)
    r = O.RefGpuSolver(n=n, pressure_solver="multigrid", pressure_iterations=1, precision="f64")
    r.set_relax(relax)
    r.upload_velocity(u, v)
    r.stage("divergence", 0.01)
    d = r.read_divergence().reshape(n, n)
    r.stage("pressure", 0.01)
    p = r.read_pressure().reshape(n, n)
    pm = M.vcycle(d.copy(), (2 * np.pi / n) ** 2, relax=relax, pre=2, post=2, coarse=40)
    assert np.abs(p).max() > 1e-3
    assert np.abs(pm - p).max() <= 1e-13 * np.abs(p).max()


def test_model_tolerance_loop_converges():
    """The refinement loop of the model on a smooth mean-free right-hand side:
    every cycle cuts max|r| by at least 10x at relaxation 1.2."""
    M = _model()
    n = 128
    x = np.arange(n) * 2 * np.pi / n
    d = np.sin(3 * x)[:, None] * np.cos(5 * x)[None, :] + 0.3 * np.cos(x)[:, None] * np.sin(11 * x)[None, :]
    cycles, hist, _ = M.solve(d, tol=1e-9)
    assert hist[-1] <= 1e-9 and cycles <= 10
    assert all(b <= 0.1 * a for a, b in zip(hist, hist[1:]))
