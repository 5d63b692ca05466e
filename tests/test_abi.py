"""The C-ABI library builds, loads and exports every symbol include/fluid.h
declares; argument validation that needs no GPU.  CPU-only."""
from __future__ import annotations

import ctypes as C
import subprocess

import pytest


@pytest.fixture(scope="module")
def lib(fs):
    fs.build()
    return fs.load()


def test_every_declared_symbol_is_exported(fs, lib):
    from fluid_sim_gb300 import _lib as L

    declared = L.declared_symbols()
    assert len(declared) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", str(L.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    # and nothing beyond the ABI leaks out of the library
    extra = [s for s in exported if s.startswith("fs_") and s not in declared]
    assert not extra, extra
    for name in declared:
        assert name in L.SIGNATURES, f"{name} has no ctypes signature"


def test_params_default_matches_reference_defaults(lib):
    from fluid_sim_gb300 import _lib as L

    p = L.Params()
    lib.fs_params_default(C.byref(p))
    # GPUFluidSolver constructor defaults, src/gpu/solver.js:65-72
    assert (p.nx, p.ny) == (256, 256)
    assert p.nu == 0.0 and p.confinement == 0.0
    assert p.advection == 1  # maccormack
    assert p.solid_mask_width == 1.5
    assert p.pressure_solver == 0 and p.pressure_iterations == 40  # jacobi, 40
    # Multigrid(solver, {preSmooth: 2, postSmooth: 2, coarseSweeps: 40}), minSize 8
    assert (p.mg_pre_smooth, p.mg_post_smooth, p.mg_coarse_sweeps, p.mg_min_size) == (2, 2, 40, 8)
    # every V-cycle smooths the finest level like the others, as the reference's do
    assert (p.mg_first_pre, p.mg_first_post) == (-1, -1)
    assert p.relax == 1.0 and p.pressure_tol_relative == 0


def test_invalid_parameters_fail_before_touching_a_device(lib):
    from fluid_sim_gb300 import _lib as L

    def create(**kw):
        p = L.Params()
        lib.fs_params_default(C.byref(p))
        for k, v in kw.items():
            setattr(p, k, v)
        h = C.c_void_p()
        st = lib.fs_create(C.byref(p), C.byref(h))
        return st, lib.fs_last_error(None).decode()

    assert create(advection=7)[0] == 1
    assert create(pressure_solver=9)[0] == 1
    assert create(precision=3)[0] == 1
    assert create(nx=1)[0] == 1
    st, msg = create(confinement=0.5)
    assert st == 6 and "confinement" in msg
    assert create(pressure_solver=2, nx=64, ny=32)[0] == 1  # multigrid needs a square grid
    assert create(mg_first_pre=3)[0] == 1  # more than the cycle's mg_pre_smooth
    assert create(mg_first_post=-2)[0] == 1
    st, msg = create(mg_first_pre=0, kernel_variant=1)
    assert st == 6 and "fused" in msg
    assert lib.fs_status_string(4) == b"pressure tolerance not met"


def test_null_handle_is_rejected(lib):
    assert lib.fs_step(None, 0.01) == 1
    assert lib.fs_sync(None) == 1
    assert lib.fs_launch_count(None) == 0
