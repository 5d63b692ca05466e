"""fs_max_divergence_noalloc: the allocation-free entry point.

Callers that cannot allocate device memory while they run (a host that owns
the GPU through its own memory pool, a frame loop that must not call
cudaMalloc because it can synchronise the device) pass device buffers they
already hold; the reduction's scratch is a static device array the library
reserves for itself.  This test calls it
through the C ABI twice in a row, on two different fields, and checks each
result against the solver's own fs_max_divergence on the same field, within
the 1e-6 relative tolerance the f32 kernels are held to.  It allocates its own
device buffers with the CUDA runtime -- the entry point itself allocates
nothing.  The file name sorts last so that a stop-at-first-failure run has
already run every other test.
"""
from __future__ import annotations

import ctypes as C
import ctypes.util
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so",
                 ctypes.util.find_library("cudart")):
        if not name:
            continue
        try:
            rt = C.CDLL(name)
        except OSError:
            continue
        rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        rt.cudaFree.argtypes = [C.c_void_p]
        rt.cudaStreamCreateWithFlags.argtypes = [C.POINTER(C.c_void_p), C.c_uint]
        rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
        rt.cudaStreamDestroy.argtypes = [C.c_void_p]
        return rt
    pytest.skip("CUDA runtime library not found")


H2D, D2H = 1, 2


def _to_device(rt, a: np.ndarray) -> C.c_void_p:
    p = C.c_void_p()
    assert rt.cudaMalloc(C.byref(p), a.nbytes) == 0
    assert rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, H2D) == 0
    return p


@pytest.fixture(scope="module")
def G(fs):
    fs.build()
    fs.load()
    return fs


def test_noalloc_max_divergence_matches_solver_twice(G, O):
    lib = G.load()
    rt = _cudart()
    nx, ny = 200, 150  # partial 32x8 blocks at both edges
    lx = ly = 2 * math.pi
    out = C.c_void_p()
    assert rt.cudaMalloc(C.byref(out), 8) == 0
    results = []
    for seed in (991, 4242):
        a, b = O.lcg_uv(seed, nx * ny)
        u = np.ascontiguousarray(a, dtype=np.float32)
        v = np.ascontiguousarray(b, dtype=np.float32)
        s = G.GPUFluidSolver(nx=nx, ny=ny, lx=lx, ly=ly)
        s.upload_velocity(u, v)
        expected = s.max_divergence()
        s.destroy()
        du, dv = _to_device(rt, u), _to_device(rt, v)
        st = lib.fs_max_divergence_noalloc(du, dv, nx, ny, lx, ly, out, None)
        assert st == 0, lib.fs_last_error(None)
        got = np.zeros(1)
        assert rt.cudaMemcpy(got.ctypes.data, out, 8, D2H) == 0
        rt.cudaFree(du)
        rt.cudaFree(dv)
        assert got[0] == pytest.approx(expected, rel=1e-6)
        results.append(got[0])
    assert results[0] != results[1]  # the second call did not return the first call's maximum
    # beyond the static scratch: rejected with a message, nothing launched
    st = lib.fs_max_divergence_noalloc(out, out, 8192, 8192, lx, ly, out, None)
    assert st == 1
    assert b"static scratch" in lib.fs_last_error(None)
    # a narrow grid taller than 65535 rows of blocks (65536 blocks in all, within
    # the scratch, but above the launch's grid-y limit): rejected the same way
    st = lib.fs_max_divergence_noalloc(out, out, 32, 524288, lx, ly, out, None)
    assert st == 1
    assert b"static scratch" in lib.fs_last_error(None)
    rt.cudaFree(out)


def test_noalloc_back_to_back_on_a_caller_stream(G, O):
    """Two calls enqueued one after the other on a non-blocking stream the
    caller created, with no synchronisation between them, each writing its own
    output slot: the second call's counter reset and block maxima must not mix
    with the first's.  Each result equals fs_max_divergence of its field."""
    lib = G.load()
    rt = _cudart()
    nx, ny = 256, 96
    lx = ly = 2 * math.pi
    stream = C.c_void_p()
    assert rt.cudaStreamCreateWithFlags(C.byref(stream), 1) == 0  # cudaStreamNonBlocking
    out = C.c_void_p()
    assert rt.cudaMalloc(C.byref(out), 16) == 0
    expected, bufs = [], []
    for seed in (17, 23):
        a, b = O.lcg_uv(seed, nx * ny)
        u = np.ascontiguousarray(a * (1 + seed), dtype=np.float32)
        v = np.ascontiguousarray(b, dtype=np.float32)
        s = G.GPUFluidSolver(nx=nx, ny=ny, lx=lx, ly=ly)
        s.upload_velocity(u, v)
        expected.append(s.max_divergence())
        s.destroy()
        bufs.append((_to_device(rt, u), _to_device(rt, v)))
    for k, (du, dv) in enumerate(bufs):
        slot = C.c_void_p(out.value + 8 * k)
        st = lib.fs_max_divergence_noalloc(du, dv, nx, ny, lx, ly, slot, stream)
        assert st == 0, lib.fs_last_error(None)
    assert rt.cudaStreamSynchronize(stream) == 0
    got = np.zeros(2)
    assert rt.cudaMemcpy(got.ctypes.data, out, 16, D2H) == 0
    for du, dv in bufs:
        rt.cudaFree(du)
        rt.cudaFree(dv)
    rt.cudaFree(out)
    rt.cudaStreamDestroy(stream)
    assert got[0] == pytest.approx(expected[0], rel=1e-6)
    assert got[1] == pytest.approx(expected[1], rel=1e-6)
    assert got[0] != got[1]
