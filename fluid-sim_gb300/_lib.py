"""Build and bind libfluidcuda.so (the CUDA sm_103a library behind include/fluid.h).

The library is compiled in-tree with nvcc into ``fluid-sim_gb300/_build/``; the
package never falls back to a CPU path: if the library is missing, or no CUDA
device is present, calls raise ``FluidError``.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB_PATH = BUILD / "libfluidcuda.so"
HEADER = ROOT / "include" / "fluid.h"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]

# status codes (include/fluid.h fs_status)
FS_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
          4: "pressure tolerance not met", 5: "non-finite residual", 6: "unsupported", 7: "no CUDA device"}


class FluidError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise FileNotFoundError("nvcc not found")


def sources():
    return sorted(CSRC.glob("*.cu"))


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every .cu for sm_103a (one -gencode) in parallel and link the .so."""
    BUILD.mkdir(exist_ok=True)
    deps = list(CSRC.glob("*.cuh")) + [HEADER]
    newest_dep = max(p.stat().st_mtime for p in deps)
    objs = []
    jobs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_dep):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not LIB_PATH.exists():
        run([nvcc(), *ARCH, "-shared", "-o", str(LIB_PATH), *map(str, objs), "-lcudart"])
    return LIB_PATH


# ------------------------------------------------------------------ structs
class Params(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("lx", C.c_double), ("ly", C.c_double),
                ("nu", C.c_double), ("confinement", C.c_double), ("advection", C.c_int32),
                ("solid_mask_width", C.c_double), ("pressure_solver", C.c_int32),
                ("pressure_iterations", C.c_int32), ("precision", C.c_int32),
                ("pressure_tol", C.c_double), ("max_cycles", C.c_int32), ("mg_pre_smooth", C.c_int32),
                ("mg_post_smooth", C.c_int32), ("mg_coarse_sweeps", C.c_int32), ("mg_min_size", C.c_int32),
                ("warm_start", C.c_int32), ("device", C.c_int32), ("kernel_variant", C.c_int32),
                ("dye_fade", C.c_double),
                ("relax", C.c_double), ("pressure_tol_relative", C.c_int32), ("mg_first_pre", C.c_int32),
                ("mg_first_post", C.c_int32)]


class Mode(C.Structure):
    _fields_ = [("kx", C.c_double), ("ky", C.c_double), ("phase", C.c_double)]


class Band(C.Structure):
    _fields_ = [("kind", C.c_int32), ("kf", C.c_double), ("width", C.c_double), ("amplitude", C.c_double),
                ("seed", C.c_uint64), ("drag", C.c_double)]


class Channel(C.Structure):
    _fields_ = [("wall_y", C.c_double), ("wall_half", C.c_double), ("fringe_x", C.c_double),
                ("fringe_half", C.c_double), ("fringe_ramp", C.c_double), ("inflow_u", C.c_double)]


class Disk(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("r", C.c_double), ("vx", C.c_double),
                ("vy", C.c_double), ("omega", C.c_double)]


class StepStats(C.Structure):
    _fields_ = [("cycles", C.c_int32), ("converged", C.c_int32), ("residual_max", C.c_double),
                ("residual_initial", C.c_double)]


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_int32), ("total_ms", C.c_double),
                ("bytes", C.c_double)]


VP = C.c_void_p
I = C.c_int
D = C.c_double

# every entry point include/fluid.h declares, with its ctypes signature
SIGNATURES = {
    "fs_params_default": (None, [C.POINTER(Params)]),
    "fs_create": (I, [C.POINTER(Params), C.POINTER(VP)]),
    "fs_destroy": (None, [VP]),
    "fs_last_error": (C.c_char_p, [VP]),
    "fs_status_string": (C.c_char_p, [I]),
    "fs_get_params": (I, [VP, C.POINTER(Params)]),
    "fs_upload_velocity": (I, [VP, VP, VP, I]),
    "fs_read_velocity": (I, [VP, VP, VP, I]),
    "fs_read_field": (I, [VP, I, VP, I]),
    "fs_upload_field": (I, [VP, I, VP, I]),
    "fs_set_forcing": (I, [VP, C.POINTER(Mode), I, D, D, D]),
    "fs_set_solids": (I, [VP, C.POINTER(Disk), I]),
    "fs_set_band_forcing": (I, [VP, C.POINTER(Band)]),
    "fs_set_channel": (I, [VP, C.POINTER(Channel)]),
    "fs_solid_impulse": (I, [VP, C.POINTER(C.c_double), I]),
    "fs_step": (I, [VP, D]),
    "fs_advance": (I, [VP, D, I]),
    "fs_sync": (I, [VP]),
    "fs_last_stats": (I, [VP, C.POINTER(StepStats)]),
    "fs_get_time": (I, [VP, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "fs_run_stage": (I, [VP, I, D]),
    "fs_max_divergence": (I, [VP, C.POINTER(C.c_double)]),
    "fs_poisson_residual_after": (I, [VP, I, D, C.POINTER(C.c_double)]),
    "fs_time_steps": (I, [VP, D, I, C.POINTER(C.c_double)]),
    "fs_profile_step": (I, [VP, D, I, C.POINTER(KernelTime), I, C.POINTER(I)]),
    "fs_launch_count": (C.c_int64, [VP]),
    "fs_host_alloc": (VP, [C.c_size_t]),
    "fs_host_free": (None, [VP]),
    "fs_max_divergence_noalloc": (I, [VP, VP, C.c_int32, C.c_int32, D, D, VP, VP]),
    "fs_conv3x3_bf16": (I, [VP, VP, VP, VP, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                            VP, VP]),
    "fs_tc_gemm_check": (I, [VP, VP, VP, C.c_int32, C.c_int32, VP, VP]),
    "fs_guess_create": (I, [C.c_int32, C.c_uint64, C.POINTER(VP)]),
    "fs_guess_destroy": (None, [VP]),
    "fs_guess_num_params": (C.c_int64, [VP]),
    "fs_guess_get_params": (I, [VP, VP, C.c_int64]),
    "fs_guess_set_params": (I, [VP, VP, C.c_int64]),
    "fs_guess_predict": (I, [VP, VP, VP, C.c_int32, C.c_int32, C.c_int32, VP]),
    "fs_guess_loss_grad": (I, [VP, VP, VP, VP, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_double), VP]),
    "fs_guess_train_step": (I, [VP, VP, VP, VP, C.c_int32, C.c_int32, C.c_int32, C.c_float,
                                C.POINTER(C.c_double)]),
    "fs_guess_set_loss": (I, [VP, D, D]),
    "fs_guess_sync": (I, [VP]),
    "fs_guess_launch_count": (C.c_int64, [VP]),
    "fs_set_guess": (I, [VP, VP, C.c_int32]),
    "fs_upload_dye": (I, [VP, VP]),
    "fs_read_dye": (I, [VP, VP]),
    "fs_render": (I, [VP, C.c_int32, D, VP]),
    "fs_set_mg_sweeps": (I, [VP, C.c_int32, C.c_int32]),
    "fs_total_cycles": (I, [VP, C.POINTER(C.c_int64)]),
    "fs_convergence_record": (I, [VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(D)]),
    "fs_autotune": (I, [VP, D, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(D)]),
    "fs_set_mg_tiles": (I, [VP, C.POINTER(C.c_int32), C.c_int32]),
    "fs_get_mg_tiles": (I, [VP, C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32)]),
    "fs_autotune_tiles": (I, [VP, D, C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32),
                              C.POINTER(D)]),
    "fs_diagnose": (I, [VP, VP]),
    "fs_energy_spectrum": (I, [VP, VP, VP, C.c_int32, C.POINTER(C.c_int32), VP]),
    "fs_batch_create": (I, [C.POINTER(Params), C.c_int32, C.POINTER(VP)]),
    "fs_batch_destroy": (None, [VP]),
    "fs_batch_size": (C.c_int32, [VP]),
    "fs_batch_member": (VP, [VP, C.c_int32]),
    "fs_batch_last_error": (C.c_char_p, [VP]),
    "fs_batch_step": (I, [VP, C.POINTER(D)]),
    "fs_batch_sync": (I, [VP]),
    "fs_batch_time_steps": (I, [VP, C.POINTER(D), C.c_int32, C.POINTER(D)]),
    "fs_batch_launch_count": (C.c_int64, [VP]),
    "fs_batch_autotune_tiles": (I, [VP, C.POINTER(D), C.c_int32, C.POINTER(D)]),
    "fs_batch_autotune": (I, [VP, C.POINTER(D), C.c_int32, C.POINTER(D)]),
    "fs_dump_pair": (I, [VP, C.c_int32, VP, VP, VP]),
    "fs_dump_pair_device": (I, [VP, C.c_int32, VP, VP, VP]),
    "fs_write_pair_file": (I, [C.c_char_p, C.c_int32, C.c_int32, D, VP, VP, VP]),
    "fs_read_pair_file": (I, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(D), VP, VP, VP]),
}

_lib = None


def load(path: Path | None = None):
    """Load the built library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FluidError(2, f"{p} is missing: run __graft_entry__.build() (the CUDA path has no fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status: int, handle=None) -> None:
    if status != FS_OK:
        msg = load().fs_last_error(handle)
        raise FluidError(status, msg.decode() if msg else "")


def declared_symbols() -> list[str]:
    """Function names declared FS_API in include/fluid.h."""
    import re

    text = HEADER.read_text()
    return re.findall(r"FS_API\s+[\w\s\*]+?\b(fs_\w+)\s*\(", text)
