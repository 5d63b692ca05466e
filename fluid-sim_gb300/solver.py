"""Host-side mirror of fluid-sim's GPU backend API (src/gpu/solver.js).

``GPUFluidSolver`` keeps the reference class's constructor options, method
names and argument meaning (camelCase aliases included), and drives the CUDA
library through its C ABI.  Reads return numpy arrays; every GPU failure
raises ``FluidError`` -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Iterable, Sequence

import numpy as np

from . import _lib as L

ADVECTION = {"semi-lagrangian": 0, "maccormack": 1}
PRESSURE = {"jacobi": 0, "red-black": 1, "multigrid": 2}
PRECISION = {"f32": 0, "mixed": 1}
FIELDS = {"u": 0, "v": 1, "pressure": 2, "divergence": 3, "impulse_x": 4, "impulse_y": 5, "impulse_torque": 6}
STAGES = {"advect": 0, "diffuse": 1, "forcing": 2, "solid": 3, "divergence": 4, "pressure": 5,
          "subtract_gradient": 6, "project": 7}


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def make_params(n: int = 256, nx: int | None = None, ny: int | None = None, lx: float = 2 * math.pi,
                ly: float = 2 * math.pi, nu: float = 0.0, confinement: float = 0.0, advection: str = "maccormack",
                solid_mask_width: float = 1.5, pressure_solver: str = "jacobi", pressure_iterations: int = 40,
                precision: str = "f32", pressure_tol: float = 0.0, max_cycles: int = 50, mg_pre_smooth: int = 2,
                mg_post_smooth: int = 2, mg_coarse_sweeps: int = 40, mg_min_size: int = 8,
                warm_start: bool = False, device: int = 0, kernel_variant: int = 0, dye_fade: float = 0.0,
                relax: float = 1.0, pressure_tol_relative: bool = False, mg_first_pre: int = -1,
                mg_first_post: int = -1, **camel) -> "L.Params":
    """fs_params from the reference's option names (camelCase accepted);
    unknown names are rejected (the reference silently defaults)."""
    solid_mask_width = camel.pop("solidMaskWidth", solid_mask_width)
    pressure_solver = camel.pop("pressureSolver", pressure_solver)
    pressure_iterations = camel.pop("pressureIterations", pressure_iterations)
    dye_fade = camel.pop("dyeFade", dye_fade)
    if camel:
        raise TypeError(f"unknown options {sorted(camel)}")
    lib = L.load()
    p = L.Params()
    lib.fs_params_default(C.byref(p))
    p.nx = nx or n
    p.ny = ny or n
    p.lx, p.ly, p.nu, p.confinement = lx, ly, nu, confinement
    if advection not in ADVECTION:
        raise L.FluidError(1, f"unknown advection scheme {advection!r}")
    if pressure_solver not in PRESSURE:
        raise L.FluidError(1, f"unknown pressure solver {pressure_solver!r}")
    if precision not in PRECISION:
        raise L.FluidError(1, f"unknown precision {precision!r}")
    p.advection = ADVECTION[advection]
    p.solid_mask_width = solid_mask_width
    p.pressure_solver = PRESSURE[pressure_solver]
    p.pressure_iterations = pressure_iterations
    p.precision = PRECISION[precision]
    p.pressure_tol = pressure_tol
    p.max_cycles = max_cycles
    p.mg_pre_smooth, p.mg_post_smooth = mg_pre_smooth, mg_post_smooth
    p.mg_coarse_sweeps, p.mg_min_size = mg_coarse_sweeps, mg_min_size
    p.warm_start = int(bool(warm_start))
    p.device = device
    p.kernel_variant = kernel_variant
    p.dye_fade = dye_fade
    p.relax = relax
    p.pressure_tol_relative = int(bool(pressure_tol_relative))
    p.mg_first_pre, p.mg_first_post = mg_first_pre, mg_first_post
    return p


class GPUFluidSolver:
    """new GPUFluidSolver(device, {n, nx, ny, lx, ly, nu, confinement, advection,
    solidMaskWidth, pressureSolver, pressureIterations}) -- src/gpu/solver.js:65-98.

    Extra options: ``precision`` ("f32" | "mixed"), ``pressure_tol`` (> 0 runs
    cycles until max|div u| <= tol), ``max_cycles``, ``warm_start``, the
    multigrid sweep counts, ``relax`` (the relaxation factor of every sweep,
    param_a of the reference's smoother shaders; 1.0 as the reference) and
    ``device`` (CUDA ordinal).
    """

    def __init__(self, n: int = 256, nx: int | None = None, ny: int | None = None, lx: float = 2 * math.pi,
                 ly: float = 2 * math.pi, nu: float = 0.0, confinement: float = 0.0,
                 advection: str = "maccormack", solid_mask_width: float = 1.5,
                 pressure_solver: str = "jacobi", pressure_iterations: int = 40, precision: str = "f32",
                 pressure_tol: float = 0.0, max_cycles: int = 50, mg_pre_smooth: int = 2,
                 mg_post_smooth: int = 2, mg_coarse_sweeps: int = 40, mg_min_size: int = 8,
                 warm_start: bool = False, device: int = 0, kernel_variant: int = 0, dye_fade: float = 0.0,
                 relax: float = 1.0, **camel):
        p = make_params(n=n, nx=nx, ny=ny, lx=lx, ly=ly, nu=nu, confinement=confinement, advection=advection,
                        solid_mask_width=solid_mask_width, pressure_solver=pressure_solver,
                        pressure_iterations=pressure_iterations, precision=precision, pressure_tol=pressure_tol,
                        max_cycles=max_cycles, mg_pre_smooth=mg_pre_smooth, mg_post_smooth=mg_post_smooth,
                        mg_coarse_sweeps=mg_coarse_sweeps, mg_min_size=mg_min_size, warm_start=warm_start,
                        device=device, kernel_variant=kernel_variant, dye_fade=dye_fade, relax=relax,
                        **camel)
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.fs_create(C.byref(p), C.byref(h)), None)
        self._adopt(lib, h, p, owned=True)

    def _adopt(self, lib, h, p, owned: bool) -> None:
        self._h = h
        self._lib = lib
        self._owned = owned
        self.params = p
        self.nx, self.ny = p.nx, p.ny
        self.n = p.nx * p.ny
        self.lx, self.ly = p.lx, p.ly
        self.dx, self.dy = p.lx / p.nx, p.ly / p.ny
        self.nu = p.nu
        self.advection = {v: k for k, v in ADVECTION.items()}[p.advection]
        self.pressure_solver = {v: k for k, v in PRESSURE.items()}[p.pressure_solver]
        self.pressure_iterations = p.pressure_iterations
        self.precision = {v: k for k, v in PRECISION.items()}[p.precision]
        self.solid = None

    @classmethod
    def _member(cls, lib, handle, keep_alive):
        """A solver owned by a batch (fs_batch_member): same methods, not destroyed here."""
        self = cls.__new__(cls)
        p = L.Params()
        h = C.c_void_p(handle)
        L.check(lib.fs_get_params(h, C.byref(p)), None)
        self._adopt(lib, h, p, owned=False)
        self._batch = keep_alive
        return self

    # ------------------------------------------------------------ lifecycle
    def destroy(self) -> None:
        """destroy() (solver.js:898-911); a batch member is freed with its batch"""
        if getattr(self, "_h", None):
            if getattr(self, "_owned", True):
                self._lib.fs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def _chk(self, st: int) -> None:
        L.check(st, self._h)

    # ---------------------------------------------------------------- upload
    def upload_velocity(self, u: np.ndarray, v: np.ndarray) -> None:
        """uploadVelocity(u, v) (solver.js:301-315), f64 or f32 arrays of n*n."""
        dt = np.float64 if np.asarray(u).dtype == np.float64 else np.float32
        u = np.ascontiguousarray(u, dtype=dt).reshape(-1)
        v = np.ascontiguousarray(v, dtype=dt).reshape(-1)
        if u.size != self.n or v.size != self.n:
            raise L.FluidError(1, f"expected {self.n} values per component")
        self._chk(self._lib.fs_upload_velocity(self._h, _ptr(u), _ptr(v), 1 if dt is np.float64 else 0))

    uploadVelocity = upload_velocity

    def read_velocity(self, dtype=np.float64):
        """readVelocity() (solver.js:356-362) -> (u, v)"""
        u = np.empty(self.n, dtype=dtype)
        v = np.empty(self.n, dtype=dtype)
        self._chk(self._lib.fs_read_velocity(self._h, _ptr(u), _ptr(v), 1 if dtype == np.float64 else 0))
        return u, v

    readVelocity = read_velocity

    def read_field(self, field: str, dtype=np.float64) -> np.ndarray:
        """readTexture for pressure / divergence / impulse fields (solver.js:336-353)"""
        out = np.empty(self.n, dtype=dtype)
        self._chk(self._lib.fs_read_field(self._h, FIELDS[field], _ptr(out), 1 if dtype == np.float64 else 0))
        return out

    def upload_pressure(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1)
        self._chk(self._lib.fs_upload_field(self._h, FIELDS["pressure"], _ptr(p), 1))

    # ------------------------------------------------------- forces, solids
    def set_forcing(self, modes: Sequence | None, amplitude: float = 1.0, drag: float = 0.0,
                    phase_drift: float = 0.3) -> None:
        """setForcing(modes, {amplitude, drag, phaseDrift}) (solver.js:370-385)"""
        modes = list(modes or [])
        arr = (L.Mode * max(1, len(modes)))()
        for k, m in enumerate(modes):
            if isinstance(m, dict):
                arr[k] = L.Mode(m["kx"], m["ky"], m["phase"])
            else:
                arr[k] = L.Mode(*m)
        self._chk(self._lib.fs_set_forcing(self._h, arr, len(modes), amplitude, drag, phase_drift))

    setForcing = set_forcing

    BAND_KINDS = {"reference": 0, "gaussian": 1}

    def set_band_forcing(self, kind: str | None = "reference", kf: float = 28.0, width: float = 2.0,
                         amplitude: float = 0.4, seed: int = 1, drag: float = 0.0) -> None:
        """bandForcing(g, u, v, {kf, width, amp, seed++}) + linearDrag(alpha)
        every step (src/cpu/solver.js:179-237; defaults are bandForcing's).
        kind "reference": its 24 LCG modes; "gaussian": every lattice mode in
        the band with a Philox complex Gaussian amplitude; None removes it."""
        if kind is None:
            self._chk(self._lib.fs_set_band_forcing(self._h, None))
            return
        if kind not in self.BAND_KINDS:
            raise L.FluidError(1, f"unknown band forcing kind {kind!r}")
        b = L.Band(self.BAND_KINDS[kind], kf, width, amplitude, seed, drag)
        self._chk(self._lib.fs_set_band_forcing(self._h, C.byref(b)))

    def set_channel(self, channel: dict | None) -> None:
        """Channel walls and inflow fringe (fs_set_channel): a dict with
        wall_y, wall_half, fringe_x, fringe_half, fringe_ramp, inflow_u, or
        None to remove them."""
        if channel is None:
            self._chk(self._lib.fs_set_channel(self._h, None))
            return
        c = L.Channel(**channel)
        self._chk(self._lib.fs_set_channel(self._h, C.byref(c)))

    def set_solids(self, disks: Iterable) -> None:
        """setSolid(disk) generalised to several disks (solver.js:425-438)"""
        disks = list(disks or [])
        arr = (L.Disk * max(1, len(disks)))()
        for k, d in enumerate(disks):
            if isinstance(d, dict):
                arr[k] = L.Disk(d["x"], d["y"], d["r"], d.get("vx", 0.0), d.get("vy", 0.0), d.get("omega", 0.0))
            else:
                arr[k] = L.Disk(*d)
        self._chk(self._lib.fs_set_solids(self._h, arr, len(disks)))
        self.solid = disks[0] if disks else None

    def set_solid(self, disk) -> None:
        self.set_solids([disk] if disk is not None else [])

    setSolid = set_solid

    def solid_impulse(self) -> np.ndarray:
        """per-disk (fx, fy, torque) impulse of the last coupling pass, summed on the device"""
        k = len(self.solid and [self.solid] or [])
        out = np.zeros(3 * 64)
        self._chk(self._lib.fs_solid_impulse(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), 64))
        return out.reshape(64, 3)

    # ------------------------------------------------------------------ step
    def step(self, dt: float) -> None:
        """step(dt) (solver.js:518-591)"""
        self._chk(self._lib.fs_step(self._h, dt))

    def advance(self, dt: float, nsteps: int) -> None:
        self._chk(self._lib.fs_advance(self._h, dt, nsteps))

    def sync(self) -> None:
        self._chk(self._lib.fs_sync(self._h))

    def run_stage(self, stage: str, dt: float) -> None:
        self._chk(self._lib.fs_run_stage(self._h, STAGES[stage], dt))

    def last_stats(self) -> dict:
        st = L.StepStats()
        self._chk(self._lib.fs_last_stats(self._h, C.byref(st)))
        return {"cycles": st.cycles, "converged": bool(st.converged), "residual_max": st.residual_max,
                "residual_initial": st.residual_initial}

    @property
    def t(self) -> float:
        t = C.c_double()
        self._lib.fs_get_time(self._h, C.byref(t), None)
        return t.value

    @property
    def steps(self) -> int:
        n = C.c_int64()
        self._lib.fs_get_time(self._h, None, C.byref(n))
        return n.value

    # ----------------------------------------------------------- diagnostics
    def max_divergence(self) -> float:
        """maxDivergence() (solver.js:835-850)"""
        out = C.c_double()
        self._chk(self._lib.fs_max_divergence(self._h, C.byref(out)))
        return out.value

    maxDivergence = max_divergence

    def poisson_residual_after(self, iterations: int, dt: float = 0.01) -> float:
        """poissonResidualAfter(iterations, dt) (solver.js:857-896)"""
        out = C.c_double()
        self._chk(self._lib.fs_poisson_residual_after(self._h, iterations, dt, C.byref(out)))
        return out.value

    poissonResidualAfter = poisson_residual_after

    # ----------------------------------------------------------- measurement
    def time_steps(self, dt: float, nsteps: int) -> float:
        ms = C.c_double()
        self._chk(self._lib.fs_time_steps(self._h, dt, nsteps, C.byref(ms)))
        return ms.value

    def profile_step(self, dt: float, nsteps: int = 1) -> list[dict]:
        cap = 64
        arr = (L.KernelTime * cap)()
        cnt = C.c_int()
        self._chk(self._lib.fs_profile_step(self._h, dt, nsteps, arr, cap, C.byref(cnt)))
        return [{"name": arr[k].name.decode(), "launches": arr[k].launches, "total_ms": arr[k].total_ms,
                 "bytes": arr[k].bytes} for k in range(min(cap, cnt.value))]

    def launch_count(self) -> int:
        return int(self._lib.fs_launch_count(self._h))

    # ------------------------------------------------------------------ dye
    def upload_dye(self, rgba) -> None:
        """uploadDye(rgba) (solver.js:317-323): f32 RGBA per cell, [ny, nx, 4] or flat"""
        a = np.ascontiguousarray(rgba, dtype=np.float32)
        if a.size != 4 * self.n:
            raise ValueError(f"dye needs {4 * self.n} floats")
        self._chk(self._lib.fs_upload_dye(self._h, _ptr(a)))

    def read_dye(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx, 4), np.float32)
        self._chk(self._lib.fs_read_dye(self._h, _ptr(out)))
        return out

    def total_cycles(self) -> int:
        """refinement cycles run by all projections so far (device counter)"""
        c = C.c_int64()
        self._chk(self._lib.fs_total_cycles(self._h, C.byref(c)))
        return c.value

    def convergence_record(self) -> dict:
        """every tolerance-loop projection since creation: how many, how many
        missed pressure_tol, and the worst final max|div u| among them"""
        n, f, w = C.c_int64(), C.c_int64(), C.c_double()
        self._chk(self._lib.fs_convergence_record(self._h, C.byref(n), C.byref(f), C.byref(w)))
        return {"steps": n.value, "failed_steps": f.value, "worst_max_div": w.value}

    def set_mg_sweeps(self, pre: int, post: int) -> None:
        self._chk(self._lib.fs_set_mg_sweeps(self._h, pre, post))
        self.params.mg_pre_smooth, self.params.mg_post_smooth = pre, post

    def autotune(self, dt: float, nsteps: int = 5) -> dict:
        """time every (pre, post) sweep pair from the current state, keep the fastest"""
        pre, post, ms = C.c_int32(), C.c_int32(), C.c_double()
        self._chk(self._lib.fs_autotune(self._h, dt, nsteps, C.byref(pre), C.byref(post), C.byref(ms)))
        self.params.mg_pre_smooth, self.params.mg_post_smooth = pre.value, post.value
        return {"pre": pre.value, "post": post.value, "ms_per_step": ms.value}

    def set_mg_tiles(self, tiles) -> None:
        """tile side (16, 32, 64; 0 = built-in rule) of each multigrid tile level"""
        t = (C.c_int32 * 16)(*list(tiles))
        self._chk(self._lib.fs_set_mg_tiles(self._h, t, len(tiles)))

    def mg_tiles(self) -> list:
        """tile sides in use, one per multigrid tile level"""
        t, n = (C.c_int32 * 16)(), C.c_int32()
        self._chk(self._lib.fs_get_mg_tiles(self._h, t, 16, C.byref(n)))
        return list(t[: n.value])

    def autotune_tiles(self, dt: float, nsteps: int = 5) -> dict:
        """time 64, 32 and 16 cell tiles per multigrid level from the current
        state (greedy, level by level), keep the fastest; state restored"""
        t, n, ms = (C.c_int32 * 16)(), C.c_int32(), C.c_double()
        self._chk(self._lib.fs_autotune_tiles(self._h, dt, nsteps, t, 16, C.byref(n), C.byref(ms)))
        return {"tiles": self.mg_tiles(), "ms_per_step": ms.value}

    def render(self, mode: str = "vorticity", exposure: float = 1.0) -> np.ndarray:
        """RENDER arithmetic (shaders.js:677-768) into an [ny, nx, 4] f32 array"""
        out = np.empty((self.ny, self.nx, 4), np.float32)
        self._chk(self._lib.fs_render(self._h, {"vorticity": 0, "speed": 1}[mode], float(exposure), _ptr(out)))
        return out

    @staticmethod
    def save_ppm(path, rgba: np.ndarray) -> None:
        """Write a render as a binary PPM (Reinhard tone map, gamma 2.2, row 0 at the bottom)."""
        c = np.asarray(rgba, np.float64)[..., :3]
        c = (c / (1.0 + c)) ** (1 / 2.2)
        img = np.clip(np.round(c[::-1] * 255), 0, 255).astype(np.uint8)
        with open(path, "wb") as f:
            f.write(f"P6 {img.shape[1]} {img.shape[0]} 255\n".encode() + img.tobytes())

    # ------------------------------------------------------- diagnostics
    def diagnostics(self) -> dict:
        """kinetic energy, enstrophy, max and L2 divergence of the state (device reductions)"""
        out = (C.c_double * 4)()
        self._chk(self._lib.fs_diagnose(self._h, out))
        return {"kinetic_energy": out[0], "enstrophy": out[1], "max_divergence": out[2], "l2_divergence": out[3]}

    def kinetic_energy(self) -> float:
        return self.diagnostics()["kinetic_energy"]

    def enstrophy(self) -> float:
        return self.diagnostics()["enstrophy"]

    def energy_spectrum(self):
        """(k, E, counts, (sum E, kinetic energy)) -- shell-averaged spectrum on the device"""
        kmax = min(self.nx, self.ny) // 2
        E = np.zeros(kmax + 1)
        cnt = np.zeros(kmax + 1, np.int32)
        km = C.c_int32()
        pv = (C.c_double * 2)()
        self._chk(self._lib.fs_energy_spectrum(self._h, _ptr(E), _ptr(cnt), kmax + 1, C.byref(km), pv))
        return np.arange(kmax + 1), E, cnt, (pv[0], pv[1])

    # ------------------------------------------------ learned pressure guess
    def set_guess(self, guess, factor: int = 2) -> None:
        """Seed every projection with a PressureGuess running at 1/factor of
        the grid resolution (None detaches it); the cycles still run to
        pressure_tol."""
        self._chk(self._lib.fs_set_guess(self._h, guess.handle if guess is not None else None, factor))
        self._guess = guess  # keep it alive while attached

    def dump_pair(self, factor: int = 1):
        """(div, mask, p) of the last projection averaged over factor x factor
        cells, f32 [ny/factor, nx/factor] each, and their grid spacing."""
        ny, nx = self.ny // factor, self.nx // factor
        d = np.empty((ny, nx), np.float32)
        m = np.empty_like(d)
        p = np.empty_like(d)
        self._chk(self._lib.fs_dump_pair(self._h, factor, _ptr(d), _ptr(m), _ptr(p)))
        return d, m, p, self.dx * factor

    def dump_pair_device(self, factor: int, d_div: int, d_mask: int, d_p: int) -> float:
        """The same pair into device buffers (addresses of f32 arrays of
        (ny/factor) * (nx/factor)), enqueued on the solver's stream; returns
        the pair's grid spacing.  Call sync() before another stream reads them."""
        self._chk(self._lib.fs_dump_pair_device(self._h, factor, C.c_void_p(d_div), C.c_void_p(d_mask),
                                                C.c_void_p(d_p)))
        return self.dx * factor


class GPUFluidBatch:
    """Many independent solvers of uneven sizes advanced by one CUDA graph
    launch per step (fs_batch_*).  ``configs`` is a list of GPUFluidSolver
    option dicts; ``members[i]`` are GPUFluidSolver views owned by the batch
    (upload, read back, set solids, read stats as usual)."""

    def __init__(self, configs: Sequence[dict]):
        lib = L.load()
        ps = (L.Params * len(configs))()
        for i, cfg in enumerate(configs):
            ps[i] = make_params(**cfg)
        h = C.c_void_p()
        st = lib.fs_batch_create(ps, len(configs), C.byref(h))
        if st != L.FS_OK:
            raise L.FluidError(st, lib.fs_batch_last_error(None).decode())
        self._h = h
        self._lib = lib
        self.members = [GPUFluidSolver._member(lib, lib.fs_batch_member(h, i), self) for i in range(len(configs))]

    def _chk(self, st: int) -> None:
        if st != L.FS_OK:
            raise L.FluidError(st, self._lib.fs_batch_last_error(self._h).decode())

    def _dts(self, dt):
        n = len(self.members)
        d = np.broadcast_to(np.asarray(dt, np.float64), (n,)).copy()
        return d, d.ctypes.data_as(C.POINTER(C.c_double))

    def step(self, dt) -> None:
        """one step of every member (dt scalar or one per member)"""
        d, ptr = self._dts(dt)
        self._chk(self._lib.fs_batch_step(self._h, ptr))
        self._last = d

    def sync(self) -> None:
        self._chk(self._lib.fs_batch_sync(self._h))

    def time_steps(self, dt, nsteps: int) -> float:
        d, ptr = self._dts(dt)
        ms = C.c_double()
        self._chk(self._lib.fs_batch_time_steps(self._h, ptr, nsteps, C.byref(ms)))
        return ms.value

    def launch_count(self) -> int:
        return int(self._lib.fs_batch_launch_count(self._h))

    def autotune(self, dt, nsteps: int = 3) -> dict:
        """Sweep counts per size class, each candidate timed as whole batch
        steps from one saved state (fs_batch_autotune, state restored).
        Returns {(nx, ny): (pre, post)}."""
        d, arr = self._dts(dt)
        ms = C.c_double()
        self._chk(self._lib.fs_batch_autotune(self._h, arr, nsteps, C.byref(ms)))
        picks = {}
        for m in self.members:
            p = L.Params()
            m._chk(self._lib.fs_get_params(m._h, C.byref(p)))
            m.params.mg_pre_smooth, m.params.mg_post_smooth = p.mg_pre_smooth, p.mg_post_smooth
            picks.setdefault((m.nx, m.ny), (p.mg_pre_smooth, p.mg_post_smooth))
        return picks

    def autotune_tiles(self, dt, nsteps: int = 3) -> dict:
        """Tile sides per size class and multigrid level, each candidate timed
        as whole batch steps from one saved state (fs_batch_autotune_tiles).
        Returns {(nx, ny): tiles} and the tuned ms per batch step."""
        d, arr = self._dts(dt)
        ms = C.c_double()
        self._chk(self._lib.fs_batch_autotune_tiles(self._h, arr, nsteps, C.byref(ms)))
        picks = {}
        for m in self.members:
            picks.setdefault((m.nx, m.ny), m.mg_tiles())
        return {"tiles": picks, "ms_per_step": ms.value}

    def destroy(self) -> None:
        if getattr(self, "_h", None):
            for m in self.members:
                m._h = None
            self._lib.fs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
