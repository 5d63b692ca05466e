"""ctypes binding of the CPU oracle (oracle/fsoracle_*.c).

TEST INFRASTRUCTURE ONLY.  This module is the checker for the CUDA path: it is
imported by tests/, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg
of ``bench.py``, and by nothing that ships.

``CpuSolver`` restates fluid-sim's f64 ``FluidSolver`` (src/cpu/solver.js);
``RefGpuSolver`` restates the reference GPU algorithm (src/gpu/solver.js with
the WGSL kernels of src/gpu/shaders.js and src/gpu/multigrid.js) in float
(``precision="f32"``) or double (``precision="f64"``) arithmetic.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libfsoracle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compile the oracle with its Makefile (gcc, a few seconds)."""
    srcs = [HERE / f for f in ("fsoracle_cpu.c", "fsoracle_wgsl.c", "fsoracle.h", "fsoracle_wgsl_impl.h")]
    if force or not LIB_PATH.exists() or any(s.stat().st_mtime > LIB_PATH.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("lx", C.c_double), ("ly", C.c_double),
                ("dx", C.c_double), ("dy", C.c_double)]


class Params(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("lx", C.c_double), ("ly", C.c_double),
                ("nu", C.c_double), ("advection", C.c_int), ("explicit_diffusion", C.c_int),
                ("projection", C.c_int), ("proj_tol", C.c_double), ("proj_max_iter", C.c_int),
                ("mask_width", C.c_double), ("coupling_passes", C.c_int)]


class StepOpts(C.Structure):
    _fields_ = [("advect_dye", C.c_int), ("drag", C.c_double), ("gravity", C.c_double),
                ("band_forcing", C.c_int), ("band_kf", C.c_double), ("band_width", C.c_double),
                ("band_amp", C.c_double), ("band_seed", C.c_uint32), ("band_kind", C.c_int),
                ("band_key", C.c_uint64), ("band_counter", C.c_uint32)]


class Channel(C.Structure):
    _fields_ = [("wall_y", C.c_double), ("wall_half", C.c_double), ("fringe_x", C.c_double),
                ("fringe_half", C.c_double), ("fringe_ramp", C.c_double), ("inflow_u", C.c_double)]


class Disk(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("r", C.c_double), ("density", C.c_double),
                ("vx", C.c_double), ("vy", C.c_double), ("omega", C.c_double),
                ("fixed", C.c_int), ("added_mass_correction", C.c_int),
                ("mass", C.c_double), ("inertia", C.c_double), ("added_mass", C.c_double),
                ("effective_mass", C.c_double), ("effective_inertia", C.c_double),
                ("force", C.c_double * 2), ("torque", C.c_double), ("last_impulse", C.c_double * 2)]


class Mode(C.Structure):
    _fields_ = [("kx", C.c_double), ("ky", C.c_double), ("phase", C.c_double)]


D = C.c_double
DP = C.POINTER(C.c_double)
I = C.c_int
VP = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        sig = {
            "fso_grid_init": (None, [C.POINTER(Grid), I, I, D, D]),
            "fso_wrap": (I, [I, I]),
            "fso_lcg_fill": (C.c_uint32, [C.c_uint32, C.c_int64, DP]),
            "fso_lcg_fill_uv": (C.c_uint32, [C.c_uint32, C.c_int64, DP, DP]),
            "fso_bilerp": (D, [DP, I, I, D, D]),
            "fso_sample_u": (D, [C.POINTER(Grid), DP, D, D]),
            "fso_sample_v": (D, [C.POINTER(Grid), DP, D, D]),
            "fso_sample_p": (D, [C.POINTER(Grid), DP, D, D]),
            "fso_divergence": (None, [C.POINTER(Grid), DP, DP, DP]),
            "fso_subtract_gradient": (None, [C.POINTER(Grid), DP, DP, DP, D]),
            "fso_vorticity_center": (None, [C.POINTER(Grid), DP, DP, DP]),
            "fso_velocity_at_centers": (None, [C.POINTER(Grid), DP, DP, DP, DP]),
            "fso_kinetic_energy": (D, [C.POINTER(Grid), DP, DP]),
            "fso_enstrophy": (D, [C.POINTER(Grid), DP, DP]),
            "fso_max_divergence": (D, [C.POINTER(Grid), DP, DP]),
            "fso_l2_divergence": (D, [C.POINTER(Grid), DP, DP]),
            "fso_cfl": (D, [C.POINTER(Grid), DP, DP, D]),
            "fso_tg_init": (None, [C.POINTER(Grid), DP, DP, D, D]),
            "fso_tg_velocity_error": (D, [C.POINTER(Grid), DP, DP, D, D]),
            "fso_rel_l2": (D, [DP, DP, C.c_int64]),
            "fso_gaussian_scalar": (D, [D] * 8),
            "fso_fft_inplace": (None, [DP, DP, I, I]),
            "fso_dft_naive": (None, [DP, DP, DP, DP, I, I]),
            "fso_fft2": (I, [DP, I, I, DP, DP]),
            "fso_ifft2": (I, [DP, DP, I, I, DP, DP]),
            "fso_energy_spectrum": (I, [DP, DP, I, I, DP, C.POINTER(C.c_int32)]),
            "fso_advect_velocity": (None, [C.POINTER(Grid), I, DP, DP, DP, DP, D]),
            "fso_advect_scalar": (None, [C.POINTER(Grid), I, DP, DP, DP, DP, D]),
            "fso_laplacian": (None, [C.POINTER(Grid), DP, DP]),
            "fso_poisson_cg": (I, [C.POINTER(Grid), DP, DP, D, I, DP, DP, I]),
            "fso_poisson_jacobi": (I, [C.POINTER(Grid), DP, DP, I, D, DP, DP, I]),
            "fso_poisson_fft": (I, [C.POINTER(Grid), DP, DP]),
            "fso_poisson_residual": (D, [C.POINTER(Grid), DP, DP]),
            "fso_project": (I, [C.POINTER(Grid), DP, DP, DP, D, I, DP]),
            "fso_diffuse": (I, [C.POINTER(Grid), DP, DP, D, D, I, D, DP]),
            "fso_linear_drag": (None, [DP, DP, C.c_int64, D, D]),
            "fso_band_forcing": (None, [C.POINTER(Grid), DP, DP, D, D, D, C.c_uint32, D]),
            "fso_channel_forcing": (None, [C.POINTER(Grid), DP, DP, C.POINTER(Channel), D]),
            "fso_set_channel": (None, [VP, C.POINTER(Channel)]),
            "fso_gauss_band_forcing": (None, [C.POINTER(Grid), DP, DP, D, D, D, C.c_uint64, C.c_uint32, D]),
            "fso_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
            "fso_forcing_modes": (None, [C.POINTER(Grid), DP, DP, C.POINTER(Mode), I, D, D, D, D]),
            "fso_disk_init": (None, [C.POINTER(Disk), D, D, D, D, D, D, D, I, I]),
            "fso_disk_mask": (D, [C.POINTER(Disk), D, D, D, D, D]),
            "fso_apply_coupling": (None, [C.POINTER(Grid), DP, DP, C.POINTER(Disk), I, D, D, I, DP]),
            "fso_params_default": (None, [C.POINTER(Params)]),
            "fso_create": (VP, [C.POINTER(Params), C.POINTER(I)]),
            "fso_destroy": (None, [VP]),
            "fso_field": (DP, [VP, I]),
            "fso_add_solid": (I, [VP, C.POINTER(Disk)]),
            "fso_get_solid": (C.POINTER(Disk), [VP, I]),
            "fso_set_modes": (None, [VP, C.POINTER(Mode), I, D, D, D]),
            "fso_step_opts_default": (None, [C.POINTER(StepOpts)]),
            "fso_step": (None, [VP, D, C.POINTER(StepOpts)]),
            "fso_time": (D, [VP]),
            "fso_steps": (I, [VP]),
            "fso_last_iterations": (I, [VP]),
            "fso_last_residual": (D, [VP]),
            "fso_is_blown_up": (I, [VP]),
            "fso_set_threads": (None, [I]),
        }
        for suf in ("f32", "f64"):
            sig.update({
                f"fsw_{suf}_create": (VP, [I, I, D, D, D, I, I, I, D]),
                f"fsw_{suf}_destroy": (None, [VP]),
                f"fsw_{suf}_upload_velocity": (None, [VP, DP, DP]),
                f"fsw_{suf}_read_velocity": (None, [VP, DP, DP]),
                f"fsw_{suf}_read_pressure": (None, [VP, DP]),
                f"fsw_{suf}_read_divergence": (None, [VP, DP]),
                f"fsw_{suf}_read_impulse": (None, [VP, DP, DP, DP]),
                f"fsw_{suf}_set_forcing": (None, [VP, DP, I, D, D, D]),
                f"fsw_{suf}_set_solid": (None, [VP, I, D, D, D, D, D, D]),
                f"fsw_{suf}_set_iterations": (None, [VP, I]),
                f"fsw_{suf}_set_relax": (None, [VP, D]),
                f"fsw_{suf}_step": (None, [VP, D]),
                f"fsw_{suf}_stage": (None, [VP, I, D]),
                f"fsw_{suf}_poisson_residual_after": (D, [VP, I, D]),
                f"fsw_{suf}_max_divergence": (D, [VP]),
                f"fsw_{suf}_time": (D, [VP]),
            })
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(DP)


def grid(nx: int, ny: int | None = None, lx: float = 2 * math.pi, ly: float = 2 * math.pi) -> Grid:
    g = Grid()
    lib().fso_grid_init(C.byref(g), nx, nx if ny is None else ny, lx, ly)
    return g


def zeros(g: Grid) -> np.ndarray:
    return np.zeros(g.nx * g.ny, dtype=np.float64)


# ----------------------------------------------------------------- fixtures
def lcg(seed: int, n: int) -> np.ndarray:
    """The reference's inline LCG (test/core.test.js:94-98), bit-exact."""
    out = np.empty(n, dtype=np.float64)
    lib().fso_lcg_fill(seed, n, _p(out))
    return out


def lcg_uv(seed: int, n: int):
    """u[i], v[i] drawn alternately, as tools/gputest.html:116 does."""
    u = np.empty(n, dtype=np.float64)
    v = np.empty(n, dtype=np.float64)
    lib().fso_lcg_fill_uv(seed, n, _p(u), _p(v))
    return u, v


def tg_init(g: Grid, t: float = 0.0, nu: float = 0.0):
    u, v = zeros(g), zeros(g)
    lib().fso_tg_init(C.byref(g), _p(u), _p(v), t, nu)
    return u, v


def tg_error(g: Grid, u, v, t, nu) -> float:
    return lib().fso_tg_velocity_error(C.byref(g), _p(u), _p(v), t, nu)


def rel_l2(a, exact) -> float:
    a = np.ascontiguousarray(a, dtype=np.float64)
    exact = np.ascontiguousarray(exact, dtype=np.float64)
    return lib().fso_rel_l2(_p(a), _p(exact), a.size)


def fill(g: Grid, f, where: str = "p") -> np.ndarray:
    i = np.arange(g.nx)
    j = np.arange(g.ny)
    if where == "u":
        x, y = i * g.dx, (j + 0.5) * g.dy
    elif where == "v":
        x, y = (i + 0.5) * g.dx, j * g.dy
    else:
        x, y = (i + 0.5) * g.dx, (j + 0.5) * g.dy
    X, Y = np.meshgrid(x, y)
    return np.ascontiguousarray(f(X, Y), dtype=np.float64).ravel()


# -------------------------------------------------------------- operators
def divergence(g, u, v):
    out = zeros(g)
    lib().fso_divergence(C.byref(g), _p(u), _p(v), _p(out))
    return out


def subtract_gradient(g, u, v, p, scale=1.0):
    lib().fso_subtract_gradient(C.byref(g), _p(u), _p(v), _p(p), scale)


def laplacian(g, p):
    out = zeros(g)
    lib().fso_laplacian(C.byref(g), _p(p), _p(out))
    return out


def kinetic_energy(g, u, v):
    return lib().fso_kinetic_energy(C.byref(g), _p(u), _p(v))


def enstrophy(g, u, v):
    return lib().fso_enstrophy(C.byref(g), _p(u), _p(v))


def max_divergence(g, u, v):
    return lib().fso_max_divergence(C.byref(g), _p(u), _p(v))


def advect_velocity(g, u, v, dt, scheme="semi-lagrangian"):
    ou, ov = zeros(g), zeros(g)
    lib().fso_advect_velocity(C.byref(g), 1 if scheme == "maccormack" else 0, _p(u), _p(v), _p(ou), _p(ov), dt)
    return ou, ov


def advect_scalar(g, u, v, q, dt, scheme="semi-lagrangian"):
    out = zeros(g)
    lib().fso_advect_scalar(C.byref(g), 1 if scheme == "maccormack" else 0, _p(u), _p(v), _p(q), _p(out), dt)
    return out


def diffuse(g, field, nu, dt, explicit=False, tol=1e-12):
    out = zeros(g)
    it = lib().fso_diffuse(C.byref(g), _p(field), _p(out), nu, dt, 1 if explicit else 0, tol, None)
    return out, it


def poisson_cg(g, rhs, tol=1e-10, max_iter=2000, p=None):
    p = zeros(g) if p is None else p
    res = C.c_double()
    hist = np.zeros(max_iter + 1)
    it = lib().fso_poisson_cg(C.byref(g), _p(rhs), _p(p), tol, max_iter, C.byref(res), _p(hist), hist.size)
    return p, it, res.value


def poisson_jacobi(g, rhs, iterations=80, omega=1.0):
    p = zeros(g)
    res = C.c_double()
    hist = np.zeros(max(iterations, 1))
    lib().fso_poisson_jacobi(C.byref(g), _p(rhs), _p(p), iterations, omega, C.byref(res), _p(hist), hist.size)
    return p, res.value, hist[:iterations]


def poisson_fft(g, rhs):
    p = zeros(g)
    if lib().fso_poisson_fft(C.byref(g), _p(rhs), _p(p)) < 0:
        raise ValueError("fft projection needs power-of-two dimensions")
    return p


def poisson_residual(g, p, rhs):
    return lib().fso_poisson_residual(C.byref(g), _p(p), _p(rhs))


def project(g, u, v, tol=1e-10, max_iter=2000):
    p = zeros(g)
    res = C.c_double()
    it = lib().fso_project(C.byref(g), _p(u), _p(v), _p(p), tol, max_iter, C.byref(res))
    return p, it, res.value


def fft2(field, nx, ny):
    re = np.zeros(nx * ny)
    im = np.zeros(nx * ny)
    if lib().fso_fft2(_p(np.ascontiguousarray(field, dtype=np.float64)), nx, ny, _p(re), _p(im)) < 0:
        raise ValueError("fft2 needs power-of-two dimensions")
    return re, im


def energy_spectrum(cu, cv, nx, ny):
    kmax = min(nx, ny) // 2
    E = np.zeros(kmax + 1)
    counts = np.zeros(kmax + 1, dtype=np.int32)
    lib().fso_energy_spectrum(_p(cu), _p(cv), nx, ny, _p(E), counts.ctypes.data_as(C.POINTER(C.c_int32)))
    return E, counts


def velocity_at_centers(g, u, v):
    cu, cv = zeros(g), zeros(g)
    lib().fso_velocity_at_centers(C.byref(g), _p(u), _p(v), _p(cu), _p(cv))
    return cu, cv


def disk(x, y, r, density=1.0, vx=0.0, vy=0.0, omega=0.0, fixed=False, added_mass=False) -> Disk:
    d = Disk()
    lib().fso_disk_init(C.byref(d), x, y, r, density, vx, vy, omega, int(fixed), int(added_mass))
    return d


def apply_coupling(g, u, v, disks, dt, mask_width=1.5, passes=1):
    arr = (Disk * len(disks))(*disks)
    imp = np.zeros(2)
    lib().fso_apply_coupling(C.byref(g), _p(u), _p(v), arr, len(disks), dt, mask_width, passes, _p(imp))
    for k in range(len(disks)):
        disks[k] = arr[k]
    return imp


def philox4x32_10(ctr, key):
    """Philox4x32-10 of four 32-bit counter words and two key words."""
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    out = (C.c_uint32 * 4)()
    lib().fso_philox4x32_10(c, k, out)
    return tuple(out)


def band_forcing(g: Grid, u, v, kf, width, amp, seed, dt):
    """bandForcing (src/cpu/solver.js:179-217) applied to u, v in place."""
    lib().fso_band_forcing(C.byref(g), _p(u), _p(v), kf, width, amp, seed, dt)


def gauss_band_forcing(g: Grid, u, v, kf, width, amp, key, counter, dt):
    """The Philox Gaussian lattice band forcing applied to u, v in place."""
    lib().fso_gauss_band_forcing(C.byref(g), _p(u), _p(v), kf, width, amp, key, counter, dt)


def channel_forcing(g: Grid, u, v, channel: dict, mask_width: float = 1.5):
    """The channel's fringe and wall forcing applied to u, v in place."""
    lib().fso_channel_forcing(C.byref(g), _p(u), _p(v), C.byref(Channel(**channel)), mask_width)


def set_threads(n: int) -> None:
    lib().fso_set_threads(int(n))


# ---------------------------------------------------------------- solvers
ADVECTION = {"semi-lagrangian": 0, "maccormack": 1}
PROJECTION = {"cg": 0, "fft": 1, "jacobi": 2}


class CpuSolver:
    """f64 restatement of FluidSolver (src/cpu/solver.js:241-418)."""

    def __init__(self, n=64, nx=None, ny=None, lx=2 * math.pi, ly=2 * math.pi, nu=0.01,
                 advection="semi-lagrangian", explicit_diffusion=False, proj_tol=1e-10,
                 proj_max_iter=2000, projection="cg", mask_width=1.5, coupling_passes=2):
        if advection not in ADVECTION:
            raise ValueError(f"unknown advection scheme {advection}")
        if projection not in PROJECTION:
            raise ValueError(f"unknown projection {projection}")
        p = Params()
        lib().fso_params_default(C.byref(p))
        p.nx = nx or n
        p.ny = ny or n
        p.lx, p.ly, p.nu = lx, ly, nu
        p.advection = ADVECTION[advection]
        p.explicit_diffusion = int(explicit_diffusion)
        p.projection = PROJECTION[projection]
        p.proj_tol, p.proj_max_iter = proj_tol, proj_max_iter
        p.mask_width, p.coupling_passes = mask_width, coupling_passes
        err = C.c_int()
        self._h = lib().fso_create(C.byref(p), C.byref(err))
        if not self._h:
            raise ValueError(f"invalid solver parameters (code {err.value})")
        self.g = grid(p.nx, p.ny, lx, ly)
        self.n = p.nx * p.ny

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().fso_destroy(h)
            self._h = None

    def _view(self, which):
        ptr = lib().fso_field(self._h, which)
        return np.ctypeslib.as_array(ptr, shape=(self.n,))

    @property
    def u(self):
        return self._view(0)

    @property
    def v(self):
        return self._view(1)

    @property
    def p(self):
        return self._view(2)

    @property
    def dye(self):
        return self._view(3)

    def init_tg(self, nu=0.0, t=0.0):
        u, v = tg_init(self.g, t, nu)
        self.u[:] = u
        self.v[:] = v
        return self

    def add_solid(self, d: Disk) -> int:
        return lib().fso_add_solid(self._h, C.byref(d))

    def solid(self, i) -> Disk:
        return lib().fso_get_solid(self._h, i).contents

    def set_forcing(self, modes, amplitude=1.0, drag=0.0, phase_drift=0.3):
        arr = (Mode * len(modes))(*[Mode(m[0], m[1], m[2]) for m in modes])
        lib().fso_set_modes(self._h, arr, len(modes), amplitude, drag, phase_drift)

    def set_channel(self, channel):
        """channel: dict of fso_channel fields, or None to remove it"""
        lib().fso_set_channel(self._h, C.byref(Channel(**channel)) if channel else None)

    def step(self, dt, advect_dye=True, drag=0.0, gravity=0.0, band=None, gauss_band=None):
        """band = (kf, width, amp, seed): bandForcing as opts.force;
        gauss_band = (kf, width, amp, key, counter): the Philox Gaussian band"""
        o = StepOpts()
        lib().fso_step_opts_default(C.byref(o))
        o.advect_dye = int(advect_dye)
        o.drag = drag
        o.gravity = gravity
        if band is not None:
            o.band_forcing = 1
            o.band_kf, o.band_width, o.band_amp, o.band_seed = band
        if gauss_band is not None:
            o.band_forcing = 1
            o.band_kind = 1
            o.band_kf, o.band_width, o.band_amp, o.band_key, o.band_counter = gauss_band
        lib().fso_step(self._h, dt, C.byref(o))
        return self

    @property
    def t(self):
        return lib().fso_time(self._h)

    @property
    def steps(self):
        return lib().fso_steps(self._h)

    @property
    def last_iterations(self):
        return lib().fso_last_iterations(self._h)

    def kinetic_energy(self):
        return kinetic_energy(self.g, self.u, self.v)

    def enstrophy(self):
        return enstrophy(self.g, self.u, self.v)

    def max_divergence(self):
        return max_divergence(self.g, self.u, self.v)

    def is_blown_up(self):
        return bool(lib().fso_is_blown_up(self._h))


SOLVERS = {"jacobi": 0, "red-black": 1, "multigrid": 2}
STAGES = {"advect": 0, "diffuse": 1, "forcing": 2, "solid": 3, "divergence": 4, "pressure": 5,
          "subtract_gradient": 6, "project": 7}


class RefGpuSolver:
    """Restatement of GPUFluidSolver's algorithm (src/gpu/solver.js) in f32 or f64."""

    def __init__(self, n=256, nx=None, ny=None, lx=2 * math.pi, ly=2 * math.pi, nu=0.0,
                 advection="maccormack", pressure_solver="jacobi", pressure_iterations=40,
                 solid_mask_width=1.5, precision="f32"):
        self.suf = precision
        self.nx, self.ny = nx or n, ny or n
        self.n = self.nx * self.ny
        self.dx = lx / self.nx
        # the reference GPU solver silently treats unknown names as SL / Jacobi
        adv = 1 if advection == "maccormack" else 0
        sol = SOLVERS.get(pressure_solver, 0)
        self._h = self._f("create")(self.nx, self.ny, lx, ly, nu, adv, sol, pressure_iterations,
                                    solid_mask_width)

    def _f(self, name):
        return getattr(lib(), f"fsw_{self.suf}_{name}")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._f("destroy")(h)
            self._h = None

    def upload_velocity(self, u, v):
        self._f("upload_velocity")(self._h, _p(np.ascontiguousarray(u, dtype=np.float64)),
                                   _p(np.ascontiguousarray(v, dtype=np.float64)))

    def read_velocity(self):
        u, v = np.zeros(self.n), np.zeros(self.n)
        self._f("read_velocity")(self._h, _p(u), _p(v))
        return u, v

    def read_pressure(self):
        p = np.zeros(self.n)
        self._f("read_pressure")(self._h, _p(p))
        return p

    def read_divergence(self):
        d = np.zeros(self.n)
        self._f("read_divergence")(self._h, _p(d))
        return d

    def read_impulse(self):
        a, b, c = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n)
        self._f("read_impulse")(self._h, _p(a), _p(b), _p(c))
        return a, b, c

    def set_iterations(self, it):
        self._f("set_iterations")(self._h, it)

    def set_relax(self, relax):
        """param_a of every Jacobi / red-black sweep (the reference passes 1.0)"""
        self._f("set_relax")(self._h, relax)

    def set_forcing(self, modes, amplitude=1.0, drag=0.0, phase_drift=0.3):
        flat = np.ascontiguousarray(np.asarray(modes, dtype=np.float64).reshape(-1))
        self._f("set_forcing")(self._h, _p(flat), len(modes), amplitude, drag, phase_drift)

    def set_solid(self, x, y, r, vx=0.0, vy=0.0, omega=0.0, on=True):
        self._f("set_solid")(self._h, int(on), x, y, vx, vy, omega, r)

    def step(self, dt):
        self._f("step")(self._h, dt)

    def stage(self, name, dt):
        self._f("stage")(self._h, STAGES[name], dt)

    def poisson_residual_after(self, iterations, dt=0.01):
        return self._f("poisson_residual_after")(self._h, iterations, dt)

    def max_divergence(self):
        return self._f("max_divergence")(self._h)

    @property
    def t(self):
        return self._f("time")(self._h)
