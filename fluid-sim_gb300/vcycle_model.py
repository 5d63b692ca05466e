"""A numpy model of the solver's multigrid projection, for design questions.

It restates, in f64 and whole-array form, what the tolerance loop of the
mixed-precision solve does on the GPU (fs_multigrid.cu, fs_pressure.cu):
each iteration forms the residual r = d - lap p of the pressure, runs one
V-cycle on r from a zero iterate -- red-black Gauss-Seidel with
over-relaxation w (cur + w (gs - cur), the smoother of the reference's
RED_BLACK_GS, src/gpu/shaders.js:340-372), the residual's 4-cell restriction
and the cell-centred bilinear prolongation of src/gpu/multigrid.js:48-131,
periodic, levels halving down to an 8^2 level smoothed by a fixed number of
sweeps -- and adds the correction to p, until max|r| <= tol.  Run on a
right-hand side dumped from the GPU solver it reproduces the GPU's final
residuals to about three digits (the GPU cycle works in f32 on the residual,
the model in f64), so it answers "how many cycles would this change need"
without a GPU: relaxation factors and schedules, pre/post sweep counts, coarse
sweeps, and how good an initial pressure would have to be to save cycles.

    python vcycle_model.py dump  OUT_DIR  [--steps 20,100,200]   (GPU: writes rhs_<k>.npy)
    python vcycle_model.py cycles RHS.npy [--relax 1.2 --pre 2 --post 2 --coarse 8]
    python vcycle_model.py guess  RHS.npy                         (cycles left from disturbed exact pressures)

This is an analysis tool: nothing in the solver imports it.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def sum4(x):
    return np.roll(x, 1, 0) + np.roll(x, -1, 0) + np.roll(x, 1, 1) + np.roll(x, -1, 1)


_MASKS: dict = {}


def _colour(n, c):
    if (n, c) not in _MASKS:
        i = np.arange(n)
        _MASKS[(n, c)] = ((i[:, None] + i[None, :]) & 1) == c
    return _MASKS[(n, c)]


def smooth(x, rhs, h2, sweeps, w):
    """red-black sweeps in place: colour 0, then colour 1, per sweep"""
    for _ in range(sweeps):
        for c in (0, 1):
            m = _colour(x.shape[0], c)
            gs = (sum4(x) - h2 * rhs) * 0.25
            x[m] += w * (gs[m] - x[m])


def residual(x, rhs, h2):
    return rhs - (sum4(x) - 4.0 * x) / h2


def restrict(r):
    return 0.25 * (r[0::2, 0::2] + r[0::2, 1::2] + r[1::2, 0::2] + r[1::2, 1::2])


def prolong(e):
    """cell-centred bilinear: fine cell 2a takes 3/4 of coarse a and 1/4 of
    a - 1, fine cell 2a + 1 3/4 of a and 1/4 of a + 1, in each direction"""
    n = e.shape[0]
    t = np.empty((n, 2 * n))
    t[:, 0::2] = 0.75 * e + 0.25 * np.roll(e, 1, 1)
    t[:, 1::2] = 0.75 * e + 0.25 * np.roll(e, -1, 1)
    f = np.empty((2 * n, 2 * n))
    f[0::2, :] = 0.75 * t + 0.25 * np.roll(t, 1, 0)
    f[1::2, :] = 0.75 * t + 0.25 * np.roll(t, -1, 0)
    return f


def vcycle(rhs, h2, relax=1.2, pre=2, post=2, coarse=8, nmin=8):
    x = np.zeros_like(rhs)
    if rhs.shape[0] <= nmin:
        smooth(x, rhs, h2, coarse, relax)
        return x
    smooth(x, rhs, h2, pre, relax)
    e = vcycle(restrict(residual(x, rhs, h2)), 4.0 * h2, relax, pre, post, coarse, nmin)
    x += prolong(e)
    smooth(x, rhs, h2, post, relax)
    return x


def solve(d, p0=None, tol=1e-6, max_cycles=12, **cycle):
    """the tolerance loop: cycles until max|d - lap p| <= tol; returns
    (cycles, history of max|r|, p).  The grid spans [0, 2 pi]^2."""
    n = d.shape[0]
    h2 = (2.0 * np.pi / n) ** 2
    p = np.zeros_like(d) if p0 is None else p0.copy()
    r = residual(p, d, h2)
    hist = [float(np.abs(r).max())]
    while hist[-1] > tol and len(hist) <= max_cycles:
        p += vcycle(r, h2, **cycle)
        r = residual(p, d, h2)
        hist.append(float(np.abs(r).max()))
    return len(hist) - 1, hist, p


def load_rhs(path):
    d = np.load(path).astype(np.float64)
    n = int(round(np.sqrt(d.size)))
    d = d.reshape(n, n)
    return d - d.mean()


def guess_table(d, seed=0):
    """cycles left to tol 1e-6 from the exact pressure disturbed by smooth
    (|k| <~ 16) or grid-scale error of a given size relative to max|p|, and
    from the exact pressure rounded to bf16 and to f32"""
    n = d.shape[0]
    _, _, p = solve(d, tol=0.0, max_cycles=12)
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((n, n))
    k = np.fft.fftfreq(n) * n
    smooth_err = np.real(np.fft.ifft2(np.fft.fft2(white) * np.exp(-(k[:, None] ** 2 + k[None, :] ** 2) / 512.0)))
    pm = np.abs(p).max()
    rows = [("zero", solve(d)[0], float(np.abs(d).max()))]
    for name, err in (("smooth", smooth_err), ("grid-scale", white)):
        err = err / np.abs(err).max()
        for rel in (1e-1, 1e-2, 1e-3, 1e-4, 1e-5):
            c, hist, _ = solve(d, p0=p + rel * pm * err)
            rows.append((f"{name} {rel:.0e}", c, hist[0]))
    b = p.astype(np.float32).view(np.uint32)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).view(np.float32).astype(np.float64)
    for name, q in (("bf16", b), ("f32", p.astype(np.float32).astype(np.float64))):
        c, hist, _ = solve(d, p0=q)
        rows.append((f"exact rounded to {name}", c, hist[0]))
    return rows


def dump(out_dir, steps):
    """step the bench's 2048^2 channel workload on the GPU and write the
    projection's right-hand side (the divergence field) after the given steps"""
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench  # the workload and the solver settings of the benchmark

    pkg = bench._package()
    u0, v0, disks, dt, ch = bench.make_workload(bench.N, bench.SEED)
    s = bench.make_solver(pkg, bench.N, 0)
    s.upload_velocity(u0, v0)
    s.set_channel(ch)
    s.set_solids(disks)
    for k in range(1, max(steps) + 1):
        s.step(dt)
        if k in steps:
            np.save(os.path.join(out_dir, f"rhs_{k}.npy"), s.read_field("divergence").astype(np.float32))
            st = s.last_stats()
            print(k, "cycles", st["cycles"], "residual", st["residual_initial"], "->", st["residual_max"])
    s.destroy()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("dump")
    a.add_argument("out_dir")
    a.add_argument("--steps", default="20,100,200")
    a = sub.add_parser("cycles")
    a.add_argument("rhs")
    a.add_argument("--relax", type=float, default=1.2)
    a.add_argument("--pre", type=int, default=2)
    a.add_argument("--post", type=int, default=2)
    a.add_argument("--coarse", type=int, default=8)
    a.add_argument("--tol", type=float, default=1e-6)
    a = sub.add_parser("guess")
    a.add_argument("rhs")
    args = ap.parse_args(argv)
    if args.cmd == "dump":
        dump(args.out_dir, sorted(int(x) for x in args.steps.split(",")))
    elif args.cmd == "cycles":
        c, hist, _ = solve(load_rhs(args.rhs), tol=args.tol, relax=args.relax, pre=args.pre, post=args.post,
                           coarse=args.coarse)
        q = (hist[-1] / hist[0]) ** (1.0 / max(c, 1))
        print(f"cycles {c}, max|r| {hist[0]:.3g} -> {hist[-1]:.3g}, factor per cycle {q:.4f}")
    else:
        for name, c, r0 in guess_table(load_rhs(args.rhs)):
            print(f"{name:28s} initial max|r| {r0:10.3g}  cycles {c}")


if __name__ == "__main__":
    main()
