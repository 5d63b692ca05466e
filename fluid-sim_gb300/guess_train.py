"""Train the pressure guess on pairs the solver dumps from its own runs, and
measure what it saves.

    python fluid-sim_gb300/guess_train.py --n 2048 --runs 8 --steps 48 \\
        --iters 2000 --out weights/guess_2048.fsguess [--pairs-dir DIR]

1. Pairs: for `runs` fresh workload seeds (disjoint from the benchmark's),
   the solver steps the seeded channel flow with a mixed-precision multigrid
   projection to max|div u| <= tol and, every `every` steps, dumps the
   (divergence, solid mask, pressure) of that projection at half resolution
   (fs_dump_pair, factor 2); optionally each pair is also written as an
   FSPAIR file.  Pairs are normalised (normalize_pair) and kept on the device.
2. Training: Adam on random minibatches, cosine learning-rate decay, loss
   w_p * mean-free pressure MSE + w_r * mean (lap error)^2 (the second term
   is the initial residual of the projection the guess seeds).
3. Evaluation on a held-out seed: V-cycles per step and ms per step with and
   without the guess, and the initial residual max|d - lap p0| of each.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import math
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _package():
    name = "fluid_sim_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, HERE / "__init__.py", submodule_search_locations=[str(HERE)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def make_solver(pkg, n, disks, tol=1e-6, guess=None, factor=2, warm=False):
    s = pkg.GPUFluidSolver(n=n, nu=1e-4, advection="maccormack", pressureSolver="multigrid", pressureIterations=1,
                           precision="mixed", pressure_tol=tol, max_cycles=60, warm_start=warm)
    s.set_solids(disks)
    if guess is not None:
        s.set_guess(guess, factor)
    return s


def dump_pairs(pkg, n, runs, steps, every=2, factor=2, seed0=1000, tol=1e-6, pairs_dir=None):
    """-> device tensors (div_n, mask, p_n) of shape [P, n/factor, n/factor]."""
    import torch

    divs, masks, ps = [], [], []
    for r in range(runs):
        u, v, disks, dt = pkg.workload.make_workload(n, seed0 + r)
        s = make_solver(pkg, n, disks, tol)
        s.upload_velocity(u, v)
        for k in range(steps):
            s.step(dt)
            if k % every:
                continue
            d, m, p, dx = s.dump_pair(factor)
            if pairs_dir is not None:
                pkg.write_pair_file(Path(pairs_dir) / f"pair_{seed0 + r}_{k:04d}.fspair", d, m, p, dx)
            dn, mn, pn, _ = pkg.normalize_pair(d, m, p, dx)
            divs.append(torch.from_numpy(dn).cuda())
            masks.append(torch.from_numpy(mn).cuda())
            ps.append(torch.from_numpy(pn).cuda())
        s.destroy()
    return torch.stack(divs), torch.stack(masks), torch.stack(ps)


def train(guess, data, iters, batch, lr, seed=0, log_every=100):
    import torch

    div, mask, p = data
    gen = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    for it in range(iters):
        idx = torch.randint(0, div.shape[0], (batch,), generator=gen).cuda()
        lr_t = lr * 0.5 * (1 + math.cos(math.pi * it / iters))
        want = it % log_every == 0 or it == iters - 1
        loss = guess.train_step(div[idx], mask[idx], p[idx], max(lr_t, lr * 1e-3), want_loss=want)
        if want:
            hist.append((it, loss))
    return hist


def _initial_residual(s, dt):
    """Run one step and return (cycles, initial residual, final residual)."""
    s.step(dt)
    st = s.last_stats()
    return st["cycles"], st["residual_initial"], st["residual_max"]


def evaluate(pkg, n, guess, factor=2, seed=77, steps=30, tol=1e-6):
    """Cycles per step and ms per step on a held-out seed: zero initial
    pressure (plain, as the reference), the learned guess, and the previous
    step's pressure (warm start, for comparison)."""
    u, v, disks, dt = pkg.workload.make_workload(n, seed)
    out = {}
    for name, g, warm in (("plain", None, False), ("guess", guess, False), ("warm", None, True)):
        s = make_solver(pkg, n, disks, tol, g, factor, warm)
        s.upload_velocity(u, v)
        cyc, r0 = [], []
        for _ in range(steps):
            c, ri, _ = _initial_residual(s, dt)
            cyc.append(c)
            r0.append(ri)
        ms = s.time_steps(dt, steps) / steps
        out[name] = {"cycles_per_step": float(np.mean(cyc)), "initial_residual": float(np.median(r0)),
                     "ms_per_step": ms}
        s.destroy()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--runs", type=int, default=8)
    ap.add_argument("--steps", type=int, default=48)
    ap.add_argument("--every", type=int, default=2)
    ap.add_argument("--factor", type=int, default=2, help="the network runs at 1/factor of the grid")
    ap.add_argument("--iters", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--w-pressure", type=float, default=0.05)
    ap.add_argument("--w-residual", type=float, default=1.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", type=str, default=None, help="weights file (FSGUESS)")
    ap.add_argument("--report", type=str, default=None, help="JSON summary")
    ap.add_argument("--pairs-dir", type=str, default=None)
    ap.add_argument("--eval-steps", type=int, default=30)
    a = ap.parse_args(argv)
    pkg = _package()
    t0 = time.time()
    data = dump_pairs(pkg, a.n, a.runs, a.steps, a.every, a.factor, pairs_dir=a.pairs_dir)
    t1 = time.time()
    g = pkg.PressureGuess(seed=a.seed)
    g.set_loss(a.w_pressure, a.w_residual)
    hist = train(g, data, a.iters, a.batch, a.lr, a.seed)
    g.sync()
    t2 = time.time()
    if a.out:
        Path(a.out).parent.mkdir(parents=True, exist_ok=True)
        g.save(a.out)
    ev = evaluate(pkg, a.n, g, a.factor, steps=a.eval_steps)
    rep = {"n": a.n, "factor": a.factor, "pairs": int(data[0].shape[0]), "net_resolution": int(data[0].shape[-1]),
           "params": g.n_params, "iters": a.iters, "batch": a.batch, "lr": a.lr,
           "loss_weights": [a.w_pressure, a.w_residual], "dump_s": t1 - t0, "train_s": t2 - t1,
           "loss_history": hist, "eval": ev}
    print(json.dumps(rep))
    if a.report:
        Path(a.report).write_text(json.dumps(rep, indent=1))
    return rep


if __name__ == "__main__":
    main()
