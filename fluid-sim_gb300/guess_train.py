"""Train the pressure guess on pairs the solver dumps from its own runs, and
measure what it saves.

    python fluid-sim_gb300/guess_train.py --n 2048 --pairs 20000 --seeds 16 \
        --out weights/guess_2048_f2.fsguess

1. Pairs, streamed: `seeds` fresh seeds of the channel workload (disjoint
   from the benchmark's) are stepped in rotation with the benchmark's
   projection (mixed-precision multigrid to max|div u| <= tol, relaxation
   1.2); after every step the solver writes the (divergence, solid mask,
   pressure) of that projection at 1/factor resolution straight into a ring
   buffer on the device (fs_dump_pair_device), where it is normalised
   (h^2 d / sigma, (p - mean p) / sigma).  `pairs` pairs in all, every one
   distinct; training batches are drawn from the ring.
2. Training: Adam on random minibatches from the ring, cosine learning-rate
   decay, loss w_p * mean-free pressure MSE + w_r * mean (lap error)^2 (the
   second term is the initial residual of the projection the guess seeds).
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


RELAX, COARSE = 1.2, 8  # the benchmark's projection


def make_solver(pkg, n, disks, channel, tol=1e-6, guess=None, factor=2, warm=False):
    s = pkg.GPUFluidSolver(n=n, nu=1e-4, advection="maccormack", pressureSolver="multigrid", pressureIterations=1,
                           precision="mixed", pressure_tol=tol, max_cycles=60, warm_start=warm, relax=RELAX,
                           mg_coarse_sweeps=COARSE)
    s.set_channel(channel)
    s.set_solids(disks)
    if guess is not None:
        s.set_guess(guess, factor)
    return s


def stream_train(pkg, guess, n, pairs, seeds, factor=2, ring=512, batch=4, steps_per_round=4, lr=2e-3,
                 seed0=1000, tol=1e-6, warmup=20, log_every=100):
    """Step `seeds` channel-flow solvers in rotation; every step's pair goes
    into a device ring of `ring` pairs; after each round (one step of every
    seed) `steps_per_round` Adam steps on batches drawn from the filled part
    of the ring.  Returns (loss history, pairs made, train steps)."""
    import torch

    m = n // factor
    div = torch.empty((ring, m, m), device="cuda")
    msk = torch.empty_like(div)
    prs = torch.empty_like(div)
    sols, dts = [], []
    for r in range(seeds):
        u, v, disks, dt, ch = pkg.workload.channel_workload(n, seed0 + r)
        s = make_solver(pkg, n, disks, ch, tol)
        s.upload_velocity(u, v)
        for _ in range(warmup):  # past the start-up transient
            s.step(dt)
        sols.append(s)
        dts.append(dt)
    gen = torch.Generator(device="cpu").manual_seed(0)
    made = it = 0
    rounds = (pairs + seeds - 1) // seeds
    iters = rounds * steps_per_round
    hist = []
    for rnd in range(rounds):
        for s, dt in zip(sols, dts):
            if made >= pairs:
                break
            s.step(dt)
            k = made % ring
            h = s.dump_pair_device(factor, div[k].data_ptr(), msk[k].data_ptr(), prs[k].data_ptr())
            s.sync()
            x = div[k] * (h * h)
            sigma = torch.sqrt(torch.mean(x * x)).clamp_min(1e-30)
            div[k] = x / sigma
            prs[k] = (prs[k] - prs[k].mean()) / sigma
            made += 1
        filled = min(made, ring)
        for _ in range(steps_per_round):
            idx = torch.randint(0, filled, (batch,), generator=gen).cuda()
            lr_t = max(lr * 0.5 * (1 + math.cos(math.pi * it / iters)), lr * 1e-3)
            want = it % log_every == 0 or it == iters - 1
            loss = guess.train_step(div[idx], msk[idx], prs[idx], lr_t, want_loss=want)
            if want:
                hist.append((it, loss))
            it += 1
    for s in sols:
        s.destroy()
    return hist, made, it


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
    """Cycles per step and ms per step on a held-out seed of the channel
    workload: zero initial pressure (plain, as the reference), the learned
    guess, and the previous step's pressure (warm start, for comparison)."""
    u, v, disks, dt, ch = pkg.workload.channel_workload(n, seed)
    out = {}
    for name, g, warm in (("plain", None, False), ("guess", guess, False), ("warm", None, True)):
        s = make_solver(pkg, n, disks, ch, tol, g, factor, warm)
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


def time_train_steps(pkg, res=1024, batch=4, steps=20, warm=3, seed=0):
    """ms per fs_guess_train_step on random inputs of [batch][res][res]
    (the training configuration's shape: 2048^2 grids at factor 2)."""
    import torch

    gen = torch.Generator(device="cuda").manual_seed(seed)
    d = torch.randn(batch, res, res, device="cuda", generator=gen)
    m = (torch.rand(batch, res, res, device="cuda", generator=gen) > 0.9).float()
    t = torch.randn(batch, res, res, device="cuda", generator=gen)
    g = pkg.PressureGuess(seed=seed)
    g.set_loss(0.05, 1.0)
    for _ in range(warm):
        g.train_step(d, m, t, 1e-3, want_loss=False)
    g.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        g.train_step(d, m, t, 1e-3, want_loss=False)
    g.sync()
    return (time.perf_counter() - t0) / max(steps, 1) * 1e3


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--pairs", type=int, default=20000, help="distinct solver-dumped pairs to train on")
    ap.add_argument("--seeds", type=int, default=16, help="channel-flow seeds stepped in rotation")
    ap.add_argument("--ring", type=int, default=512, help="pairs held on the device at once")
    ap.add_argument("--steps-per-round", type=int, default=4, help="Adam steps per round of one pair per seed")
    ap.add_argument("--factor", type=int, default=2, help="the network runs at 1/factor of the grid")
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--w-pressure", type=float, default=0.05)
    ap.add_argument("--w-residual", type=float, default=1.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", type=str, default=None, help="weights file (FSGUESS)")
    ap.add_argument("--report", type=str, default=None, help="JSON summary")
    ap.add_argument("--eval-steps", type=int, default=30)
    ap.add_argument("--time-steps", type=int, default=0,
                    help="only time this many training steps on random 1024^2 batches of 4 and exit")
    a = ap.parse_args(argv)
    pkg = _package()
    if a.time_steps > 0:
        ms = time_train_steps(pkg, steps=a.time_steps)
        print(json.dumps({"train_step_ms": ms, "res": 1024, "batch": 4, "steps": a.time_steps}))
        return {"train_step_ms": ms}
    g = pkg.PressureGuess(seed=a.seed)
    g.set_loss(a.w_pressure, a.w_residual)
    t0 = time.time()
    hist, made, iters = stream_train(pkg, g, a.n, a.pairs, a.seeds, a.factor, a.ring, a.batch, a.steps_per_round,
                                     a.lr)
    g.sync()
    t1 = time.time()
    if a.out:
        Path(a.out).parent.mkdir(parents=True, exist_ok=True)
        g.save(a.out)
    ev = evaluate(pkg, a.n, g, a.factor, steps=a.eval_steps)
    rep = {"n": a.n, "factor": a.factor, "pairs": made, "seeds": a.seeds, "ring": a.ring,
           "net_resolution": a.n // a.factor, "params": g.n_params, "train_steps": iters, "batch": a.batch,
           "lr": a.lr, "loss_weights": [a.w_pressure, a.w_residual], "stream_and_train_s": t1 - t0,
           "loss_history": hist, "eval": ev}
    print(json.dumps(rep))
    if a.report:
        Path(a.report).write_text(json.dumps(rep, indent=1))
    return rep


if __name__ == "__main__":
    main()
