"""Train the warm-start U-Net on the GPU and save its weights.

  python -m incflo_gb300.train_surrogate --n 128 --samples 32 --steps 600 \
      --out incflo_gb300/weights/unet16_rt128.bin

Training pairs come from this library's own solver: variable-density fields of the 256^3 benchmark's
family (tanh interface with a random height field, k^-2 random velocity) at n^3 with held-apart
seeds, each projected to 1e-10 in the mixed form; the network learns rhs, sigma (, previous phi)
-> phi. A fraction of the pairs carries a previous phi (the solution of the same density with an
unperturbed velocity). Afterwards the script evaluates the warm start on one held-out problem at
--eval-n^3 with the network on multigrid level 1, and prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from incflo_gb300 import Geometry, NodalProjector, make_options, synth  # noqa: E402
from incflo_gb300.surrogate import WEIGHTS, Surrogate  # noqa: E402

BC = (["Periodic", "Periodic", "Neumann"], ["Periodic", "Periodic", "Neumann"])


def projector(case, vel=None, surrogate=None, level=1, rtol=1e-10):
    geom = Geometry(case["n"], case["lo"], case["hi"])
    v = torch.from_numpy(synth.with_ghosts(case["vel"] if vel is None else vel)).cuda()
    sigma = torch.from_numpy(1.0 / case["rho"]).cuda()
    p = NodalProjector(v, sigma, geom, options=make_options(0, precision="mixed", mg_rtol=rtol, mg_atol=0.0))
    p.setDomainBC(*BC)
    if surrogate is not None:
        p.setSurrogate(surrogate, level)
    return p


def make_samples(s, n, count, prev_frac, seed0):
    for i in range(count):
        case = synth.variable_density_rt(n, seed_h=seed0 + i, seed_u=seed0 + 5000 + i)
        prev = None
        if i < int(prev_frac * count):
            p0 = projector(case)
            p0.project()
            prev = p0.getPhi().clone()
            pert = synth.gaussian_random_field(case["n"], seed0 + 9000 + i)
            vel = case["vel"] + 0.3 * pert
        else:
            vel = None
        p = projector(case, vel)
        st = p.project()
        if st["status"] != 0:
            raise RuntimeError(f"training solve {i} did not converge: {st}")
        s.add_sample(p, phi_prev=prev)


def evaluate(s, n, seed, level=1, reps=3):
    case = synth.variable_density_rt(n, seed_h=seed, seed_u=seed + 5000)
    out = {}
    for name, sur in (("zero_start", None), ("learned", s)):
        p = projector(case, surrogate=sur, level=level)
        p.project()  # warm-up (plans, graphs)
        ms, st = [], None
        for _ in range(reps):
            p.vel.copy_(torch.from_numpy(synth.with_ghosts(case["vel"])).cuda())
            torch.cuda.synchronize()
            st = p.project()
            ms.append(st["ms_total"])
        out[name] = {"ms": round(float(np.median(ms)), 3), "vcycles": st["vcycles"],
                     "outer_iters": st["outer_iters"], "final_rel_resid": st["final_rel_resid"],
                     "warm_start": st["warm_start"], "warm_rel_resid": st["warm_rel_resid"],
                     "ms_warm": round(st["ms_warm"], 3)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--samples", type=int, default=32)
    ap.add_argument("--prev-frac", type=float, default=0.25)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval-n", type=int, default=256)
    args = ap.parse_args()
    from incflo_gb300.build import build

    build()
    torch.cuda.init()
    s = Surrogate(seed=args.seed)
    t0 = time.time()
    make_samples(s, args.n, args.samples, args.prev_frac, 1000)
    t1 = time.time()
    torch.cuda.synchronize()
    losses = s.train(args.steps, lr=args.lr, seed=args.seed)
    torch.cuda.synchronize()
    t2 = time.time()
    s.save(args.out)
    ev = evaluate(s, args.eval_n, 777) if args.eval_n else None
    print(json.dumps({"samples": args.samples, "n": args.n, "steps": args.steps, "sample_s": round(t1 - t0, 1),
                      "train_s": round(t2 - t1, 2), "ms_per_step": round(1e3 * (t2 - t1) / max(1, args.steps), 3),
                      "loss_first": float(np.mean(losses[:20])), "loss_last": float(np.mean(losses[-20:])),
                      "weights": os.path.relpath(args.out, ROOT), "eval": ev}), flush=True)


if __name__ == "__main__":
    main()
