"""Train the warm-start U-Net on the GPU and save its weights.

  python -m incflo_gb300.train_surrogate --n 128 --pairs 2000 --seq-len 20 \
      --out incflo_gb300/weights/unet16_seq128.bin

Training pairs come from this library's own plain (FP64) solver, written while it steps through time
sequences at n^3 (the setting of an incflo run, where every projection has the previous one's phi):
half of the sequences are slowly displaced variable-density interfaces (synth.rt_sequence: the 256^3
benchmark's family, tanh interface of random height, turning k^-2 velocity), half are double shear
layers (synth.double_shear_sequence: u = tanh(30 (y - 1/4)) / tanh(30 (3/4 - y)), v = 0.05 sin(2 pi x),
plus a turning k^-2 perturbation), seeds held apart from the evaluation's. Each projection of a
sequence is solved to rtol 1e-10 from the previous phi and gives one pair: inputs (rhs - A phi_prev,
sigma, phi_prev) -> target phi - phi_prev, the increment the solver's initial_guess = previous start is
missing (channel 0 is the residual of that start, so the increment is A^-1 of it; the first projection of
a sequence: phi_prev = 0, channel 0 = rhs, target phi). The pairs stream through
gbp_surrogate_train_step (one Adam step each, nothing stored), so `--pairs` pairs cost one solve and one
training step apiece. Afterwards the script evaluates the three starts (zero, previous phi, previous phi
+ the network's increment) on a held-out interface sequence at --eval-n^3 with the network on multigrid
level 1, and prints one JSON line.
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


def projector(case, precision="mixed", initial_guess="zero", surrogate=None, level=1, rtol=1e-10, vel=None):
    geom = Geometry(case["n"], case["lo"], case["hi"])
    v = vel if vel is not None else torch.from_numpy(synth.with_ghosts(case["vel"])).cuda()
    sigma = case["sigma_t"] if "sigma_t" in case else torch.from_numpy(1.0 / case["rho"]).cuda()
    p = NodalProjector(v, sigma, geom, options=make_options(0, precision=precision, mg_rtol=rtol, mg_atol=0.0,
                                                            initial_guess=initial_guess))
    p.setDomainBC(*BC)
    if surrogate is not None:
        p.setSurrogate(surrogate, level)
    return p


def lr_at(k, total, lr):
    """step schedule: lr for the first 60 % of the pairs, lr / 3 to 85 %, lr / 10 after"""
    f = k / max(1, total)
    return lr if f < 0.6 else (lr / 3.0 if f < 0.85 else lr / 10.0)


def stream_pairs(s, n, pairs, seq_len, lr, seed0):
    """solve the training sequences with the plain solver and take one Adam step per projection"""
    NodalProjector._plans.clear()
    losses = []
    k = 0
    q = 0
    while k < pairs:
        gen = (synth.rt_sequence(n, seed=seed0 + q, steps=seq_len) if q % 2 == 0
               else synth.double_shear_sequence(n, seed=seed0 + q, steps=seq_len))
        prev = None
        for case in gen:
            if k >= pairs:
                break
            p = projector(case, precision="fp64", initial_guess="previous")
            st = p.project()
            if st["status"] != 0:
                raise RuntimeError(f"training solve {k} did not converge: {st}")
            losses.append(s.train_step(p, prev, lr=lr_at(k, pairs, lr)))
            prev = p.getPhi().clone()
            k += 1
            if k % 100 == 0:
                print(json.dumps({"pairs": k, "loss_last100": float(np.mean(losses[-100:]))}), flush=True)
        q += 1
    NodalProjector._plans.clear()
    return losses, q


def evaluate_sequence(s, n, seed, steps=8, level=1):
    """The three starts on one held-out interface sequence: per form, V-cycles and device ms of every
    projection after the first (which has no previous phi), and how the network's candidate fared."""
    cases = []
    for case in synth.rt_sequence(n, seed=seed, steps=steps):
        cases.append(dict(n=case["n"], lo=case["lo"], hi=case["hi"],
                          vel_t=torch.from_numpy(synth.with_ghosts(case["vel"])).cuda(),
                          sigma_t=torch.from_numpy(1.0 / case["rho"]).cuda()))
    out = {}
    for name, ig, sur in (("zero_start", "zero", None), ("previous_phi", "previous", None),
                          ("learned_increment", "previous", s)):
        NodalProjector._plans.clear()
        # warm-up on the first case (plan, graphs), then the sequence on the same plan: its first step
        # starts from zero and, with initial_guess = previous, leaves its phi as the next step's start
        projector(cases[0], vel=cases[0]["vel_t"].clone()).project()
        ms, vc, used, rel = [], [], [], []
        for q, c in enumerate(cases):
            p = projector(c, initial_guess=ig, surrogate=sur if q > 0 else None, level=level,
                          vel=c["vel_t"].clone())
            torch.cuda.synchronize()
            st = p.project()
            if q == 0:
                continue
            ms.append(st["ms_total"])
            vc.append(st["vcycles"])
            used.append(int(st["warm_start"]))
            rel.append((st["prev_rel_resid"], st["warm_rel_resid"]))
        out[name] = {"ms_per_projection": round(float(np.mean(ms)), 3), "vcycles_per_projection": float(np.mean(vc)),
                     "vcycles": vc, "warm_start": used,
                     "prev_rel_resid": [round(a, 6) for a, _ in rel], "warm_rel_resid": [round(b, 6) for _, b in rel]}
    NodalProjector._plans.clear()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--pairs", type=int, default=2000)
    ap.add_argument("--seq-len", type=int, default=20)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval-n", type=int, default=256)
    ap.add_argument("--eval-seed", type=int, default=7777)
    args = ap.parse_args()
    from incflo_gb300.build import build

    build()
    torch.cuda.init()
    s = Surrogate(seed=args.seed)
    t0 = time.time()
    losses, nseq = stream_pairs(s, args.n, args.pairs, args.seq_len, args.lr, 1000)
    torch.cuda.synchronize()
    t1 = time.time()
    s.save(args.out)
    ev = evaluate_sequence(s, args.eval_n, args.eval_seed) if args.eval_n else None
    print(json.dumps({"pairs": len(losses), "sequences": nseq, "n": args.n, "train_s": round(t1 - t0, 1),
                      "loss_first": float(np.mean(losses[:50])), "loss_last": float(np.mean(losses[-50:])),
                      "weights": os.path.relpath(args.out, ROOT), "eval": ev}), flush=True)


if __name__ == "__main__":
    main()
