"""Run one level-0 kernel of a nodal plan in isolation (for CUDA-event timing or an ncu capture).

  python -m incflo_gb300.profile_kernels --n 256 --which 1 --reps 3

which: 0 FP64 Jacobi sweep, 1 FP32 Jacobi sweep, 2 FP64 residual, 3 FP32 residual, 4 streaming triad
over the same arrays, 5 FP32 Jacobi through the plain kernel, 6 FP32 prolongation level 1 -> 0,
7 FP32 restriction level 0 -> 1. The plan holds the 256^3 variable-density workload's sigma (periodic x/y,
walls z); the only launches of the selected kernel are the level-0 ones, so `ncu -k regex:<kernel>`
captures exactly those.

  python -m incflo_gb300.profile_kernels --unet 128 --reps 5

times the warm-start U-Net's forward pass, and

  python -m incflo_gb300.profile_kernels --project mixed --n 256 --reps 1

runs whole projections of the 256^3 variable-density workload in one form (mixed | fp64), so that an
ncu launch list covers exactly one form.

  python -m incflo_gb300.profile_kernels --row eb_nodal --reps 1

runs the workload of one bench.py row (amr | mac | eb_mac | eb_nodal | tensor: the two-level composite
projection, the MAC projection of the headline grid, the cut-cell MAC and nodal projections of the
cylinder channel, the tensor diffusion solve)
with `reps` timed solves after one warm-up, so that an ncu launch list covers that row alone.

The U-Net mode runs the tensor-core convolutions on a 128 x 128 x 136 network grid (the multigrid
level 1 of a 256^3 projection) and reports the convolution FLOP rate.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from incflo_gb300 import _abi, synth  # noqa: E402
from incflo_gb300.projection import Geometry, _Plan, array4, make_options  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--which", type=int, default=1)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--unet", type=int, default=0, help="time the U-Net forward on an n x n x (n+8) grid")
    ap.add_argument("--project", default="", choices=["", "mixed", "fp64"])
    ap.add_argument("--opt", action="append", default=[], help="option override key=value (projection mode)")
    ap.add_argument("--row", default="", choices=["", "amr", "mac", "eb_mac", "eb_nodal", "tensor"])
    ap.add_argument("--rtol", type=float, default=1e-10)
    args = ap.parse_args()
    from incflo_gb300.build import build

    build()
    lib = _abi.load()
    if args.unet:
        return unet_forward(args.unet, args.reps)
    if args.project:
        return projections(args.n, args.project, args.reps, args.opt)
    if args.row:
        import bench

        run = getattr(bench, "run_" + args.row)
        args.no_parity = True  # the row alone: no oracle comparison inside the profiled run
        print(json.dumps(run(args, torch.device("cuda", 0), steps=args.reps, warmup=1)))
        return None
    n = args.n
    rho = synth.variable_density_rt(n)["rho"]
    geom = Geometry((n, n, n))
    plan = _Plan(geom, _abi.GBP_NODAL, (0, 0, 2), (0, 0, 2), make_options(0))
    r = torch.from_numpy(np.ascontiguousarray(rho)).cuda()
    _abi.check(lib.gbp_nodal_set_sigma_from_density(plan.ptr, ctypes.byref(array4(r)), 1.0, 1.0), "sigma")
    ms, by = ctypes.c_double(), ctypes.c_double()
    _abi.check(lib.gbp_plan_time_kernel(plan.ptr, args.which, args.reps, ctypes.byref(ms), ctypes.byref(by)), "time")
    print(json.dumps({"which": args.which, "n": n, "ms_per_launch": ms.value, "bytes_per_launch": by.value,
                      "GBps": by.value / ms.value / 1e6}))


def projections(n, form, reps, extra=()):
    from incflo_gb300 import apply_nodal_projection, make_options

    w = synth.variable_density_rt(n)
    geom = Geometry(w["n"], w["lo"], w["hi"])
    vel0 = torch.from_numpy(synth.with_ghosts(w["vel"], 1)).cuda()
    rho = torch.from_numpy(np.ascontiguousarray(w["rho"])).cuda()
    vel = vel0.clone()
    gp = torch.zeros((3,) + rho.shape, dtype=torch.float64, device="cuda")
    p_nd = torch.zeros((n + 1, n + 1, n + 1), dtype=torch.float64, device="cuda")
    opts = make_options(0, precision=form, mg_rtol=1e-10, mg_atol=0.0, **dict(kv.split("=", 1) for kv in extra))
    out = []
    for _ in range(reps):
        vel.copy_(vel0)
        gp.zero_()
        st = apply_nodal_projection(geom, w["bclo"], w["bchi"], vel, rho, gp, p_nd, set_inflow_bc=False,
                                    options=opts)
        out.append({k: st[k] for k in ("status", "vcycles", "outer_iters", "final_rel_resid", "ms_total")})
    print(json.dumps({"form": form, "n": n, "runs": out}))


def unet_forward(n, reps):
    from incflo_gb300.surrogate import Surrogate

    dims = (n, n, n + 8)
    rows = (dims[0] + 2) * (dims[1] + 2) * (dims[2] + 2)
    s = Surrogate(seed=0)
    x0 = torch.zeros((rows, 16), dtype=torch.bfloat16, device="cuda")
    x0[:, :3] = torch.randn((rows, 3), device="cuda").to(torch.bfloat16)
    s.predict(x0, dims)  # workspace, weights, warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        s.predict(x0, dims)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # conv FLOPs: 2 x voxels x taps x cin x cout per layer on its level's grid
    # (level, taps, input channels, output channels) of the 15 layers: encoder a/b per level, decoder
    # a (upsampled + skip) / b for levels 2, 1, 0, and the 1x1x1 head
    c = [16, 32, 64, 128]
    layers = []
    for lvl in range(4):
        layers += [(lvl, 27, 16 if lvl == 0 else c[lvl - 1], c[lvl]), (lvl, 27, c[lvl], c[lvl])]
    for lvl in (2, 1, 0):
        layers += [(lvl, 27, c[lvl + 1] + c[lvl], c[lvl]), (lvl, 27, c[lvl], c[lvl])]
    layers.append((0, 1, 16, 16))
    flops, vox = 0.0, dims[0] * dims[1] * dims[2]
    for lvl, t, ci, co in layers:
        flops += 2.0 * vox / 8 ** lvl * t * ci * co
    print(json.dumps({"unet_forward_ms": ms, "dims": dims, "gflop": flops / 1e9, "tflops": flops / ms / 1e9}))


if __name__ == "__main__":
    main()
