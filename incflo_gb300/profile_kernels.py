"""Run one level-0 kernel of a nodal plan in isolation (for CUDA-event timing or an ncu capture).

  python -m incflo_gb300.profile_kernels --n 256 --which 1 --reps 3

which: 0 FP64 Jacobi sweep, 1 FP32 Jacobi sweep, 2 FP64 residual, 3 FP32 residual. The plan holds the
256^3 variable-density workload's sigma (periodic x/y, walls z); the only launches of the selected
kernel are the level-0 ones, so `ncu -k regex:<kernel>` captures exactly those.
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
    args = ap.parse_args()
    from incflo_gb300.build import build

    build()
    lib = _abi.load()
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


if __name__ == "__main__":
    main()
