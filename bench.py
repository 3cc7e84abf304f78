"""Benchmark of the projection hot path: ms per nodal projection to 1e-10 relative residual on the
256^3 variable-density workload (rho 1 -> 3 tanh interface, periodic x/y, walls in z, sigma = 1/rho,
velocity a k^-2 Gaussian random field), chosen form (FP32 V-cycles inside FP64 iterative
refinement) against the plain FP64 multigrid, one GB300 per rank.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 256]

A step is one full projection (right-hand side, solve, velocity / gp / p_nd update) through the C
ABI (incflo::ApplyNodalProjection semantics) on device-resident inputs; the velocity is restored
from a pristine copy before each step (outside the per-step CUDA-event window). The inputs
(velocity 3x258^3, sigma, phi: > 1 GB) are larger than L2, so no flush is needed between steps.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/projection to 1e-10 rel. resid, 256³: learned+FP32-MG vs FP64 MG, one GB300"


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        backend = "nccl"
        try:
            import torch

            if not torch.cuda.is_available():
                backend = "gloo"
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce_max(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.proc = None
        # the raw samples (a few KB) go to BENCH_CLOCKS_DIR when set, else the system temp directory
        out_dir = os.environ.get("BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"clocks_bench_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(summary_name):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant kernel,
    read from the committed ncu summary's `traffic_bytes_per_launch:` line, if present."""
    p = os.path.join(ROOT, "profiles", summary_name)
    if os.path.exists(p):
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":", 1)[1].strip())
    return None


def cpu_projection(n, rtol):
    """The oracle's FP64 PCG-multigrid (C, OpenMP, all host threads) on one full projection of the
    benchmark workload at n^3: returns (ms, threads, stats, phi, projected velocity)."""
    import oracle as O
    from incflo_gb300 import synth

    w = synth.variable_density_rt(n)
    g = O.Grid(w["n"], lo=w["lo"], hi=w["hi"], bclo=w["bclo"], bchi=w["bchi"])
    vel = synth.with_ghosts(w["vel"], 1)
    sigma = 1.0 / w["rho"]
    t0 = time.perf_counter()
    vel_new, phi, _, st = O.nodal_project(g, sigma, vel, rtol=rtol, atol=0.0)
    dt = time.perf_counter() - t0
    return dt * 1e3, O.num_threads(), st, phi, vel_new


def run_reference(args, ws, rank):
    """The CPU reference arm: one full n^3 projection of the workload per timed step (warm-up steps at
    32^3, untimed: they only page the code and the OpenMP pool in)."""
    if rank != 0:
        return
    vals = []
    st = None
    for i in range(args.warmup + args.steps):
        ms, cores, st, _, _ = cpu_projection(args.n if i >= args.warmup else min(32, args.n), args.rtol)
        if i >= args.warmup:
            vals.append(ms)
    v = sum(vals) / len(vals)
    sample = (f"one full {args.n}^3 projection of the same workload per step (CPU oracle FP64 PCG-multigrid, "
              f"{cores} OpenMP threads)")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "ms/projection", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(v, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
        "config": {"workload": f"variable-density nodal projection {args.n}^3, periodic x/y, walls z, sigma=1/rho, "
                               f"rtol {args.rtol:g}", "n": args.n},
        "cpu_baseline": {"value": round(v, 3), "unit": "ms/projection", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(v, 3), "unit": "ms/projection", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own MLMG (AMReX / AMReX-Hydro) is not vendored and cannot be built here; "
                "the CPU oracle port stands in for it",
        "oracle_iters": st["iters"] if st else None,
    }
    print(json.dumps(line), flush=True)


def rel_l2(a, b):
    import numpy as np

    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def parity_cfg1(dev):
    """cfg1 (64^3 Taylor-Green + noise, triply periodic, rho = 1): nodal and MAC projections in both
    forms at incflo's tolerances (rtol 1e-11, atol 1e-14), phi error against the oracle (1e-13)."""
    import numpy as np
    import torch

    import oracle as O
    from incflo_gb300 import Geometry, MacProjector, NodalProjector, make_options, synth

    c = synth.taylor_green_noise(64)
    g = O.Grid(c["n"], c["lo"], c["hi"], c["bclo"], c["bchi"])
    vel = synth.with_ghosts(c["vel"])
    sigma = np.ones(g.cell_shape)
    _, phi_or, _, _ = O.nodal_project(g, sigma, vel, rtol=1e-13)
    n = c["n"]
    umac = []
    for d in range(3):
        u, ax = c["vel"][d], 2 - d
        m = u.shape[ax]
        umac.append(np.ascontiguousarray(0.5 * (np.take(u, np.arange(-1, m), axis=ax, mode="wrap") +
                                                np.take(u, np.arange(0, m + 1), axis=ax, mode="wrap"))))
    beta = [np.ones(x.shape) for x in umac]
    _, mphi_or, _ = O.mac_project(g, beta, umac, rtol=1e-13)
    out = {}
    for prec in ("fp64", "mixed"):
        vt = torch.from_numpy(vel).to(dev)
        proj = NodalProjector(vt, torch.from_numpy(sigma).to(dev), Geometry(n, c["lo"], c["hi"]),
                              options=make_options(0, precision=prec))
        proj.setDomainBC(c["bclo"], c["bchi"])
        st = proj.project(rtol=1e-11, atol=1e-14)
        nz, ny, nx = g.node_shape
        out[f"nodal_{prec}"] = rel_l2(proj.getPhi().cpu().numpy()[:nz, :ny, :nx], phi_or)
        mp = MacProjector(Geometry(n, c["lo"], c["hi"]), options=make_options(1, precision=prec))
        mp.initProjector(beta=1.0)
        mp.setDomainBC(c["bclo"], c["bchi"])
        mp.setUMAC([torch.from_numpy(u).to(dev) for u in umac])
        ph = torch.zeros(g.cell_shape, dtype=torch.float64, device=dev)
        st2 = mp.project(rtol=1e-11, atol=1e-14, phi=ph, phi_guess=False)
        if st["status"] or st2["status"]:
            raise RuntimeError(f"cfg1 projection failed: {st} {st2}")
        out[f"mac_{prec}"] = rel_l2(ph.cpu().numpy(), mphi_or)
    return {k: float(f"{v:.3e}") for k, v in out.items()}


def run_amr(args, dev, steps=3, warmup=1):
    """ms per two-level composite projection (mixed form): base n^3 variable-density interface, fine level
    (ratio 2) from tagging: cells within +-0.1 of the interface or with |vorticity| above its 90th
    percentile, blocking_factor 32, max_grid_size 64 (synth.rt_amr_tagged); inputs restored before each
    call (outside the timed region)."""
    import numpy as np
    import torch

    from incflo_gb300 import AmrNodalProjector, Geometry, make_options, synth

    w = synth.rt_amr_tagged(args.n)
    b = w["base"]
    n = b["n"]
    geom = Geometry(n, b["lo"], b["hi"])
    proj = AmrNodalProjector(geom, b["bclo"], b["bchi"], w["boxes"],
                             options=make_options(0, precision="mixed", mg_rtol=args.rtol, mg_atol=0.0))
    vel0 = torch.from_numpy(np.ascontiguousarray(b["vel"])).to(dev)
    rho_c = torch.from_numpy(np.ascontiguousarray(b["rho"])).to(dev)
    vel_c = vel0.clone()
    gp_c = torch.zeros_like(vel0)
    p_c = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device=dev)
    vel_f0 = [torch.from_numpy(v).to(dev) for v in w["vel_f"]]
    vel_f = [v.clone() for v in vel_f0]
    rho_f = [torch.from_numpy(r).to(dev) for r in w["rho_f"]]
    gp_f = [torch.zeros_like(v) for v in vel_f]
    p_f = [torch.zeros((hi[2] - lo[2] + 2, hi[1] - lo[1] + 2, hi[0] - lo[0] + 2), dtype=torch.float64, device=dev)
           for lo, hi in w["boxes"]]
    times, st = [], None
    for i in range(warmup + steps):
        vel_c.copy_(vel0)
        gp_c.zero_()
        for v, v0, g in zip(vel_f, vel_f0, gp_f):
            v.copy_(v0)
            g.zero_()
        torch.cuda.synchronize()
        st = proj.apply(vel_c, rho_c, gp_c, p_c, vel_f, rho_f, gp_f, p_f, scaling_factor=1.0)
        if st["status"] != 0:
            raise RuntimeError(f"amr projection failed: {st}")
        if i >= warmup:
            times.append(st["ms_total"])
    fine_cells = sum((hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) for lo, hi in w["boxes"])
    zlo = min(lo[2] for lo, _ in w["boxes"])
    zhi = max(hi[2] for _, hi in w["boxes"])
    out = {"workload": f"{args.n}^3 base + ratio-2 fine level from tagging (interface +-0.1 or |vorticity| > "
                       f"90th percentile; blocking_factor 32, max_grid_size 64): {len(w['boxes'])} fine boxes, "
                       f"{fine_cells} fine cells, fine z {zlo}..{zhi}; composite nodal projection, FP32 two-level "
                       f"steps (coarse V-cycle, fine Jacobi sweeps) inside FP64 refinement, rtol {args.rtol:g}",
           "ms_per_projection": round(sum(times) / len(times), 3), "outer_iters": st["outer_iters"],
           "vcycles": st["vcycles"], "final_rel_resid": st["final_rel_resid"],
           "device_bytes": proj.device_bytes()}
    del proj
    if not args.no_parity:
        out["parity"] = amr_parity(dev)
    return out


def amr_parity(dev, n=16):
    """phi against the composite FE oracle (scipy direct solve) on the same construction at a base the
    oracle solves in seconds (n^3, the same tagging, box rules scaled to blocking_factor 8 and
    max_grid_size 16), plain FP64 and mixed forms, rtol 1e-12."""
    import numpy as np
    import torch

    from incflo_gb300 import AmrNodalProjector, Geometry, make_options, synth
    from oracle.amr_nodal import CompositeNodal as Oracle

    w = synth.rt_amr_tagged(n, blocking=8, max_grid=16)
    b = w["base"]
    boxes = w["boxes"]
    nc = b["n"]
    nf = [2 * v for v in nc]
    fm = np.zeros((nf[2], nf[1], nf[0]), bool)
    rho_f = np.ones((nf[2], nf[1], nf[0]))
    u_f = np.zeros((3, nf[2], nf[1], nf[0]))
    for (lo, hi), r, v in zip(boxes, w["rho_f"], w["vel_f"]):
        sl = (slice(lo[2], hi[2] + 1), slice(lo[1], hi[1] + 1), slice(lo[0], hi[0] + 1))
        fm[sl] = True
        rho_f[sl] = r
        u_f[(slice(None),) + sl] = v
    ref = Oracle(nc, [1.0 / v for v in nc], b["bclo"], b["bchi"], fm).project(1.0 / b["rho"], 1.0 / rho_f, b["vel"],
                                                                            u_f)
    geom = Geometry(nc, b["lo"], b["hi"])
    out = {"base": n, "fine_boxes": len(boxes), "oracle": "scipy direct solve of the composite Q1 system"}
    for precision in ("fp64", "mixed"):
        proj = AmrNodalProjector(geom, b["bclo"], b["bchi"], boxes,
                                 options=make_options(0, precision=precision, mg_rtol=1e-12, mg_atol=0.0))
        vc = torch.from_numpy(np.ascontiguousarray(b["vel"])).to(dev)
        gc = torch.zeros_like(vc)
        pc = torch.zeros((nc[2] + 1, nc[1] + 1, nc[0] + 1), dtype=torch.float64, device=dev)
        vf = [torch.from_numpy(v).to(dev) for v in w["vel_f"]]
        gf = [torch.zeros_like(v) for v in vf]
        pf = [torch.zeros((hi[2] - lo[2] + 2, hi[1] - lo[1] + 2, hi[0] - lo[0] + 2), dtype=torch.float64,
                          device=dev) for lo, hi in boxes]
        st = proj.apply(vc, torch.from_numpy(np.ascontiguousarray(b["rho"])).to(dev), gc, pc, vf,
                        [torch.from_numpy(r).to(dev) for r in w["rho_f"]], gf, pf, scaling_factor=1.0)
        err_c = rel_l2(pc.cpu().numpy(), ref["phi_c"])
        num = den = 0.0
        for t, (lo, hi) in zip(pf, boxes):
            r = ref["phi_f"][lo[2]:hi[2] + 2, lo[1]:hi[1] + 2, lo[0]:hi[0] + 2]
            num += float(((t.cpu().numpy() - r) ** 2).sum())
            den += float((r ** 2).sum())
        out[precision] = {"status": st["status"], "phi_rel_l2_coarse": float(f"{err_c:.3e}"),
                          "phi_rel_l2_fine": float(f"{(num / den) ** 0.5:.3e}")}
        del proj
    return out


def run_mac(args, dev, steps=5, warmup=3):
    """ms per MAC projection on the headline workload's grid and density: n^3 unit cube, periodic x / y,
    walls z, face velocities from the k^-2 random field (cell values averaged to faces, zero normal
    velocity on the walls), beta = dt / rho_face with rho the tanh interface field (dt = 1), mixed form,
    rtol 1e-10."""
    import numpy as np
    import torch

    from incflo_gb300 import Geometry, MacProjector, make_options, synth

    w = synth.variable_density_rt(args.n)
    n = w["n"]
    P, N = 0, 2
    v = w["vel"]
    rho = w["rho"]
    shapes = [(n[2], n[1], n[0] + 1), (n[2], n[1] + 1, n[0]), (n[2] + 1, n[1], n[0])]
    u = [np.zeros(sh) for sh in shapes]
    u[0][:, :, 1:-1] = 0.5 * (v[0][:, :, 1:] + v[0][:, :, :-1])
    u[0][:, :, 0] = u[0][:, :, -1] = 0.5 * (v[0][:, :, 0] + v[0][:, :, -1])
    u[1][:, 1:-1, :] = 0.5 * (v[1][:, 1:, :] + v[1][:, :-1, :])
    u[1][:, 0, :] = u[1][:, -1, :] = 0.5 * (v[1][:, 0, :] + v[1][:, -1, :])
    u[2][1:-1] = 0.5 * (v[2][1:] + v[2][:-1])  # walls: zero normal velocity on faces 0 and n
    beta = [np.zeros(sh) for sh in shapes]
    beta[0][:, :, 1:-1] = 2.0 / (rho[:, :, 1:] + rho[:, :, :-1])
    beta[0][:, :, 0] = beta[0][:, :, -1] = 2.0 / (rho[:, :, 0] + rho[:, :, -1])
    beta[1][:, 1:-1, :] = 2.0 / (rho[:, 1:, :] + rho[:, :-1, :])
    beta[1][:, 0, :] = beta[1][:, -1, :] = 2.0 / (rho[:, 0, :] + rho[:, -1, :])
    beta[2][1:-1] = 2.0 / (rho[1:] + rho[:-1])
    beta[2][0], beta[2][-1] = 1.0 / rho[0], 1.0 / rho[-1]
    u0 = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in u]
    ut = [x.clone() for x in u0]
    mp = MacProjector(Geometry(n, w["lo"], w["hi"]),
                      options=make_options(1, precision="mixed", mg_rtol=args.rtol, mg_atol=0.0))
    mp.initProjector(beta=[torch.from_numpy(np.ascontiguousarray(b)).to(dev) for b in beta])
    mp.setDomainBC((P, P, N), (P, P, N))
    mp.setUMAC(ut)
    times, st = [], None
    for i in range(warmup + steps):
        for a, b in zip(ut, u0):
            a.copy_(b)
        torch.cuda.synchronize()
        st = mp.project(rtol=args.rtol, atol=0.0)
        if st["status"] != 0:
            raise RuntimeError(f"MAC projection failed: {st}")
        if i >= warmup:
            times.append(st["ms_total"])
    parity = None
    if not args.no_parity:
        import oracle as O

        for a, b in zip(ut, u0):
            a.copy_(b)
        ph = torch.zeros((n[2], n[1], n[0]), dtype=torch.float64, device=dev)
        mp.project(rtol=args.rtol, atol=0.0, phi=ph, phi_guess=False)
        g = O.Grid(n, w["lo"], w["hi"], (P, P, N), (P, P, N))
        _, phi_or, st_or = O.mac_project(g, beta, u, rtol=1e-12)
        parity = {"phi_rel_l2_chosen": float(f"{rel_l2(ph.cpu().numpy(), phi_or):.3e}"),
                  "oracle": f"CPU FP64 PCG-multigrid to rtol 1e-12 ({st_or['iters']} iterations)"}
    return {"workload": f"MAC projection {args.n}^3, variable density (rho 1->3 tanh interface, beta = 1/rho_face), "
                        f"periodic x/y, walls z, FP32 V-cycles inside FP64 refinement, rtol {args.rtol:g}",
            "ms_per_projection": round(sum(times) / len(times), 3), "outer_iters": st["outer_iters"],
            "vcycles": st["vcycles"], "final_rel_resid": st["final_rel_resid"], "parity": parity}


def run_eb_mac(args, dev, steps=5, warmup=3):
    """ms per cut-cell MAC projection on the cylinder channel: [0,4]x[0,1]^2 at 256x64x64, cylinder
    r = 0.125 at (1, 0.5) along z, inflow u = 1 + 1e-3 noise at x = 0, outflow x = 4, walls y,
    periodic z, rho = 1 (beta = dt = 1), mixed form, rtol 1e-10 (the cfg4 geometry)."""
    import numpy as np
    import torch

    from incflo_gb300 import Geometry, MacProjector, eb, make_options

    n, ext = (256, 64, 64), (4.0, 1.0, 1.0)
    P, D, N, I = 0, 1, 2, 3
    geo = eb.cylinder(n, (0, 0, 0), ext, (1.0, 0.5, 0.0), 0.125, small_volfrac=1e-4)
    rng = np.random.Generator(np.random.PCG64(4))
    shapes = [(n[2], n[1], n[0] + 1), (n[2], n[1] + 1, n[0]), (n[2] + 1, n[1], n[0])]
    u = [1e-3 * rng.uniform(-1.0, 1.0, sh) for sh in shapes]
    u[0] += 1.0
    u[0][:, :, 0] = 1.0
    u[1][:, 0, :] = 0.0
    u[1][:, -1, :] = 0.0
    u[2][-1] = u[2][0]
    u0 = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in u]
    ut = [x.clone() for x in u0]
    mp = MacProjector(Geometry(n, (0, 0, 0), ext),
                      options=make_options(1, precision="mixed", mg_rtol=args.rtol, mg_atol=0.0))
    mp.initProjector(beta=1.0)
    mp.setDomainBC((I, N, P), (D, N, P))
    mp.setEB(torch.from_numpy(geo["vfrac"]).to(dev), [torch.from_numpy(geo[k]).to(dev) for k in ("apx", "apy", "apz")],
             [torch.from_numpy(np.ascontiguousarray(np.moveaxis(geo[k], -1, 0))).to(dev) for k in ("fcx", "fcy", "fcz")])
    mp.setUMAC(ut)
    times, st = [], None
    for i in range(warmup + steps):
        for a, b in zip(ut, u0):
            a.copy_(b)
        torch.cuda.synchronize()
        st = mp.project(rtol=args.rtol, atol=0.0)
        if st["status"] != 0:
            raise RuntimeError(f"EB MAC projection failed: {st}")
        if i >= warmup:
            times.append(st["ms_total"])
    cut = int(((geo["vfrac"] > 0) & (geo["vfrac"] < 1)).sum())
    parity = None
    if not args.no_parity:
        # too large for the direct cut-cell oracle: the oracle's own divergence of the projected faces
        from oracle.eb_mac import EBMac

        ap = [geo["apx"], geo["apy"], geo["apz"]]
        fc = [geo["fcx"], geo["fcy"], geo["fcz"]]
        m = EBMac(n, [ext[d] / n[d] for d in range(3)], (I, N, P), (D, N, P), geo["vfrac"], ap, fc,
                  [np.ones(a.shape) for a in ap])
        d0, d1 = m.divergence(u), m.divergence([x.cpu().numpy() for x in ut])
        parity = {"oracle_divergence_ratio": float(f"{d1 / d0:.3e}"),
                  "check": "max |cut-cell divergence| / (kappa V) of the projected face velocities in the oracle's "
                           "operator, relative to the input's (the direct oracle solve does not fit this size)"}
    return {"workload": f"cut-cell MAC projection, cylinder channel 256x64x64 ({cut} cut cells), inflow / outflow "
                        f"/ walls / periodic, FP32 V-cycles inside FP64 refinement, rtol {args.rtol:g}",
            "ms_per_projection": round(sum(times) / len(times), 3), "outer_iters": st["outer_iters"],
            "vcycles": st["vcycles"], "final_rel_resid": st["final_rel_resid"], "parity": parity}


def run_eb_nodal(args, dev, steps=5, warmup=3):
    """ms per cut-cell nodal projection on the cylinder channel of run_eb_mac (inflow u = 1 through
    the ghost cells at x = 0, outflow x = 4, walls y, periodic z, rho = 1), mixed form, rtol 1e-10."""
    import numpy as np
    import torch

    from incflo_gb300 import Geometry, apply_nodal_projection, eb, make_options

    n, ext = (256, 64, 64), (4.0, 1.0, 1.0)
    P, D, N, I = 0, 1, 2, 3
    M = eb.moments_components(eb.cylinder_moments(n, (0, 0, 0), ext, (1.0, 0.5, 0.0), 0.125, small_volfrac=1e-4))
    rng = np.random.Generator(np.random.PCG64(4))
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vel[:, 1:-1, 1:-1, 1:-1] = 1e-3 * rng.uniform(-1.0, 1.0, (3, n[2], n[1], n[0]))
    vel[0, 1:-1, 1:-1, 1:-1] += 1.0
    vel[0, :, :, 0] = 1.0  # inflow ghost cells
    v0 = torch.from_numpy(vel).to(dev)
    vt = v0.clone()
    rho = torch.ones((n[2], n[1], n[0]), dtype=torch.float64, device=dev)
    gp = torch.zeros((3, n[2], n[1], n[0]), dtype=torch.float64, device=dev)
    pnd = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device=dev)
    Mt = torch.from_numpy(M).to(dev)
    opts = make_options(0, precision="mixed", mg_rtol=args.rtol, mg_atol=0.0)
    geom = Geometry(n, (0, 0, 0), ext)
    times, st = [], None
    for i in range(warmup + steps):
        vt.copy_(v0)
        gp.zero_()
        torch.cuda.synchronize()
        st = apply_nodal_projection(geom, (I, N, P), (D, N, P), vt, rho, gp, pnd, set_inflow_bc=True, options=opts,
                                    eb_moments=Mt)
        if st["status"] != 0:
            raise RuntimeError(f"EB nodal projection failed: {st}")
        if i >= warmup:
            times.append(st["ms_total"])
    kap = M[0]
    parity = None
    if not args.no_parity:
        # the GPU phi's residual in the oracle's cut-cell operator (the direct solve does not fit this size)
        from oracle.eb_nodal import EBNodal

        Mfull = eb.cylinder_moments(n, (0, 0, 0), ext, (1.0, 0.5, 0.0), 0.125, small_volfrac=1e-4)
        o = EBNodal(n, [ext[d] / n[d] for d in range(3)], (I, N, P), (D, N, P), Mfull)
        r = o.residual_norm(np.ones((n[2], n[1], n[0])), np.ascontiguousarray(vel[:, 1:-1, 1:-1, 1:-1]),
                            pnd.cpu().numpy(), vel)
        parity = {"oracle_rel_resid": float(f"{r:.3e}"),
                  "check": "max |b - A phi| / (fluid dual volume) of the GPU phi in the oracle's cut-cell operator, "
                           "relative to |b| (the direct oracle solve does not fit this size)"}
    return {"workload": f"cut-cell nodal projection, cylinder channel 256x64x64 ({int(((kap > 0) & (kap < 1)).sum())} "
                        f"cut cells), inflow / outflow / walls / periodic, FP32 V-cycles inside FP64 refinement, "
                        f"rtol {args.rtol:g}",
            "ms_per_projection": round(sum(times) / len(times), 3), "outer_iters": st["outer_iters"],
            "vcycles": st["vcycles"], "final_rel_resid": st["final_rel_resid"], "parity": parity}


def run_tensor(args, dev, steps=3, warmup=3):
    """ms per tensor (velocity) diffusion solve, DiffusionTensorOp::diffuse_velocity on an n^3 channel (256^3)
    (periodic x / z, no-slip walls y with a moving upper wall), rho 1..2 and eta 0.01..0.02 seeded
    random, dt = 0.5 h, rhs = rho u, rtol 1e-10, FP32 block V-cycles inside FP64 defect correction."""
    import torch

    from incflo_gb300 import Geometry, make_options
    from incflo_gb300.diffusion import TensorOp, diffuse_tensor_bc

    n = args.n
    bclo, bchi = diffuse_tensor_bc(("periodic", "no_slip_wall", "periodic"), ("periodic", "no_slip_wall", "periodic"))
    g = torch.Generator(device=dev).manual_seed(11)
    rho = 1.0 + torch.rand((n, n, n), dtype=torch.float64, device=dev, generator=g)
    eta = 0.01 * (1.0 + torch.rand((n, n, n), dtype=torch.float64, device=dev, generator=g))
    v0 = torch.zeros((3, n + 2, n + 2, n + 2), dtype=torch.float64, device=dev)
    v0[:, 1:-1, 1:-1, 1:-1] = torch.randn((3, n, n, n), dtype=torch.float64, device=dev, generator=g)
    v0[0, 1:-1, -1, 1:-1] = 1.0  # moving upper wall
    rhs = (rho[None] * v0[:, 1:-1, 1:-1, 1:-1]).contiguous()
    op = TensorOp(Geometry((n, n, n), (0, 0, 0), (1.0, 1.0, 1.0)), options=make_options(1, precision="mixed"))
    op.setDomainBC(bclo, bchi)
    op.setScalars(1.0, 0.5 / n)
    op.setACoeffs(0, rho)
    op.setShearViscosity(0, eta)
    vt = v0.clone()
    times, st = [], None
    for i in range(warmup + steps):
        vt.copy_(v0)
        torch.cuda.synchronize()
        st = op.solve(vt, rhs, rtol=args.rtol, atol=0.0)
        if st["status"] != 0:
            raise RuntimeError(f"tensor solve failed: {st}")
        if i >= warmup:
            times.append(st["ms_solve"])
    del op
    return {"workload": f"tensor (velocity) diffusion {n}^3, periodic x/z, no-slip walls y, rho 1..2, eta 0.01..0.02, "
                        f"dt = 0.5 h, rtol {args.rtol:g}, FP32 block V-cycles inside FP64 defect correction",
            "ms_per_solve": round(sum(times) / len(times), 3), "outer_iters": st["outer_iters"],
            "block_vcycles": st["vcycles"], "final_rel_resid": st["final_rel_resid"]}


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch

    from __graft_entry__ import build
    from incflo_gb300 import Geometry, _abi, apply_nodal_projection, make_options, synth
    from incflo_gb300.projection import _Plan, array4  # noqa: F401

    build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if rank != 0:
        args.no_parity = True  # the oracle checks run once, on rank 0
    n = args.n
    w = synth.variable_density_rt(n)
    geom = Geometry(w["n"], w["lo"], w["hi"])
    bclo, bchi = w["bclo"], w["bchi"]
    vel0 = torch.from_numpy(synth.with_ghosts(w["vel"], 1)).to(dev)
    rho = torch.from_numpy(np.ascontiguousarray(w["rho"])).to(dev)
    vel = vel0.clone()
    gp = torch.zeros((3,) + rho.shape, dtype=torch.float64, device=dev)
    p_nd = torch.zeros((n + 1, n + 1, n + 1), dtype=torch.float64, device=dev)
    lib = _abi.load()

    surrogate = None
    if not args.no_warm_start:
        from incflo_gb300.surrogate import WEIGHTS, Surrogate

        if not os.path.exists(WEIGHTS):
            raise RuntimeError(f"{WEIGHTS} is missing: train it with python -m incflo_gb300.train_surrogate")
        surrogate = Surrogate(path=WEIGHTS)

    def run_form(precision, steps, warmup, sur=None):
        opts = make_options(0, precision=precision, mg_rtol=args.rtol, mg_atol=0.0,
                            ir_inner_cycles=args.inner)
        stream = torch.cuda.current_stream()
        evs = []
        stats = []
        for i in range(warmup + steps):
            vel.copy_(vel0)
            gp.zero_()
            if i == warmup:
                barrier(ws)
                torch.cuda.synchronize()
                t_wall = time.perf_counter()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = apply_nodal_projection(geom, bclo, bchi, vel, rho, gp, p_nd, scaling_factor=1.0, incremental=False,
                                        set_inflow_bc=False, options=opts, surrogate=sur,
                                        surrogate_level=args.warm_level)
            e1.record(stream)
            if st["status"] != 0:
                raise RuntimeError(f"projection failed: {st}")
            if i >= warmup:
                evs.append((e0, e1))
                stats.append(st)
        torch.cuda.synchronize()
        barrier(ws)
        wall = time.perf_counter() - t_wall
        dev_ms = [a.elapsed_time(b) for a, b in evs]
        return dev_ms, stats, wall

    sampler = ClockSampler(local)
    sampler.start()
    ms_mixed, st_mixed, wall_mixed = run_form("mixed", args.steps, args.warmup, surrogate)
    clocks = sampler.stop()
    # the last timed step's outputs, for the error against the oracle (checked after all timing)
    phi_mixed_out = p_nd.cpu().numpy()
    vel_mixed_out = vel.cpu().numpy()
    warm = None
    if surrogate is not None:
        codes = [s_["warm_start"] for s_ in st_mixed]
        attempted = [s_ for s_ in st_mixed if s_["warm_start"] in (1, 2)]
        ms_plain_mixed, st_plain_mixed, _ = run_form("mixed", max(1, min(args.steps, 5)), 1)
        warm = {"network_level": args.warm_level, "used": codes.count(1), "bypassed": codes.count(2),
                "skipped": codes.count(3),
                "warm_rel_resid": attempted[0]["warm_rel_resid"] if attempted else None,
                "ms_warm_attempt": round(attempted[0]["ms_warm"], 3) if attempted else None,
                "mixed_without_warm_start_ms": round(sum(ms_plain_mixed) / len(ms_plain_mixed), 4),
                "mixed_without_warm_start_vcycles": st_plain_mixed[0]["vcycles"]}
    ms_fp64, st_fp64, wall_fp64 = run_form("fp64", max(1, min(args.steps, args.fp64_steps)), 1)
    phi_fp64_out = p_nd.cpu().numpy()

    tot_mixed = allreduce_max(ws, sum(ms_mixed))
    per_step = tot_mixed / len(ms_mixed)
    value = tot_mixed / (len(ms_mixed) * ws)
    fp64_ms = allreduce_max(ws, sum(ms_fp64)) / len(ms_fp64)

    # dominant kernel of the chosen form: the level-0 FP32 Jacobi sweep; time it live
    key = (tuple(geom.n_cell), tuple(geom.prob_lo), tuple(geom.prob_hi), tuple(bclo), tuple(bchi), 100,
           torch.cuda.current_device())
    from incflo_gb300.projection import NodalProjector

    plan = NodalProjector._plans[key]
    ms_k, bytes_k = ctypes.c_double(), ctypes.c_double()
    _abi.check(lib.gbp_plan_time_kernel(plan.ptr, 1, 50, ctypes.byref(ms_k), ctypes.byref(bytes_k)), "time_kernel")
    ms64, bytes64 = ctypes.c_double(), ctypes.c_double()
    _abi.check(lib.gbp_plan_time_kernel(plan.ptr, 0, 10, ctypes.byref(ms64), ctypes.byref(bytes64)), "time_kernel")
    peak, peak_kind = measured_peaks()
    ach = bytes_k.value / (ms_k.value * 1e-3) / 1e9
    ach64 = bytes64.value / (ms64.value * 1e-3) / 1e9

    # end to end: host buffers through the C ABI, copies inside the timed call
    e2e = None
    if not args.no_e2e:
        nc = n ** 3
        vel_h0 = np.ascontiguousarray(w["vel"])
        vel_h = torch.empty((3, n, n, n), dtype=torch.float64).pin_memory()
        rho_h = torch.from_numpy(np.ascontiguousarray(w["rho"])).pin_memory()
        gp_h = torch.zeros((3, n, n, n), dtype=torch.float64).pin_memory()
        p_h = torch.zeros((n + 1, n + 1, n + 1), dtype=torch.float64).pin_memory()
        hplan = _Plan(geom, _abi.GBP_NODAL, bclo, bchi,
                      make_options(0, precision="mixed", mg_rtol=args.rtol, mg_atol=0.0, ir_inner_cycles=args.inner))
        if surrogate is not None:
            _abi.check(lib.gbp_plan_set_surrogate(hplan.ptr, surrogate.ptr, args.warm_level, 1), "set_surrogate")
        times = []
        # the same warm-up count as the device-resident run (the warm-start bypass rule settles in it)
        e2e_warm = max(1, args.warmup)
        for i in range(e2e_warm + args.e2e_steps):
            vel_h.numpy()[...] = vel_h0
            gp_h.zero_()
            sth = _abi.Stats()
            t0 = time.perf_counter()
            rc = lib.gbp_apply_nodal_projection_host(hplan.ptr, vel_h.data_ptr(), rho_h.data_ptr(), 1.0,
                                                     gp_h.data_ptr(), p_h.data_ptr(), 1.0, 0, ctypes.byref(sth))
            dt = time.perf_counter() - t0
            _abi.check(rc, "gbp_apply_nodal_projection_host")
            if i >= e2e_warm:
                times.append(dt * 1e3)
        e2e_ms = allreduce_max(ws, sum(times)) / (len(times) * ws)
        e2e = {"value": round(e2e_ms, 3), "unit": "ms/projection", "h2d_bytes_per_step": 7 * nc * 8,
               "d2h_bytes_per_step": 6 * nc * 8 + (n + 1) ** 3 * 8}
        del hplan

    # two-level (AMR) composite projection: the 256^3 base plus a refined interface band (cfg5-like)
    amr = None
    if not args.no_amr:
        amr = run_amr(args, dev)
    eb_mac = eb_nodal = None
    if not args.no_eb:
        eb_mac = run_eb_mac(args, dev)
        eb_nodal = run_eb_nodal(args, dev)
    tensor = None if args.no_tensor else run_tensor(args, dev)
    mac = None if args.no_mac else run_mac(args, dev)
    # the warm start where it has a previous solution: successive projections of a slowly displaced
    # interface (held-out seed), zero start vs previous-phi start vs previous phi + the network's increment
    if warm is not None and not args.no_sequence:
        from incflo_gb300.train_surrogate import evaluate_sequence

        warm["sequence"] = {"workload": f"{n}^3, 8 successive projections of synth.rt_sequence(seed 7777), "
                                        "timed: the 7 that have a previous phi",
                            **evaluate_sequence(surrogate, n, 7777, steps=8, level=args.warm_level)}

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        ms_cpu, cores, st_cpu, _, _ = cpu_projection(n, args.rtol)
        cpu = {"value": round(ms_cpu, 1), "unit": "ms/projection", "cores": cores, "kind": "port",
               "sample": f"one full {n}^3 projection of the same workload (CPU oracle FP64 PCG-multigrid, "
                         f"{st_cpu['iters']} iterations to rtol {args.rtol:g})"}
    if rank == 0 and not args.no_parity:
        # error of each form against the FP64 oracle solved to 1e-12 (outside every timed region)
        import oracle as O

        _, _, st_ref, phi_ref, vel_ref = cpu_projection(n, 1e-12)
        gref = O.Grid(w["n"], lo=w["lo"], hi=w["hi"], bclo=bclo, bchi=bchi)
        nz, ny, nx = gref.node_shape
        div_ref = float(np.abs(O.nodal_rhs(gref, vel_ref)).max())
        parity = {"oracle": f"CPU FP64 PCG-multigrid to rtol 1e-12 ({st_ref['iters']} iterations)",
                  "cfg2_nodal_256": {
                      "phi_rel_l2_chosen": float(f"{rel_l2(phi_mixed_out[:nz, :ny, :nx], phi_ref):.3e}"),
                      "phi_rel_l2_plain_fp64": float(f"{rel_l2(phi_fp64_out[:nz, :ny, :nx], phi_ref):.3e}"),
                      "max_div_after_chosen": float(f"{np.abs(O.nodal_rhs(gref, vel_mixed_out)).max():.6e}"),
                      "max_div_after_oracle": float(f"{div_ref:.6e}")}}
        del phi_ref, vel_ref
        if mac is not None:
            parity["cfg2_mac_256"] = mac.pop("parity", None)
        parity["cfg1_tg_64"] = parity_cfg1(dev)
        for row, key in ((eb_mac, "cfg4_eb_mac"), (eb_nodal, "cfg4_eb_nodal")):
            if row is not None and "parity" in row:
                parity[key] = row.pop("parity")

    launches = int(sum(s["kernel_launches"] for s in st_mixed))
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "ms/projection", "n_gpus": ws,
        "steps": len(ms_mixed), "warmup": args.warmup, "ms_per_step": round(per_step, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64 (f32 inner V-cycles)",
        "data": "synthetic (seeded PCG64)",
        "config": {"workload": f"variable-density nodal projection {n}^3 (rho 1->3 tanh interface, k^-2 random "
                               f"velocity), periodic x/y, walls z, sigma=1/rho, rtol {args.rtol:g}",
                   "n": n, "form": ("learned warm start (U-Net on multigrid level 1, bypass rule) + " if surrogate
                                    else "") + "FP32 V-cycles inside FP64 iterative refinement",
                   "ir_inner_cycles": args.inner, "l2": "inputs larger than L2 (no flush)",
                   "parallelism": f"replicas x{ws}"},
        "plain_fp64": {"ms_per_projection": round(fp64_ms, 3), "vcycles": st_fp64[0]["vcycles"],
                       "final_rel_resid": st_fp64[0]["final_rel_resid"]},
        "chosen": {"vcycles": st_mixed[0]["vcycles"], "outer_iters": st_mixed[0]["outer_iters"],
                   "final_rel_resid": st_mixed[0]["final_rel_resid"],
                   "speedup_vs_plain_fp64": round(fp64_ms / per_step, 3)},
        "warm_start": warm,
        "wall_ms_per_step": round(wall_mixed * 1e3 / len(ms_mixed), 3),
        "roofline": {"bound": "hbm", "kernel": "k_vsweep32<0> (FP32 Jacobi sweep, level 0, whole-row TMA tiles)", "achieved": round(ach, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4),
                     "traffic": ncu_traffic("k_vsweep32_nodal_256.md"), "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": bytes_k.value, "ms_per_launch": round(ms_k.value, 5)},
        "roofline_fp64_jacobi": {"achieved_gbs": round(ach64, 1), "frac_hbm": round(ach64 / peak, 4),
                                 "ms_per_launch": round(ms64.value, 5)},
        "cpu_baseline": cpu,
        "parity": parity,
        "e2e": e2e,
        "amr": amr,
        "mac": mac,
        "eb_mac": eb_mac,
        "eb_nodal": eb_nodal,
        "tensor_diffusion": tensor,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    # --size: the same, for command lines under torchrun (whose own options take every --n... prefix)
    ap.add_argument("--n", "--size", dest="n", type=int, default=256)
    ap.add_argument("--rtol", type=float, default=1e-10)
    ap.add_argument("--inner", type=int, default=5)
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-amr", action="store_true")
    ap.add_argument("--no-eb", action="store_true")
    ap.add_argument("--no-tensor", action="store_true")
    ap.add_argument("--no-mac", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--no-warm-start", action="store_true")
    ap.add_argument("--no-sequence", action="store_true")
    ap.add_argument("--warm-level", type=int, default=1)
    args = ap.parse_args()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
