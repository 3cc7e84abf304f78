"""Multi-box levels (a MultiFab split into FABs by max_grid_size): the per-FAB entry points against the
single-box entry points on the same data. The boxes are gathered into the plan's single-box staging,
solved by the same kernels and scattered back, so every output is bit-identical; FAB ghost cells that the
solve does not read and FAB cells outside their box are left untouched."""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
from incflo_gb300 import (Geometry, MacProjector, _abi, apply_nodal_projection, apply_nodal_projection_boxes,
                          make_options)
from incflo_gb300.projection import array4
from tests.helpers import D, I, N, P, cuda, face_fields

pytestmark = pytest.mark.gpu


def split(n, mgs):
    """incflo's max_grid_size chop of the domain box into a BoxArray (x fastest)"""
    cuts = [list(range(0, n[d], mgs[d])) for d in range(3)]
    boxes = []
    for z0 in cuts[2]:
        for y0 in cuts[1]:
            for x0 in cuts[0]:
                lo = (x0, y0, z0)
                hi = tuple(min(lo[d] + mgs[d], n[d]) - 1 for d in range(3))
                boxes.append((lo, hi))
    return boxes


def fab(full, box, ng, off, comps=True, nodal=False):
    """copy of a FAB: box grown by ng ghost cells (nodal: nodes lo..hi+1), from an array whose index
    origin sits at `off` (the array index of cell / node 0), padded with NaN where the source has no data
    (ghost cells the solve must not read)"""
    lo, hi = box
    ext = [hi[d] - lo[d] + 1 + (1 if nodal else 2 * ng) for d in range(3)]
    shape = ((full.shape[0],) if comps else ()) + (ext[2], ext[1], ext[0])
    out = np.full(shape, np.nan)
    base = [lo[d] - (0 if nodal else ng) for d in range(3)]
    sl_src, sl_dst = [], []
    for d in (2, 1, 0):
        a0 = base[d] + off
        a1 = a0 + ext[d]
        n_full = full.shape[-3 + (2 - d)]
        s0, s1 = max(a0, 0), min(a1, n_full)
        sl_src.append(slice(s0, s1))
        sl_dst.append(slice(s0 - a0, s1 - a0))
    if comps:
        out[(slice(None),) + tuple(sl_dst)] = full[(slice(None),) + tuple(sl_src)]
    else:
        out[tuple(sl_dst)] = full[tuple(sl_src)]
    return cuda(out)


def unfab(full_shape, fabs, boxes, ng, off, comps=True, nodal=False):
    """assemble the valid region of every FAB into one array (nodal: all nodes of each box)"""
    out = np.full(full_shape, np.nan)
    for t, (lo, hi) in zip(fabs, boxes):
        a = t.cpu().numpy()
        sl_src, sl_dst = [], []
        for d in (2, 1, 0):
            m = hi[d] - lo[d] + 1 + (1 if nodal else 0)
            g0 = 0 if nodal else ng
            sl_src.append(slice(g0, g0 + m))
            sl_dst.append(slice(lo[d] + off, lo[d] + off + m))
        if comps:
            out[(slice(None),) + tuple(sl_dst)] = a[(slice(None),) + tuple(sl_src)]
        else:
            out[tuple(sl_dst)] = a[tuple(sl_src)]
    return out


NODAL = {
    "walls-periodic": ((32, 32, 24), (P, P, N), (P, P, N), (16, 16, 8)),
    "inflow-outflow": ((40, 24, 16), (I, N, P), (D, N, P), (16, 16, 16)),
}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(NODAL))
def test_nodal_projection_boxes_match_single_box(gpu_lib, name, precision):
    n, bclo, bchi, mgs = NODAL[name]
    boxes = split(n, mgs)
    assert len(boxes) > 1
    rng = np.random.default_rng(21)
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vel[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((3, n[2], n[1], n[0]))
    if bclo[0] == I:
        vel[0, :, :, 0] = 1.0
    rho = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    gp = 0.1 * rng.standard_normal((3, n[2], n[1], n[0]))
    geom = Geometry(n, (0, 0, 0), (1.0, n[1] / n[0], n[2] / n[0]))
    opts = make_options(0, precision=precision, mg_rtol=1e-11, mg_atol=0.0)
    # single box
    vt, gt = cuda(vel), cuda(gp)
    pt = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device="cuda")
    st1 = apply_nodal_projection(geom, bclo, bchi, vt, cuda(rho), gt, pt, options=opts)
    # the same level as FABs (ghost cells across inflow sides from the full array, NaN elsewhere)
    vf = [fab(vel, b, 1, 1) for b in boxes]
    rf = [fab(rho, b, 0, 0, comps=False) for b in boxes]
    gf = [fab(gp, b, 0, 0) for b in boxes]
    pf = [cuda(np.full((b[1][2] - b[0][2] + 2, b[1][1] - b[0][1] + 2, b[1][0] - b[0][0] + 2), np.nan)) for b in boxes]
    st2 = apply_nodal_projection_boxes(geom, bclo, bchi, boxes, vf, rf, gf, pf, options=opts)
    assert st1["status"] == 0 and st2["status"] == 0
    assert st1["vcycles"] == st2["vcycles"] and st1["final_rel_resid"] == st2["final_rel_resid"]
    v2 = unfab((3, n[2], n[1], n[0]), vf, boxes, 1, 0)
    np.testing.assert_array_equal(v2, vt.cpu().numpy()[:, 1:-1, 1:-1, 1:-1])
    np.testing.assert_array_equal(unfab((3, n[2], n[1], n[0]), gf, boxes, 0, 0), gt.cpu().numpy())
    np.testing.assert_array_equal(unfab((n[2] + 1, n[1] + 1, n[0] + 1), pf, boxes, 0, 0, comps=False, nodal=True),
                                  pt.cpu().numpy())
    # FAB ghost cells are inputs only: untouched
    for t, b in zip(vf, boxes):
        a = t.cpu().numpy()
        ref = fab(vel, b, 1, 1).cpu().numpy()
        for sl in ((slice(None), 0), (slice(None), -1)):
            np.testing.assert_array_equal(a[:, :, :, sl[1]], ref[:, :, :, sl[1]])


def test_nodal_boxes_reject_bad_box_arrays(gpu_lib):
    n, bclo, bchi, mgs = NODAL["walls-periodic"]
    boxes = split(n, mgs)
    geom = Geometry(n, (0, 0, 0), (1.0, 1.0, 0.75))
    z = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vf = [fab(z, b, 1, 1) for b in boxes]
    rf = [fab(np.ones((n[2], n[1], n[0])), b, 0, 0, comps=False) for b in boxes]
    gf = [fab(np.zeros((3, n[2], n[1], n[0])), b, 0, 0) for b in boxes]
    with pytest.raises(Exception, match="cover"):
        apply_nodal_projection_boxes(geom, bclo, bchi, boxes[:-1], vf[:-1], rf[:-1], gf[:-1], None)
    overlap = list(boxes)
    overlap[1] = ((overlap[1][0][0] - 1,) + tuple(overlap[1][0][1:]), overlap[1][1])
    with pytest.raises(Exception, match="overlap"):
        apply_nodal_projection_boxes(geom, bclo, bchi, overlap, vf, rf, gf, None)


MAC = {
    "walls-periodic": ((32, 24, 16), (P, N, P), (P, N, P), (16, 8, 16)),
    "inflow-outflow": ((48, 16, 16), (I, N, P), (D, N, P), (16, 16, 8)),
}


@pytest.mark.parametrize("name", list(MAC))
def test_mac_projection_boxes_match_single_box(gpu_lib, name):
    n, bclo, bchi, mgs = MAC[name]
    boxes = split(n, mgs)
    g = O.Grid(n, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(5)
    umac = face_fields(g, rng)
    rho = np.ones((n[2] + 2, n[1] + 2, n[0] + 2))
    rho[1:-1, 1:-1, 1:-1] = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    geom = Geometry(n, (0, 0, 0), (1.0, n[1] / n[0], n[2] / n[0]))  # cubic cells
    dt = 0.1
    out = []
    for multi in (False, True):
        mp = MacProjector(geom, options=make_options(1, precision="mixed", mg_rtol=1e-11, mg_atol=0.0))
        mp.initProjector(beta=1.0)
        mp.setDomainBC(bclo, bchi)
        if multi:
            mp.setBetaFromDensityBoxes(boxes, [fab(rho, b, 1, 1, comps=False) for b in boxes], dt)
            # face FABs of direction d: faces lo..hi+1 in d
            uf = [[cuda(umac[d][tuple(slice(lo[e], hi[e] + 1 + (1 if e == d else 0)) for e in (2, 1, 0))])
                   for d in range(3)] for lo, hi in boxes]
            phf = [cuda(np.zeros((b[1][2] - b[0][2] + 1, b[1][1] - b[0][1] + 1, b[1][0] - b[0][0] + 1)))
                   for b in boxes]
            st = mp.projectBoxes(boxes, uf, phf, phi_guess=False)
            u = [np.zeros_like(umac[d]) for d in range(3)]
            for bi, (lo, hi) in enumerate(boxes):
                for d in range(3):
                    sl = tuple(slice(lo[e], hi[e] + 1 + (1 if e == d else 0)) for e in (2, 1, 0))
                    u[d][sl] = uf[bi][d].cpu().numpy()
            phi = unfab((n[2], n[1], n[0]), phf, boxes, 0, 0, comps=False)
        else:
            mp._ensure()
            rt = cuda(rho)
            _abi.check(_abi.load().gbp_mac_set_beta_from_density(mp.plan.ptr, ctypes.byref(array4(rt, 1)), dt),
                       "beta")
            mp.beta = None
            ut = [cuda(x) for x in umac]
            mp.setUMAC(ut)
            pt = cuda(np.zeros((n[2], n[1], n[0])))
            st = mp.project(phi=pt, phi_guess=False)
            u = [x.cpu().numpy() for x in ut]
            phi = pt.cpu().numpy()
        assert st["status"] == 0
        out.append((st, u, phi))
    (s1, u1, p1), (s2, u2, p2) = out
    assert s1["vcycles"] == s2["vcycles"] and s1["final_rel_resid"] == s2["final_rel_resid"]
    np.testing.assert_array_equal(p1, p2)
    for d in range(3):
        np.testing.assert_array_equal(u1[d], u2[d])
