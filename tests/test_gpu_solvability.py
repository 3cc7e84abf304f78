"""Inflow/outflow solvability on the GPU against the oracle (both the cell-velocity form used
before the nodal projection and the face form used before the MAC projection)."""
import numpy as np
import pytest
import torch

import oracle as O
from incflo_gb300 import Geometry, MacProjector, NodalProjector

pytestmark = pytest.mark.gpu


def test_cell_form_matches_oracle(gpu_lib):
    n, ext = (16, 12, 10), (1.0, 0.75, 0.625)
    g = O.Grid(n, hi=ext, bclo=(3, 2, 3), bchi=(3, 2, 2))
    rng = np.random.default_rng(3)
    vel = rng.standard_normal((3, n[2] + 2, n[1] + 2, n[0] + 2))
    dd_lo, dd_hi = (1, 0, 1), (1, 0, 0)
    ref, inflow, outflow = O.enforce_inout_solvability(g, vel, dd_lo, dd_hi)
    vt = torch.from_numpy(vel).cuda()
    p = NodalProjector(vt, 1.0, Geometry(n, (0, 0, 0), ext))
    p.setDomainBC(["inflow", "Neumann", "inflow"], ["inflow", "Neumann", "Neumann"])
    fi, fo = p.enforceInOutSolvability(dd_lo, dd_hi)
    assert abs(fi - inflow) <= 1e-12 * abs(inflow) and abs(fo - outflow) <= 1e-12 * abs(outflow)
    np.testing.assert_allclose(vt.cpu().numpy(), ref, rtol=1e-14, atol=1e-15)


def test_face_form_matches_oracle(gpu_lib):
    n = (12, 10, 8)
    g = O.Grid(n, bclo=(2, 2, 2))
    rng = np.random.default_rng(4)
    umac = [rng.standard_normal(g.face_shape(d)) for d in range(3)]
    dd_lo, dd_hi = (1, 0, 1), (1, 1, 0)
    ref, inflow, outflow = O.mac_enforce_inout_solvability(g, umac, dd_lo, dd_hi)
    ut = [torch.from_numpy(u).cuda() for u in umac]
    mp = MacProjector(Geometry(n))
    mp.initProjector(beta=1.0)
    mp.setDomainBC(["Neumann"] * 3, ["Neumann"] * 3)
    mp.setUMAC(ut)
    fi, fo = mp.enforceInOutSolvability(dd_lo, dd_hi)
    assert abs(fi - inflow) <= 1e-12 * abs(inflow) and abs(fo - outflow) <= 1e-12 * abs(outflow)
    for d in range(3):
        np.testing.assert_allclose(ut[d].cpu().numpy(), ref[d], rtol=1e-14, atol=1e-15)


def test_average_down_matches_numpy(gpu_lib):
    """amrex::average_down of gp (3 components) over a refined region, ratio 2, into a larger
    coarse array (cells outside the region untouched)."""
    from incflo_gb300.projection import average_down

    rng = np.random.default_rng(8)
    fine = rng.standard_normal((3, 8, 12, 16))       # fine cells (z, y, x), global fine index lo (4, 6, 2)
    crse = rng.standard_normal((3, 10, 10, 12))      # coarse cells, global coarse index lo (0, 0, 0)
    ref = crse.copy()
    f = fine.reshape(3, 4, 2, 6, 2, 8, 2).mean(axis=(2, 4, 6))
    ref[:, 1:5, 3:9, 2:10] = f                       # fine lo (x4, y6, z2) -> coarse (2, 3, 1)
    ft, ct = torch.from_numpy(fine).cuda(), torch.from_numpy(crse).cuda()
    average_down(ft, ct, ratio=(2, 2, 2), fine_lo=(4, 6, 2), crse_box_lo=(0, 0, 0))
    np.testing.assert_allclose(ct.cpu().numpy(), ref, rtol=1e-15, atol=1e-15)
