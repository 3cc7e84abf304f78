"""Cut-cell (embedded-boundary) nodal projection on the GPU against the cut-cell nodal oracle
(oracle/eb_nodal.py, a direct sparse solve of the Q1 system restricted to the fluid): flow past a
cylinder with walls and an outflow, and a singular periodic case; phi on the nodes that touch fluid
(relative L2 <= 1e-9, gauge-aligned for singular systems), projected velocity and gp on the fluid cells,
FP64 and FP32-in-FP64 forms."""
import numpy as np
import pytest
import torch

from incflo_gb300 import Geometry, apply_nodal_projection, eb, make_options
from oracle.eb_nodal import EBNodal
from tests.helpers import D, I, N, P, cuda, rel_l2

pytestmark = pytest.mark.gpu

CASES = {
    "walls-outflow": ((32, 16, 4), (2.0, 1.0, 0.25), (N, N, P), (D, N, P), (0.7, 0.5), 0.2),
    "singular": ((32, 16, 4), (2.0, 1.0, 0.25), (P, N, P), (P, N, P), (0.9, 0.45), 0.23),
}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(CASES))
def test_eb_nodal_projection_matches_oracle(gpu_lib, name, precision):
    n, ext, bclo, bchi, c, r = CASES[name]
    h = [ext[d] / n[d] for d in range(3)]
    M = eb.cylinder_moments(n, (0, 0, 0), ext, (c[0], c[1], 0.0), r, small_volfrac=1e-4)
    rng = np.random.default_rng(6)
    rho = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    sig = 1.0 / rho
    u = rng.standard_normal((3, n[2], n[1], n[0]))
    u[0] += 1.0
    gp = 0.2 * rng.standard_normal((3, n[2], n[1], n[0]))
    o = EBNodal(n, h, bclo, bchi, M)
    ref = o.project(sig, u + sig[None] * gp)
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vel[:, 1:-1, 1:-1, 1:-1] = u
    vt, gt, rt = cuda(vel), cuda(gp), cuda(rho)
    pt = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device="cuda")
    st = apply_nodal_projection(Geometry(n, (0, 0, 0), ext), bclo, bchi, vt, rt, gt, pt, set_inflow_bc=False,
                                options=make_options(0, precision=precision, mg_rtol=1e-12, mg_atol=0.0),
                                eb_moments=cuda(eb.moments_components(M)))
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    # nodes that touch fluid (all positions, periodic duplicates included)
    kap = M[..., 0, 0, 0]
    fl = np.zeros((n[2] + 1, n[1] + 1, n[0] + 1), bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                fl[dz:dz + n[2], dy:dy + n[1], dx:dx + n[0]] |= kap > 0
    got = pt.cpu().numpy()
    want = ref["phi"]
    if o.singular:
        got = got - got[fl].mean()
        want = want - want[fl].mean()
    assert rel_l2(got[fl], want[fl]) <= 1e-9
    fluid = kap > 0
    un = vt.cpu().numpy()[:, 1:-1, 1:-1, 1:-1]
    for d in range(3):
        np.testing.assert_allclose(un[d][fluid], ref["u"][d][fluid], rtol=0, atol=1e-9 * np.abs(ref["u"]).max())
        np.testing.assert_allclose(gt.cpu().numpy()[d][fluid], ref["grad"][d][fluid], rtol=0,
                                   atol=1e-9 * np.abs(ref["grad"]).max())
    # the plan drops the cut cells again when called without them
    vt2 = cuda(vel)
    st2 = apply_nodal_projection(Geometry(n, (0, 0, 0), ext), bclo, bchi, vt2, rt, cuda(gp), pt, set_inflow_bc=False,
                                 options=make_options(0, precision=precision, mg_rtol=1e-12, mg_atol=0.0))
    assert st2["status"] == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_eb_inflow_velocity_matches_oracle(gpu_lib, precision):
    """getLinOp().setEBInflowVelocity: a cylinder blowing into a channel with an inflow side and an outflow
    (incflo's eb_flow.vel_mag on the cut cells); phi, the projected velocity and gp against the cut-cell
    nodal oracle with the boundary term in its right-hand side."""
    n, ext, c, r = (32, 16, 4), (2.0, 1.0, 0.25), (0.7, 0.5), 0.2
    bclo, bchi = (I, N, P), (D, N, P)
    h = [ext[d] / n[d] for d in range(3)]
    M = eb.cylinder_moments(n, (0, 0, 0), ext, (c[0], c[1], 0.0), r, small_volfrac=1e-4)
    bd = eb.cylinder_boundary(n, (0, 0, 0), ext, (c[0], c[1], 0.0), r, small_volfrac=1e-4)
    ev = eb.eb_inflow_velocity(bd["bnorm"], vel_mag=2.0)
    rng = np.random.default_rng(8)
    rho = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    sig = 1.0 / rho
    u = rng.standard_normal((3, n[2], n[1], n[0]))
    u[0] += 1.0
    gp = np.zeros((3, n[2], n[1], n[0]))
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vel[:, 1:-1, 1:-1, 1:-1] = u
    vel[0, :, :, 0] = 1.0  # the inflow side's ghost cells
    o = EBNodal(n, h, bclo, bchi, M)
    ref = o.project(sig, u, u_ghost=vel, eb_inflow=(ev, bd["dap"], bd["bcent"]))
    vt, rt = cuda(vel), cuda(rho)
    gt = cuda(gp)
    pt = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device="cuda")
    st = apply_nodal_projection(Geometry(n, (0, 0, 0), ext), bclo, bchi, vt, rt, gt, pt, set_inflow_bc=True,
                                options=make_options(0, precision=precision, mg_rtol=1e-12, mg_atol=0.0),
                                eb_moments=cuda(eb.moments_components(M)),
                                eb_inflow=(cuda(ev), cuda(bd["dap"]), cuda(bd["bcent"])))
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    kap = M[..., 0, 0, 0]
    fl = np.zeros((n[2] + 1, n[1] + 1, n[0] + 1), bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                fl[dz:dz + n[2], dy:dy + n[1], dx:dx + n[0]] |= kap > 0
    assert rel_l2(pt.cpu().numpy()[fl], ref["phi"][fl]) <= 1e-9
    fluid = kap > 0
    un = vt.cpu().numpy()[:, 1:-1, 1:-1, 1:-1]
    for d in range(3):
        np.testing.assert_allclose(un[d][fluid], ref["u"][d][fluid], rtol=0, atol=1e-9 * np.abs(ref["u"]).max())
        np.testing.assert_allclose(gt.cpu().numpy()[d][fluid], ref["grad"][d][fluid], rtol=0,
                                   atol=1e-9 * np.abs(ref["grad"]).max())
    # the boundary source shows in the solution: without the inflow phi differs at O(1)
    ref0 = o.project(sig, u, u_ghost=vel)
    assert rel_l2(ref0["phi"][fl], ref["phi"][fl]) > 1e-2
