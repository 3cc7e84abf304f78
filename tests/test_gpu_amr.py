"""Two-level (AMR) composite nodal projection on the GPU against the composite oracle
(oracle/amr_nodal.py, a direct sparse solve of the conforming composite system): phi on both levels
(relative L2 <= 1e-9), projected velocities and gp per level, for walls + outflow, a singular periodic
case, and a fine region that spans a periodic direction; FP64 and FP32-in-FP64 forms."""
import numpy as np
import pytest
import torch

from incflo_gb300 import AmrNodalProjector, Geometry, make_options
from oracle.amr_nodal import CompositeNodal
from tests.helpers import D, N, P, cuda, rel_l2

pytestmark = pytest.mark.gpu

CASES = {
    "walls-outflow": ((16, 12, 8), (1.0, 0.75, 0.5), (N, N, N), (N, D, N),
                      [((4, 4, 2), (19, 13, 11)), ((20, 6, 4), (27, 13, 9))]),
    "periodic": ((16, 16, 8), (1.0, 1.0, 0.5), (P, P, N), (P, P, N),
                 [((6, 8, 4), (21, 23, 11)), ((22, 10, 4), (29, 19, 9))]),
    "spanning": ((16, 8, 8), (1.0, 0.5, 0.5), (P, N, N), (P, N, D),
                 [((0, 4, 4), (31, 11, 11))]),
}


def _case(name, seed=5):
    n, ext, bclo, bchi, boxes = CASES[name]
    nf = [2 * v for v in n]
    h = [ext[d] / n[d] for d in range(3)]
    rng = np.random.default_rng(seed)
    rho_c = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    rho_f = rng.uniform(0.5, 2.0, (nf[2], nf[1], nf[0]))
    u_c = rng.standard_normal((3, n[2], n[1], n[0]))
    u_f = rng.standard_normal((3, nf[2], nf[1], nf[0]))
    gp_c = 0.3 * rng.standard_normal((3, n[2], n[1], n[0]))
    gp_f = 0.3 * rng.standard_normal((3, nf[2], nf[1], nf[0]))
    fm = np.zeros((nf[2], nf[1], nf[0]), bool)
    for lo, hi in boxes:
        fm[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = True
    return n, nf, ext, h, bclo, bchi, boxes, rho_c, rho_f, u_c, u_f, gp_c, gp_f, fm


def _box(a, lo, hi, nodes=False):
    e = 1 if nodes else 0
    return a[..., lo[2]:hi[2] + 1 + e, lo[1]:hi[1] + 1 + e, lo[0]:hi[0] + 1 + e]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(CASES))
def test_amr_composite_projection_matches_oracle(gpu_lib, name, precision):
    n, nf, ext, h, bclo, bchi, boxes, rho_c, rho_f, u_c, u_f, gp_c, gp_f, fm = _case(name)
    s = 1.0
    sig_c, sig_f = s / rho_c, s / rho_f
    # non-incremental: the projection sees u + s gp / rho
    ref = CompositeNodal(n, h, bclo, bchi, fm).project(sig_c, sig_f, u_c + sig_c[None] * gp_c,
                                                       u_f + sig_f[None] * gp_f)
    proj = AmrNodalProjector(Geometry(n, (0, 0, 0), ext), bclo, bchi, boxes,
                             options=make_options(0, precision=precision, mg_rtol=1e-12, mg_atol=0.0))
    vel_c, gpc, rc = cuda(u_c), cuda(gp_c), cuda(rho_c)
    p_c = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device="cuda")
    vel_f = [cuda(_box(u_f, lo, hi)) for lo, hi in boxes]
    gp_fb = [cuda(_box(gp_f, lo, hi)) for lo, hi in boxes]
    rho_fb = [cuda(_box(rho_f, lo, hi)) for lo, hi in boxes]
    p_f = [torch.zeros((hi[2] - lo[2] + 2, hi[1] - lo[1] + 2, hi[0] - lo[0] + 2), dtype=torch.float64,
                       device="cuda") for lo, hi in boxes]
    st = proj.apply(vel_c, rc, gpc, p_c, vel_f, rho_fb, gp_fb, p_f, scaling_factor=s)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    assert st["outer_iters"] <= 40
    assert rel_l2(p_c.cpu().numpy(), ref["phi_c"]) <= 1e-9
    np.testing.assert_allclose(vel_c.cpu().numpy(), ref["u_c"], rtol=0, atol=1e-9 * np.abs(ref["u_c"]).max())
    np.testing.assert_allclose(gpc.cpu().numpy(), ref["gphi_c"], rtol=0, atol=1e-9 * np.abs(ref["gphi_c"]).max())
    for b, (lo, hi) in enumerate(boxes):
        pf_ref = _box(ref["phi_f"], lo, hi, nodes=True)
        assert rel_l2(p_f[b].cpu().numpy(), pf_ref) <= 1e-9
        uf_ref = _box(ref["u_f"], lo, hi)
        np.testing.assert_allclose(vel_f[b].cpu().numpy(), uf_ref, rtol=0, atol=1e-9 * np.abs(uf_ref).max())
        gf_ref = _box(ref["gphi_f"], lo, hi)
        np.testing.assert_allclose(gp_fb[b].cpu().numpy(), gf_ref, rtol=0, atol=1e-9 * np.abs(gf_ref).max())


def test_amr_rejects_bad_boxes(gpu_lib):
    g = Geometry((8, 8, 8))
    with pytest.raises(Exception):
        AmrNodalProjector(g, (N, N, N), (N, N, N), [((1, 0, 0), (4, 3, 3))])  # not whole coarse cells
    with pytest.raises(Exception):
        AmrNodalProjector(g, (N, N, N), (N, N, N), [((0, 0, 0), (7, 7, 7)), ((6, 0, 0), (9, 3, 3))])  # overlap


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_amr_tagged_many_boxes_matches_oracle(gpu_lib, precision):
    """The benchmark's two-level construction at a 16^3 base: the fine level from tagging (interface +-0.1 or
    vorticity above its 90th percentile, blocking_factor 8, max_grid_size 16 at this size) in many boxes,
    against the composite oracle on both levels."""
    from incflo_gb300 import synth

    w = synth.rt_amr_tagged(16, blocking=8, max_grid=16)
    b, boxes = w["base"], w["boxes"]
    assert len(boxes) > 8
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
    ref = CompositeNodal(nc, [1.0 / v for v in nc], b["bclo"], b["bchi"], fm).project(1.0 / b["rho"], 1.0 / rho_f,
                                                                                      b["vel"], u_f)
    proj = AmrNodalProjector(Geometry(nc, b["lo"], b["hi"]), b["bclo"], b["bchi"], boxes,
                             options=make_options(0, precision=precision, mg_rtol=1e-12, mg_atol=0.0))
    vc = cuda(b["vel"])
    pc = torch.zeros((nc[2] + 1, nc[1] + 1, nc[0] + 1), dtype=torch.float64, device="cuda")
    vf = [cuda(v) for v in w["vel_f"]]
    pf = [torch.zeros((hi[2] - lo[2] + 2, hi[1] - lo[1] + 2, hi[0] - lo[0] + 2), dtype=torch.float64,
                      device="cuda") for lo, hi in boxes]
    st = proj.apply(vc, cuda(b["rho"]), torch.zeros_like(vc), pc, vf, [cuda(r) for r in w["rho_f"]],
                    [torch.zeros_like(v) for v in vf], pf, scaling_factor=1.0)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    assert rel_l2(pc.cpu().numpy(), ref["phi_c"]) <= 1e-9
    for t, (lo, hi) in zip(pf, boxes):
        assert rel_l2(t.cpu().numpy(), ref["phi_f"][lo[2]:hi[2] + 2, lo[1]:hi[1] + 2, lo[0]:hi[0] + 2]) <= 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_amr_previous_phi_start(gpu_lib, precision):
    """initial_guess = previous on the composite solve: the second projection of a box layout starts from
    the first one's phi on both levels. With every input scaled by 1.1 the start's residual is about a
    tenth of the right-hand side's, and phi comes out 1.1 times the oracle's."""
    n, nf, ext, h, bclo, bchi, boxes, rho_c, rho_f, u_c, u_f, gp_c, gp_f, fm = _case("walls-outflow")
    sig_c, sig_f = 1.0 / rho_c, 1.0 / rho_f
    ref = CompositeNodal(n, h, bclo, bchi, fm).project(sig_c, sig_f, u_c + sig_c[None] * gp_c,
                                                       u_f + sig_f[None] * gp_f)
    proj = AmrNodalProjector(Geometry(n, (0, 0, 0), ext), bclo, bchi, boxes,
                             options=make_options(0, precision=precision, mg_rtol=1e-12, mg_atol=0.0,
                                                  initial_guess="previous"))
    stats = []
    for scale in (1.0, 1.1):
        vel_c, gpc, rc = cuda(scale * u_c), cuda(scale * gp_c), cuda(rho_c)
        p_c = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device="cuda")
        vel_f = [cuda(_box(scale * u_f, lo, hi)) for lo, hi in boxes]
        gp_fb = [cuda(_box(scale * gp_f, lo, hi)) for lo, hi in boxes]
        rho_fb = [cuda(_box(rho_f, lo, hi)) for lo, hi in boxes]
        p_f = [torch.zeros((hi[2] - lo[2] + 2, hi[1] - lo[1] + 2, hi[0] - lo[0] + 2), dtype=torch.float64,
                           device="cuda") for lo, hi in boxes]
        st = proj.apply(vel_c, rc, gpc, p_c, vel_f, rho_fb, gp_fb, p_f, scaling_factor=1.0)
        assert st["status"] == 0
        stats.append(st)
    assert stats[0]["prev_rel_resid"] == 0.0
    assert 0.01 < stats[1]["prev_rel_resid"] < 0.5, stats[1]
    assert rel_l2(p_c.cpu().numpy(), 1.1 * ref["phi_c"]) <= 1e-9
    for b, (lo, hi) in enumerate(boxes):
        assert rel_l2(p_f[b].cpu().numpy(), 1.1 * _box(ref["phi_f"], lo, hi, nodes=True)) <= 1e-9
