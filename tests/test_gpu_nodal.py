"""Nodal projection on the GPU (through the C ABI) against the CPU oracle.

Parity bar: phi relative L2 <= 1e-9 (gauge: zero volume-weighted mean on singular systems),
projected velocity and grad(phi) within 1e-9 of the oracle's scale, final relative residual
<= the requested tolerance. Both the plain FP64 form and the mixed form (FP32 V-cycles inside
FP64 iterative refinement) must meet it: the FP64 outer residual decides convergence.
"""
import numpy as np
import pytest
import torch

import oracle as O
from incflo_gb300 import Geometry, NodalProjector, apply_nodal_projection, make_options
from tests.helpers import D, I, N, P, cuda, nodal_case, rel_l2, unique_nodes

pytestmark = pytest.mark.gpu

CASES = [
    ((16, 16, 16), (1.0, 1.0, 1.0), (P, P, P), (P, P, P)),
    ((16, 12, 20), (1.0, 0.75, 1.25), (P, P, N), (P, P, N)),
    ((12, 16, 8), (1.5, 2.0, 1.0), (N, D, P), (I, N, P)),
    ((16, 8, 8), (1.0, 1.0, 0.5), (D, N, N), (D, I, D)),   # anisotropic spacing
    ((24, 20, 32), (1.0, 0.8, 0.4), (P, N, N), (P, N, D)),  # aspect ratio 3.3: the smoother weight is capped
    ((10, 12, 14), (1.0, 1.2, 1.4), (N, N, N), (N, N, N)),  # odd coarse sizes
    ((2, 2, 2), (1.0, 1.0, 1.0), (P, N, N), (P, N, N)),     # bottom-only hierarchy
    ((32, 32, 32), (1.0, 1.0, 1.0), (P, P, N), (P, P, N)),
]


_ORACLE = {}


def _run(case, precision, graphs=True, seed=0):
    n, ext, bclo, bchi = case
    g, sigma, vel = nodal_case(n, ext, bclo, bchi, seed=seed)
    key = (case, seed)
    if key not in _ORACLE:  # one oracle solve per case (both precisions compare against it)
        _ORACLE[key] = O.nodal_project(g, sigma, vel, rtol=1e-13)
    vel_or, phi_or, grad_or, st_or = _ORACLE[key]
    assert st_or["status"] == 0
    vt = cuda(vel)
    opts = make_options(0, precision=precision, use_graphs=int(graphs))
    proj = NodalProjector(vt, cuda(sigma), Geometry(n, (0, 0, 0), ext), options=opts)
    proj.setDomainBC(bclo, bchi)
    st = proj.project(rtol=1e-12, atol=0.0)
    phi = unique_nodes(g, proj.getPhi().cpu().numpy())
    return g, st, st_or, phi, phi_or, vt.cpu().numpy(), vel_or, proj.getGradPhi().cpu().numpy(), grad_or


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[2]}-{c[3]}" for c in CASES])
def test_nodal_project_matches_oracle(gpu_lib, case, precision):
    g, st, st_or, phi, phi_or, vel, vel_or, grad, grad_or = _run(case, precision)
    assert st["status"] == 0, st
    assert st["final_rel_resid"] <= 1e-12
    assert rel_l2(phi, phi_or) <= 1e-9, (rel_l2(phi, phi_or), st)
    scale = np.abs(vel_or[:, 1:-1, 1:-1, 1:-1]).max()
    assert np.abs(vel[:, 1:-1, 1:-1, 1:-1] - vel_or[:, 1:-1, 1:-1, 1:-1]).max() <= 1e-9 * scale
    assert np.abs(grad - grad_or).max() <= 1e-9 * max(np.abs(grad_or).max(), 1e-30)
    # ghost cells are never written
    np.testing.assert_array_equal(vel[:, 0], vel_or[:, 0])


LARGE = [((176, 176, 168), (1.0, 1.0, 168 / 176), (P, P, N), (P, P, N)),
         ((192, 136, 100), (1.0, 136 / 192, 100 / 192), (P, D, N), (P, I, D))]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", LARGE, ids=["periodic-xy", "dirichlet-inflow"])
def test_large_level_tma_sweeps_match_oracle(gpu_lib, precision, case):
    """Levels above the size where the TMA-staged z-marching sweeps take over from the
    one-node-per-thread kernels (5.4 M and 2.7 M nodes; the mixed form runs the whole-row FP32
    sweeps with the fused residual + restriction and prolongation + sweep on its two finest levels),
    periodic, wall, Dirichlet and inflow sides."""
    g, st, st_or, phi, phi_or, vel, vel_or, grad, grad_or = _run(case, precision)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    assert rel_l2(phi, phi_or) <= 1e-9
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))
    np.testing.assert_allclose(vel[inner], vel_or[inner], rtol=0, atol=1e-9 * np.abs(vel_or[inner]).max())


def test_nodal_graphs_and_direct_launch_agree(gpu_lib):
    case = CASES[1]
    a = _run(case, "fp64", graphs=True)
    b = _run(case, "fp64", graphs=False)
    np.testing.assert_array_equal(a[3], b[3])
    assert a[1]["outer_iters"] == b[1]["outer_iters"]


def test_nodal_plan_reuse_is_deterministic(gpu_lib):
    case = CASES[2]
    a = _run(case, "mixed")
    b = _run(case, "mixed")
    np.testing.assert_array_equal(a[3], b[3])


def test_apply_nodal_projection_fused_semantics(gpu_lib):
    """incflo::ApplyNodalProjection (non-incremental and incremental) against the oracle composition."""
    n, ext, bclo, bchi = (16, 16, 16), (1.0, 1.0, 1.0), (P, P, N), (P, P, N)
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(4)
    rho = rng.uniform(1.0, 3.0, g.cell_shape)
    s = 0.01
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vel[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((3,) + g.cell_shape)
    vel_o = rng.standard_normal((3,) + g.cell_shape)
    gp = rng.standard_normal((3,) + g.cell_shape)
    p_nd = rng.standard_normal((n[2] + 1, n[1] + 1, n[0] + 1))
    sigma = s / rho
    for incremental in (False, True):
        # oracle composition of incflo_apply_nodal_projection.cpp:29-93, 221-256
        v = vel.copy()
        if not incremental:
            v[:, 1:-1, 1:-1, 1:-1] += gp * sigma
        else:
            v[:, 1:-1, 1:-1, 1:-1] -= vel_o
        vn, phi_or, grad_or, st = O.nodal_project(g, sigma, v, rtol=1e-13)
        if incremental:
            vn[:, 1:-1, 1:-1, 1:-1] += vel_o
        gp_ref = gp + grad_or if incremental else grad_or
        vt, gpt, pt = cuda(vel), cuda(gp), cuda(p_nd)
        st = apply_nodal_projection(Geometry(n, (0, 0, 0), ext), bclo, bchi, vt, cuda(rho), gpt, pt,
                                    time=1.0, dt=s, prev_dt=s, scaling_factor=s, incremental=incremental,
                                    vel_old=cuda(vel_o), options=make_options(0, mg_rtol=1e-12, mg_atol=0))
        assert st["status"] == 0
        p_gpu = pt.cpu().numpy()
        phi_gpu = unique_nodes(g, p_gpu - p_nd) if incremental else unique_nodes(g, p_gpu)
        assert rel_l2(phi_gpu, phi_or) <= 1e-9
        np.testing.assert_allclose(vt.cpu().numpy()[:, 1:-1, 1:-1, 1:-1], vn[:, 1:-1, 1:-1, 1:-1], rtol=0,
                                   atol=1e-9 * np.abs(vn).max())
        np.testing.assert_allclose(gpt.cpu().numpy(), gp_ref, rtol=0, atol=1e-9 * np.abs(gp_ref).max())
        # periodic duplicate nodes of p_nd carry the same value (p_nd is overwritten, not accumulated)
        if not incremental:
            np.testing.assert_array_equal(p_gpu[:, :, -1], p_gpu[:, :, 0])
            np.testing.assert_array_equal(p_gpu[:, -1, :], p_gpu[:, 0, :])


@pytest.mark.parametrize("case", CASES[:4], ids=[f"{c[0]}-{c[2]}-{c[3]}" for c in CASES[:4]])
def test_nodal_divergence_matches_oracle(gpu_lib, case):
    from incflo_gb300.projection import nodal_divergence

    n, ext, bclo, bchi = case
    g, sigma, vel = nodal_case(n, ext, bclo, bchi, seed=5)
    rhs = O.nodal_rhs(g, vel)
    V = O.nodal_volume(g)
    if D not in bclo + bchi:
        rhs = rhs - V * rhs.sum() / V.sum()
    ref = -rhs / V
    m, out = nodal_divergence(Geometry(n, (0, 0, 0), ext), bclo, bchi, cuda(vel))
    div = unique_nodes(g, out.cpu().numpy())
    np.testing.assert_allclose(div, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    assert abs(m - np.abs(ref).max()) <= 1e-12 * np.abs(ref).max()


def test_divergence_after_projection_no_worse_than_oracle(gpu_lib):
    case = ((24, 24, 24), (1.0, 1.0, 1.0), (P, P, N), (P, P, N))
    g, st, st_or, phi, phi_or, vel, vel_or, grad, grad_or = _run(case, "mixed", seed=3)
    div_gpu = np.abs(O.nodal_rhs(g, vel)).max()
    div_or = np.abs(O.nodal_rhs(g, vel_or)).max()
    assert div_gpu <= div_or * (1 + 1e-6) + 1e-12


def test_not_converged_status_and_bad_args(gpu_lib):
    from incflo_gb300 import ProjectionError

    n = (16, 16, 16)
    g, sigma, vel = nodal_case(n, (1, 1, 1), (P, P, P), (P, P, P), seed=1)
    proj = NodalProjector(cuda(vel), cuda(sigma), Geometry(n), options=make_options(0, maxiter=1))
    proj.setDomainBC((P, P, P), (P, P, P))
    with pytest.raises(ProjectionError) as e:
        proj.project(rtol=1e-14, atol=0)
    assert e.value.status == 1
    bad = NodalProjector(cuda(vel[:, 1:-1]), cuda(sigma), Geometry(n))
    bad.setDomainBC((P, P, P), (P, P, P))
    with pytest.raises(ProjectionError) as e:
        bad.project()
    assert e.value.status == 3


def test_nan_rhs_reported(gpu_lib):
    from incflo_gb300 import ProjectionError

    n = (8, 8, 8)
    g, sigma, vel = nodal_case(n, (1, 1, 1), (P, P, N), (P, P, N), seed=2)
    vel[0, 3, 3, 3] = np.nan
    proj = NodalProjector(cuda(vel), cuda(sigma), Geometry(n))
    proj.setDomainBC((P, P, N), (P, P, N))
    with pytest.raises(ProjectionError) as e:
        proj.project()
    assert e.value.status == 2
    torch.cuda.synchronize()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overset_mask_matches_oracle(gpu_lib, precision):
    """incflo's mixed boundaries on the nodal side: an overset mask (0 = phi held at 0) over part of
    the high-x face and a patch of the low-z face of an otherwise all-Neumann box (which the mask
    makes nonsingular), against the oracle with the same mask."""
    n, ext, bclo, bchi = (16, 12, 10), (1.0, 0.75, 0.625), (N, N, N), (I, N, N)
    g0, sigma, vel = nodal_case(n, ext, bclo, bchi, seed=4)
    nn = g0.node_shape
    mask = np.ones(nn, np.int32)
    mask[:, : nn[1] // 2, -1] = 0          # outflow part of the high-x face
    mask[0, 2:6, 3:9] = 0                  # a patch on the low-z face
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi, mask=mask.astype(np.uint8))
    vel_or, phi_or, grad_or, st_or = O.nodal_project(g, sigma, vel, rtol=1e-13)
    assert st_or["status"] == 0
    vt = cuda(vel)
    proj = NodalProjector(vt, cuda(sigma), Geometry(n, (0, 0, 0), ext),
                          options=make_options(0, precision=precision))
    proj.setDomainBC(bclo, bchi)
    full = np.ones((n[2] + 1, n[1] + 1, n[0] + 1), np.int32)
    full[: nn[0], : nn[1], : nn[2]] = mask
    proj.setOversetMask(torch.from_numpy(full).cuda())
    st = proj.project(rtol=1e-12, atol=0.0)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    phi = unique_nodes(g, proj.getPhi().cpu().numpy())
    assert np.abs(phi[mask == 0]).max() == 0.0
    assert rel_l2(phi, phi_or) <= 1e-9
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))
    got = vt.cpu().numpy()
    np.testing.assert_allclose(got[inner], vel_or[inner], rtol=0, atol=1e-9 * np.abs(vel_or[inner]).max())
    proj.setOversetMask(None)  # the shared plan goes back to the unmasked operator


def test_whole_row_sweeps_with_overset_mask(gpu_lib):
    """A level with an overset mask (masked nodes held at 0, as on the fine level of a composite solve):
    a 128^3 mixed-form projection with slabs held at 0 below and above against the oracle (the masked
    level runs the whole-row Jacobi and residual sweeps, its transfers the plain kernels), and the
    whole-row sweeps against the one-node-per-thread kernels over every padded position, with that mask
    and with a mask that varies within the planes."""
    import ctypes

    from incflo_gb300 import _abi

    n, ext, bclo, bchi = (128, 128, 128), (1.0, 1.0, 1.0), (P, P, N), (P, P, N)
    g0, sigma, vel = nodal_case(n, ext, bclo, bchi, seed=12)
    nn = g0.node_shape
    mask = np.ones(nn, np.int32)
    mask[:16] = 0
    mask[112:] = 0
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi, mask=mask.astype(np.uint8))
    vel_or, phi_or, grad_or, st_or = O.nodal_project(g, sigma, vel, rtol=1e-13)
    assert st_or["status"] == 0
    vt = cuda(vel)
    proj = NodalProjector(vt, cuda(sigma), Geometry(n, (0, 0, 0), ext), options=make_options(0, precision="mixed"))
    proj.setDomainBC(bclo, bchi)

    def set_mask(m):
        full = np.ones((n[2] + 1, n[1] + 1, n[0] + 1), np.int32)
        full[: nn[0], : nn[1], : nn[2]] = m
        proj.setOversetMask(torch.from_numpy(full).cuda())

    def check_kernels(label):
        diff = (ctypes.c_double * 4)()
        _abi.check(_abi.load().gbp_plan_check_level_kernels(proj._plan().ptr, diff), "check_level_kernels")
        print(f"\n{label}: jacobi {diff[0]:.2e} resid {diff[1]:.2e}")
        assert 0.0 <= diff[0] <= 1e-5 and 0.0 <= diff[1] <= 1e-5
        assert diff[2] == -1.0 and diff[3] == -1.0

    set_mask(mask)
    try:
        st = proj.project(rtol=1e-12, atol=0.0)
        assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
        phi = unique_nodes(g, proj.getPhi().cpu().numpy())
        assert np.abs(phi[mask == 0]).max() == 0.0
        assert rel_l2(phi, phi_or) <= 1e-9
        check_kernels("masked slabs")
        hole = mask.copy()
        hole[:, 40:60, 30:90] = 0
        set_mask(hole)
        check_kernels("masked slabs and a hole")
    finally:
        proj.setOversetMask(None)  # the shared plan goes back to the unmasked operator


@pytest.mark.parametrize("case", [((256, 256, 256), (1.0, 1.0, 1.0), (P, P, N), (P, P, N)), LARGE[1],
                                  ((512, 64, 64), (8.0, 1.0, 1.0), (P, P, N), (P, P, N))],
                         ids=["256-periodic-xy", "192-dirichlet-inflow", "512-rows"])
def test_whole_row_level_kernels_match_plain_kernels(gpu_lib, case):
    """The FP32 whole-row sweeps (Jacobi, residual, fused residual + restriction, fused prolongation +
    Jacobi) against the one-node-per-thread kernels on seeded level data (the plan's sigma), over every
    padded position including the periodic aliases. Both compute in FP32 with different association, so
    they agree to FP32 rounding; an indexing fault would differ by O(1)."""
    import ctypes

    from incflo_gb300 import _abi

    n, ext, bclo, bchi = case
    g, sigma, vel = nodal_case(n, ext, bclo, bchi, seed=9)
    proj = NodalProjector(cuda(vel), cuda(sigma), Geometry(n, (0, 0, 0), ext),
                          options=make_options(0, precision="mixed"))
    proj.setDomainBC(bclo, bchi)
    st = proj.project(rtol=1e-10, atol=0.0)
    assert st["status"] == 0
    diff = (ctypes.c_double * 4)()
    _abi.check(_abi.load().gbp_plan_check_level_kernels(proj._plan().ptr, diff), "check_level_kernels")
    print(f"\n{n}: jacobi {diff[0]:.2e} resid {diff[1]:.2e} resid+restrict {diff[2]:.2e} "
          f"prolong+jacobi {diff[3]:.2e}")
    assert max(diff) <= 1e-5


@pytest.mark.parametrize("case", [((64, 64, 64), (1.0, 1.0, 1.0), (P, P, N), (P, P, N)),
                                  ((48, 32, 64), (1.2, 0.8, 1.6), (D, N, I), (N, D, N)),
                                  ((32, 32, 32), (1.0, 1.0, 1.0), (P, P, P), (P, P, P))],
                         ids=["64-periodic-xy", "48x32x64-mixed", "32-periodic"])
def test_cluster_coarse_cycle_matches_per_level_launches(gpu_lib, case):
    """The small levels of the hierarchy run as one thread-block-cluster launch per V-cycle. On a seeded
    right-hand side, one V-cycle from the first such level agrees with the per-level launches to FP32
    rounding (the prolongation sums in another order); an indexing or synchronisation fault would differ
    by O(1). A projection through the cluster path then matches the oracle (the parity tests run it in
    both precisions on every plan with such levels)."""
    import ctypes

    from incflo_gb300 import _abi

    n, ext, bclo, bchi = case
    g, sigma, vel = nodal_case(n, ext, bclo, bchi, seed=11)
    vel_or, phi_or, _, _ = O.nodal_project(g, sigma, vel, rtol=1e-13)
    for precision in ("mixed", "fp64"):
        vt = cuda(vel)
        proj = NodalProjector(vt, cuda(sigma), Geometry(n, (0, 0, 0), ext),
                              options=make_options(0, precision=precision))
        proj.setDomainBC(bclo, bchi)
        st = proj.project(rtol=1e-12, atol=0.0)
        assert st["status"] == 0
        phi = proj.getPhi().cpu().numpy()[: g.node_shape[0], : g.node_shape[1], : g.node_shape[2]]
        assert rel_l2(phi, phi_or) <= 1e-9
    diff = ctypes.c_double()
    _abi.check(_abi.load().gbp_plan_check_coarse_cycle(proj._plan().ptr, ctypes.byref(diff)), "check_coarse_cycle")
    print(f"\n{n}: cluster vs per-level V-cycle {diff.value:.2e}")
    assert diff.value <= 1e-5
