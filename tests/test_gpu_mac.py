"""MAC projection on the GPU (through the C ABI) against the CPU oracle: phi relative L2 <= 1e-9,
corrected face velocities within 1e-9 of scale, discrete divergence removed to solver tolerance."""
import numpy as np
import pytest

import oracle as O
from incflo_gb300 import Geometry, MacProjector, make_options
from tests.helpers import D, I, N, P, cuda, face_fields, rel_l2

pytestmark = pytest.mark.gpu

CASES = [
    ((16, 16, 16), (1.0, 1.0, 1.0), (P, P, P), (P, P, P)),
    ((16, 12, 20), (1.0, 0.75, 1.25), (P, N, D), (P, I, N)),
    ((8, 16, 8), (1.0, 1.0, 0.5), (D, D, N), (N, D, D)),
    ((12, 12, 12), (1.0, 1.0, 1.0), (N, N, N), (N, N, N)),
    ((32, 32, 32), (1.0, 1.0, 1.0), (P, P, N), (P, P, N)),
]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[2]}-{c[3]}" for c in CASES])
def test_mac_project_matches_oracle(gpu_lib, case, precision):
    n, ext, bclo, bchi = case
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(1)
    beta = face_fields(g, rng, zero_neumann=False)
    beta = [np.abs(b) + 0.2 for b in beta]
    umac = face_fields(g, rng)
    un_or, phi_or, st_or = O.mac_project(g, beta, umac, rtol=1e-13)
    assert st_or["status"] == 0
    ut = [cuda(u) for u in umac]
    mp = MacProjector(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision=precision))
    mp.initProjector(beta=[cuda(b) for b in beta])
    mp.setDomainBC(bclo, bchi)
    mp.setUMAC(ut)
    phi = cuda(np.zeros(g.cell_shape))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi, phi_guess=False)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    assert rel_l2(phi.cpu().numpy(), phi_or) <= 1e-9
    for d in range(3):
        ref = un_or[d]
        np.testing.assert_allclose(ut[d].cpu().numpy(), ref, rtol=0, atol=1e-9 * np.abs(ref).max())


def test_mac_phi_initial_guess_and_constant_beta(gpu_lib):
    """project(phi, rtol, atol) with phi as the initial guess (use_mac_phi_in_godunov path) and
    the constant-density initProjector(ba, dm, info, dt/rho0) form."""
    n, ext, bclo, bchi = (16, 16, 16), (1.0, 1.0, 1.0), (P, P, N), (P, P, N)
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(2)
    umac = face_fields(g, rng)
    beta_c = 0.02
    beta = [np.full(g.face_shape(d), beta_c) for d in range(3)]
    un_or, phi_or, st_or = O.mac_project(g, beta, umac, rtol=1e-13)
    mp = MacProjector(Geometry(n, (0, 0, 0), ext))
    mp.initProjector(beta=beta_c)
    mp.setDomainBC(bclo, bchi)
    ut = [cuda(u) for u in umac]
    mp.setUMAC(ut)
    phi = cuda(phi_or + 1e-3 * rng.standard_normal(phi_or.shape))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi)
    assert st["status"] == 0 and st["initial_rel_resid"] < 0.1
    assert rel_l2(phi.cpu().numpy(), phi_or) <= 1e-9
    for d in range(3):
        np.testing.assert_allclose(ut[d].cpu().numpy(), un_or[d], rtol=0, atol=1e-9 * np.abs(un_or[d]).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_mac_robin_faces_match_oracle(gpu_lib, precision):
    """Robin sides (incflo's mixed BC: Neumann where a = 0, Dirichlet where b = 0, in between for
    a, b > 0) against the oracle, where a Robin face with f = 0 is a zero-value Dirichlet face of
    half its effective weight beta a h / (a h / 2 + b)."""
    n, ext = (16, 12, 10), (1.0, 0.75, 0.625)
    bclo, bchi = (O.NEUMANN, P, 4), (4, P, O.NEUMANN)
    rng = np.random.default_rng(7)
    g_or = O.Grid(n, hi=ext, bclo=(O.NEUMANN, P, D), bchi=(D, P, O.NEUMANN))
    beta = [np.abs(b) + 0.2 for b in face_fields(g_or, rng, zero_neumann=False)]
    umac = face_fields(g_or, rng)
    ra = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2))
    rb = np.zeros_like(ra)
    # high-x side: outflow half (Dirichlet), inflow half (Neumann); low-z side: a, b > 0 both
    ra[1:-1, 1:-1, -1] = np.where(np.arange(n[1])[None, :] < n[1] // 2, 1.0, 0.0)
    rb[1:-1, 1:-1, -1] = 1.0 - ra[1:-1, 1:-1, -1]
    ra[0, 1:-1, 1:-1] = rng.uniform(0.5, 2.0, (n[1], n[0]))
    rb[0, 1:-1, 1:-1] = rng.uniform(0.01, 0.1, (n[1], n[0]))
    h = [ext[d] / n[d] for d in range(3)]
    beta_or = [b.copy() for b in beta]
    a_x, b_x = ra[1:-1, 1:-1, -1], rb[1:-1, 1:-1, -1]
    beta_or[0][:, :, -1] = beta[0][:, :, -1] * (a_x * h[0] / (a_x * h[0] / 2 + b_x)) / 2
    a_z, b_z = ra[0, 1:-1, 1:-1], rb[0, 1:-1, 1:-1]
    beta_or[2][0, :, :] = beta[2][0, :, :] * (a_z * h[2] / (a_z * h[2] / 2 + b_z)) / 2
    un_or, phi_or, st_or = O.mac_project(g_or, beta_or, umac, rtol=1e-13)
    assert st_or["status"] == 0
    mp = MacProjector(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision=precision))
    mp.initProjector(beta=[cuda(b) for b in beta])
    mp.setDomainBC(bclo, bchi)
    mp.setLevelBC(0, None, cuda(ra), cuda(rb), None)
    ut = [cuda(u) for u in umac]
    mp.setUMAC(ut)
    phi = cuda(np.zeros(g_or.cell_shape))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi, phi_guess=False)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    assert rel_l2(phi.cpu().numpy(), phi_or) <= 1e-9
    for d in range(3):
        np.testing.assert_allclose(ut[d].cpu().numpy(), un_or[d], rtol=0, atol=1e-9 * np.abs(un_or[d]).max())


def test_mac_robin_rejects_bad_data(gpu_lib):
    n = (8, 8, 8)
    mp = MacProjector(Geometry(n))
    mp.initProjector(beta=1.0)
    mp.setDomainBC((4, O.NEUMANN, O.NEUMANN), (O.NEUMANN, O.NEUMANN, O.NEUMANN))
    z = cuda(np.zeros((10, 10, 10)))
    with pytest.raises(Exception):
        mp.setLevelBC(0, None, z, z, None)  # a = b = 0: no boundary condition
        mp._ensure()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_mac_all_neumann_inconsistent_rhs(gpu_lib, precision):
    """Walls all round with non-zero wall-normal velocities: the divergence has a non-zero sum, the
    singular system is made consistent by removing its mean (as the oracle does) before the solve."""
    n, ext, bc = (16, 12, 8), (2.0, 1.5, 1.0), (N, N, N)
    g = O.Grid(n, hi=ext, bclo=bc, bchi=bc)
    rng = np.random.default_rng(11)
    beta = [np.abs(b) + 0.2 for b in face_fields(g, rng, zero_neumann=False)]
    umac = face_fields(g, rng, zero_neumann=False)
    un_or, phi_or, st_or = O.mac_project(g, beta, umac, rtol=1e-13)
    assert st_or["status"] == 0
    mp = MacProjector(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision=precision))
    mp.initProjector(beta=[cuda(b) for b in beta])
    mp.setDomainBC(bc, bc)
    ut = [cuda(u) for u in umac]
    mp.setUMAC(ut)
    phi = cuda(np.zeros(g.cell_shape))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi, phi_guess=False)
    assert st["status"] == 0
    assert rel_l2(phi.cpu().numpy(), phi_or) <= 1e-9
    for d in range(3):
        np.testing.assert_allclose(ut[d].cpu().numpy(), un_or[d], rtol=0, atol=1e-9 * np.abs(un_or[d]).max())


@pytest.mark.parametrize("case", [CASES[1], CASES[4]], ids=["dirichlet-inflow", "periodic-walls"])
def test_get_fluxes_are_the_projection_correction(gpu_lib, case):
    """MacProjector::getFluxes(fluxes, phi) = -beta grad phi on every face: against the oracle's
    correction (u_projected - u) from the same solve, and against the GPU's own correction."""
    n, ext, bclo, bchi = case
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(5)
    beta = [np.abs(b) + 0.2 for b in face_fields(g, rng, zero_neumann=False)]
    umac = face_fields(g, rng)
    un_or, phi_or, st_or = O.mac_project(g, beta, umac, rtol=1e-13)
    ut = [cuda(u) for u in umac]
    mp = MacProjector(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision="fp64"))
    mp.initProjector(beta=[cuda(b) for b in beta])
    mp.setDomainBC(bclo, bchi)
    mp.setUMAC(ut)
    phi = cuda(np.zeros(g.cell_shape))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi, phi_guess=False)
    assert st["status"] == 0
    flux = [cuda(np.full(u.shape, np.nan)) for u in umac]
    mp.getFluxes(flux, phi)
    for d in range(3):
        got = flux[d].cpu().numpy()
        ref = un_or[d] - umac[d]
        scale = max(np.abs(ref).max(), 1e-300)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9 * scale)
        np.testing.assert_allclose(got, ut[d].cpu().numpy() - umac[d], rtol=0, atol=1e-13 * scale)


@pytest.mark.parametrize("case", [CASES[4], ((64, 32, 32), (1.0, 0.5, 0.5), (D, N, P), (N, D, P))],
                         ids=["32-walls", "64x32x32-dirichlet"])
def test_cluster_coarse_cycle_matches_per_level_launches(gpu_lib, case):
    """The small levels of the MAC hierarchy run as one thread-block-cluster launch per V-cycle: one V-cycle
    from the first such level agrees with the per-level launches to FP32 rounding, and the projection
    through it matches the oracle."""
    import ctypes

    from incflo_gb300 import _abi

    n, ext, bclo, bchi = case
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(12)
    beta = [np.abs(b) + 0.2 for b in face_fields(g, rng, zero_neumann=False)]
    umac = face_fields(g, rng)
    un_or, phi_or, st_or = O.mac_project(g, beta, umac, rtol=1e-13)
    mp = MacProjector(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision="mixed"))
    mp.initProjector(beta=[cuda(b) for b in beta])
    mp.setDomainBC(bclo, bchi)
    mp.setUMAC([cuda(u) for u in umac])
    phi = cuda(np.zeros(g.cell_shape))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi, phi_guess=False)
    assert st["status"] == 0 and rel_l2(phi.cpu().numpy(), phi_or) <= 1e-9
    diff = ctypes.c_double()
    _abi.check(_abi.load().gbp_plan_check_coarse_cycle(mp.plan.ptr, ctypes.byref(diff)), "check_coarse_cycle")
    print(f"\n{n}: MAC cluster vs per-level V-cycle {diff.value:.2e}")
    assert diff.value <= 1e-5
