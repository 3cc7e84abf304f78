"""Cut-cell (embedded-boundary) MAC projection on the GPU against the cut-cell oracle
(oracle/eb_mac.py, a direct sparse solve): flow past a cylinder in a channel (inflow, outflow,
walls, periodic span) and a singular periodic case; phi relative L2 <= 1e-9 and face velocities
within 1e-9 of their scale, FP64 and FP32-in-FP64 forms."""
import numpy as np
import pytest

import oracle as O
from incflo_gb300 import Geometry, MacProjector, eb, make_options
from oracle.eb_mac import EBMac
from tests.helpers import D, I, N, P, cuda, face_fields, rel_l2

pytestmark = pytest.mark.gpu

CASES = {
    "channel": ((64, 16, 8), (4.0, 1.0, 0.5), (I, N, P), (D, N, P), (1.0, 0.5), 0.125),
    "singular": ((48, 24, 8), (2.0, 1.0, 1.0 / 3.0), (P, N, P), (P, N, P), (0.9, 0.45), 0.2),
}


def _case(name, seed=4, variable_beta=True):
    n, ext, bclo, bchi, c, r = CASES[name]
    geo = eb.cylinder(n, (0, 0, 0), ext, (c[0], c[1], 0.0), r)
    ap = [geo["apx"], geo["apy"], geo["apz"]]
    fc = [geo["fcx"], geo["fcy"], geo["fcz"]]
    rng = np.random.default_rng(seed)
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    umac = face_fields(g, rng)
    umac[0] += 1.0  # a mean stream along x plus noise
    if bclo[0] == I:
        umac[0][:, :, 0] = 1.0
    beta = [rng.uniform(0.5, 1.5, a.shape) if variable_beta else np.ones(a.shape) for a in ap]
    for d in range(3):
        if g.periodic(d):
            sl_n = [slice(None)] * 3
            sl_0 = [slice(None)] * 3
            sl_n[2 - d] = -1
            sl_0[2 - d] = 0
            beta[d][tuple(sl_n)] = beta[d][tuple(sl_0)]
    h = [ext[d] / n[d] for d in range(3)]
    m = EBMac(n, h, bclo, bchi, geo["vfrac"], ap, fc, beta)
    return n, ext, bclo, bchi, geo, beta, umac, m


def _gpu_projector(n, ext, bclo, bchi, geo, beta, precision):
    mp = MacProjector(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision=precision))
    mp.initProjector(beta=[cuda(b) for b in beta])
    mp.setDomainBC(bclo, bchi)
    mp.setEB(cuda(geo["vfrac"]), [cuda(geo[k]) for k in ("apx", "apy", "apz")],
             [cuda(np.moveaxis(geo[k], -1, 0)) for k in ("fcx", "fcy", "fcz")])
    return mp


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(CASES))
def test_eb_mac_project_matches_oracle(gpu_lib, name, precision):
    n, ext, bclo, bchi, geo, beta, umac, m = _case(name)
    un_or, phi_or, _ = m.project(umac)
    mp = _gpu_projector(n, ext, bclo, bchi, geo, beta, precision)
    ut = [cuda(u) for u in umac]
    mp.setUMAC(ut)
    phi = cuda(np.zeros((n[2], n[1], n[0])))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi, phi_guess=False)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    assert rel_l2(phi.cpu().numpy(), phi_or) <= 1e-9
    assert m.divergence([u.cpu().numpy() for u in ut]) <= 1e-9 * m.divergence(umac)
    for d in range(3):
        ref = un_or[d]
        got = ut[d].cpu().numpy()
        open_ = m.ap[d] > 0
        np.testing.assert_allclose(got[open_], ref[open_], rtol=0, atol=1e-9 * np.abs(ref).max())
    # V-cycle count stays near the regular-geometry count: the cut-face terms are in the smoother
    assert st["vcycles"] <= 40


def test_eb_removed_restores_regular_projection(gpu_lib):
    """setEB(None) after a cut-cell solve gives the plain MAC projection again."""
    n, ext, bclo, bchi, geo, beta, umac, m = _case("channel")
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    un_or, phi_or, st_or = O.mac_project(g, beta, umac, rtol=1e-13)
    mp = _gpu_projector(n, ext, bclo, bchi, geo, beta, "fp64")
    mp.setUMAC([cuda(u) for u in umac])
    mp.project(rtol=1e-12, atol=0.0)
    mp.setEB(None, None, None)
    ut = [cuda(u) for u in umac]
    mp.setUMAC(ut)
    phi = cuda(np.zeros((n[2], n[1], n[0])))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi, phi_guess=False)
    assert st["status"] == 0
    assert rel_l2(phi.cpu().numpy(), phi_or) <= 1e-9


def test_eb_rejects_inconsistent_geometry(gpu_lib):
    n, ext, bclo, bchi, geo, beta, umac, m = _case("channel")
    bad = dict(geo)
    v = geo["vfrac"].copy()
    j, i = np.argwhere(geo["apx"][0] == 1.0)[0]
    v[:, j, min(i, n[0] - 1)] = 0.0  # a covered cell behind an open face
    bad["vfrac"] = v
    with pytest.raises(Exception):
        _gpu_projector(n, ext, bclo, bchi, bad, beta, "fp64")._ensure()


def test_eb_get_fluxes_are_the_projection_correction(gpu_lib):
    """getFluxes with cut cells (Location::FaceCentroid): the correction the cut-cell projection applied."""
    n, ext, bclo, bchi, geo, beta, umac, m = _case("channel")
    mp = _gpu_projector(n, ext, bclo, bchi, geo, beta, "fp64")
    ut = [cuda(u) for u in umac]
    mp.setUMAC(ut)
    phi = cuda(np.zeros((n[2], n[1], n[0])))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi, phi_guess=False)
    assert st["status"] == 0
    flux = [cuda(np.zeros(u.shape)) for u in umac]
    mp.getFluxes(flux, phi)
    for d in range(3):
        corr = ut[d].cpu().numpy() - umac[d]
        np.testing.assert_allclose(flux[d].cpu().numpy(), corr, rtol=0, atol=1e-13 * max(np.abs(corr).max(), 1e-300))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_eb_inflow_velocity_matches_oracle(gpu_lib, precision):
    """MacProjector::setEBInflowVelocity: the cylinder of the channel blows into the fluid at unit speed
    (incflo's eb_flow.vel_mag); phi and the projected face velocities match the cut-cell oracle with the
    boundary flux in its divergence; removing the inflow gives the plain cut-cell projection again."""
    n, ext, bclo, bchi, geo, beta, umac, m = _case("channel")
    c, r = CASES["channel"][4], CASES["channel"][5]
    bd = eb.cylinder_boundary(n, (0, 0, 0), ext, (c[0], c[1], 0.0), r)
    ev = eb.eb_inflow_velocity(bd["bnorm"], vel_mag=1.0)
    un_or, phi_or, _ = m.project(umac, eb_vel=ev)
    mp = _gpu_projector(n, ext, bclo, bchi, geo, beta, precision)
    mp.setEBInflowVelocity(0, cuda(ev))
    ut = [cuda(u) for u in umac]
    mp.setUMAC(ut)
    phi = cuda(np.zeros((n[2], n[1], n[0])))
    st = mp.project(rtol=1e-12, atol=0.0, phi=phi, phi_guess=False)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    assert rel_l2(phi.cpu().numpy(), phi_or) <= 1e-9
    assert m.divergence([u.cpu().numpy() for u in ut], eb_vel=ev) <= 1e-9 * m.divergence(umac, eb_vel=ev)
    for d in range(3):
        open_ = m.ap[d] > 0
        np.testing.assert_allclose(ut[d].cpu().numpy()[open_], un_or[d][open_], rtol=0,
                                   atol=1e-9 * np.abs(un_or[d]).max())
    mp.setEBInflowVelocity(0, None)
    mp.setUMAC([cuda(u) for u in umac])
    phi2 = cuda(np.zeros((n[2], n[1], n[0])))
    assert mp.project(rtol=1e-12, atol=0.0, phi=phi2, phi_guess=False)["status"] == 0
    assert rel_l2(phi2.cpu().numpy(), m.project(umac)[1]) <= 1e-9
