"""The cut-cell MAC oracle (oracle/eb_mac.py) pinned on the CPU: it reduces to the plain MAC oracle on a
regular geometry, its face-centroid normal derivative is exact for bilinear potentials, its operator is
conservative with constants in its null space, and its projection removes the discrete EB divergence."""
import numpy as np
import pytest

import oracle as O
from incflo_gb300 import eb
from oracle.eb_mac import EBMac
from tests.helpers import D, I, N, P, face_fields, rel_l2


def cylinder_case(n=(32, 8, 4), hi=(2.0, 1.0, 0.5), bclo=(I, N, P), bchi=(D, N, P), radius=0.25, seed=4):
    geo = eb.cylinder(n, (0, 0, 0), hi, (0.7, 0.5, 0.0), radius)
    h = [hi[d] / n[d] for d in range(3)]
    ap = [geo["apx"], geo["apy"], geo["apz"]]
    fc = [geo["fcx"], geo["fcy"], geo["fcz"]]
    rng = np.random.default_rng(seed)
    beta = [rng.uniform(0.5, 1.5, a.shape) for a in ap]
    m = EBMac(n, h, bclo, bchi, geo["vfrac"], ap, fc, beta)
    return m, geo, rng


def test_regular_geometry_matches_plain_oracle():
    n, ext, bclo, bchi = (12, 8, 6), (1.5, 1.0, 0.75), (I, P, N), (D, P, D)
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(3)
    beta = [np.abs(b) + 0.2 for b in face_fields(g, rng, zero_neumann=False)]
    umac = face_fields(g, rng)
    un_or, phi_or, st = O.mac_project(g, beta, umac, rtol=1e-14)
    assert st["status"] == 0
    ones = [np.ones(g.face_shape(d)) for d in range(3)]
    fc = [np.zeros(g.face_shape(d) + (2,)) for d in range(3)]
    h = [ext[d] / n[d] for d in range(3)]
    m = EBMac(n, h, bclo, bchi, np.ones(g.cell_shape), ones, fc, beta)
    un, phi, _ = m.project(umac)
    assert rel_l2(phi, phi_or) <= 1e-11
    for d in range(3):
        np.testing.assert_allclose(un[d], un_or[d], rtol=0, atol=1e-11 * np.abs(un_or[d]).max())


def test_centroid_derivative_exact_for_bilinear_potential():
    """dphi/dn at a cut face's centroid from the blended face-centre differences equals the exact
    derivative for phi = x y (x faces), x y (y faces) and x y z (z faces): the blend is bilinear."""
    m, geo, _ = cylinder_case(bclo=(P, P, P), bchi=(P, P, P))
    m.beta = [np.ones_like(a) for a in m.ap]
    m._faces()
    n, h = m.n, m.h
    zc, yc, xc = np.meshgrid(*[(np.arange(n[d]) + 0.5) * h[d] for d in (2, 1, 0)], indexing="ij")
    for d, phi in ((0, xc * yc), (1, xc * yc), (2, xc * yc * zc)):
        g = m.grad_face(phi.reshape(-1))[d]
        ap = m.ap[d]
        fc = m.fc[d]
        checked = 0
        for dd, f, kind, terms in m.faces:
            if dd != d or not (0.0 < ap[f[2], f[1], f[0]] < 1.0) or f[d] == 0:
                continue
            # exact derivative at the centroid; skip faces whose blend dropped a closed neighbour
            tang = [t for t in range(3) if t != d]
            if len(terms) != 1 + sum(1 for o in fc[f[2], f[1], f[0]] if abs(o) > 0) + (
                    1 if all(abs(o) > 0 for o in fc[f[2], f[1], f[0]]) else 0):
                continue
            pos = [(f[t] + 0.5) * h[t] for t in range(3)]
            for a, t in enumerate(tang):
                pos[t] += fc[f[2], f[1], f[0], a] * h[t]
            others = [t for t in range(3) if t != d]
            exact = pos[others[0]] if d < 2 else pos[0] * pos[1]
            assert abs(g[f[2], f[1], f[0]] - exact) <= 1e-12
            checked += 1
        assert checked > 0


def test_operator_conservative_with_constant_null_space():
    m, geo, _ = cylinder_case(bclo=(N, N, P), bchi=(N, N, P))
    A = m.matrix()
    act = m.active
    ones = act.astype(np.float64)
    assert np.abs(A @ ones).max() <= 1e-12 * np.abs(A).max()
    assert np.abs(ones @ A).max() <= 1e-12 * np.abs(A).max()
    # zero centroid offsets: the aperture-weighted 7-point operator, symmetric
    m0 = EBMac(m.n, m.h, m.bclo, m.bchi, m.kap, m.ap, [0 * f for f in m.fc], m.beta)
    A0 = m0.matrix()
    assert abs(A0 - A0.T).max() <= 1e-14 * abs(A0).max()
    assert abs(A - A.T).max() > 1e-6 * abs(A).max()  # the centroid blend is not symmetric


@pytest.mark.parametrize("bcs", [((I, N, P), (D, N, P)), ((P, N, P), (P, N, P))], ids=["channel", "singular"])
def test_projection_removes_eb_divergence(bcs):
    m, geo, rng = cylinder_case(bclo=bcs[0], bchi=bcs[1])
    g = O.Grid(m.n, hi=[m.h[d] * m.n[d] for d in range(3)], bclo=bcs[0], bchi=bcs[1])
    umac = face_fields(g, rng)
    d0 = m.divergence(umac)
    un, phi, b = m.project(umac)
    assert m.divergence(un) <= 1e-11 * d0 or (m.singular and m.divergence(un) <= 1e-10 * d0)
    assert np.all(phi.reshape(-1)[~m.active] == 0.0)
    if m.singular:
        assert abs((m.kap * phi).sum()) <= 1e-12 * np.abs(phi).sum()
        assert abs(b.sum()) <= 1e-12 * np.abs(b).sum()


def test_cut_cell_generator_fractions():
    """vfrac of the cylinder generator integrates to the exact fluid volume; face centroids lie in
    [-0.5, 0.5]; apertures of faces on the axis equal the cell fractions (a prism)."""
    n, hi, r = (64, 32, 2), (2.0, 1.0, 0.25), 0.25
    g = eb.cylinder(n, (0, 0, 0), hi, (0.7, 0.5, 0.0), r)
    V = np.prod(hi) / np.prod(n)
    fluid = g["vfrac"].sum() * V
    exact = np.prod(hi) - np.pi * r * r * hi[2]
    assert abs(fluid - exact) <= 1e-13 * exact
    for k in ("fcx", "fcy", "fcz"):
        assert np.abs(g[k]).max() <= 0.5
    np.testing.assert_allclose(g["apz"][0], g["vfrac"][0], rtol=0, atol=1e-15)


def test_eb_inflow_projection_conserves_the_boundary_source():
    """A cylinder that blows into a channel at unit speed (setEBInflowVelocity from eb_flow.vel_mag):
    the projected face velocities carry no divergence once the boundary's flux is counted, and what
    leaves through the outflow side equals what the boundary puts in (the area vectors of the cut cells,
    from the area fractions, close around the body)."""
    n, ext, c, r = (48, 16, 4), (3.0, 1.0, 0.25), (1.0, 0.5), 0.125
    h = [ext[d] / n[d] for d in range(3)]
    geo = eb.cylinder(n, (0, 0, 0), ext, (c[0], c[1], 0.0), r, small_volfrac=1e-4)
    bd = eb.cylinder_boundary(n, (0, 0, 0), ext, (c[0], c[1], 0.0), r, small_volfrac=1e-4)
    ev = eb.eb_inflow_velocity(bd["bnorm"], vel_mag=1.0)
    ap = [geo["apx"], geo["apy"], geo["apz"]]
    fc = [geo["fcx"], geo["fcy"], geo["fcz"]]
    beta = [np.ones(a.shape) for a in ap]
    m = EBMac(n, h, (N, N, P), (D, N, P), geo["vfrac"], ap, fc, beta)
    umac = [np.zeros(a.shape) for a in ap]
    un, phi, b = m.project(umac, eb_vel=ev)
    assert m.divergence(un, eb_vel=ev) <= 1e-11 * m.divergence(umac, eb_vel=ev)
    source = -m.eb_flux(ev).sum()
    out = (un[0][:, :, -1] * ap[0][:, :, -1]).sum() * h[1] * h[2]
    assert source > 0.9 * 2 * np.pi * r * ext[2]
    assert abs(out - source) <= 1e-10 * source
    # the area vectors close: a uniform velocity through the body carries no net flux
    assert abs(m.eb_flux(np.broadcast_to(np.array([1.0, 0.4, 0.0]).reshape(3, 1, 1, 1), ev.shape)).sum()) <= 1e-13


def test_eb_inflow_velocity_rule():
    """incflo::set_eb_velocity: vel_mag blows along -n; a normal filter keeps only the cells whose
    boundary normal is within the tolerance of -normal; `velocity` is taken as given on cut cells."""
    n, ext = (32, 16, 2), (2.0, 1.0, 0.125)
    bd = eb.cylinder_boundary(n, (0, 0, 0), ext, (1.0, 0.5, 0.0), 0.2)
    cut = (bd["bnorm"] ** 2).sum(axis=0) > 0
    v = eb.eb_inflow_velocity(bd["bnorm"], vel_mag=2.0)
    np.testing.assert_allclose(np.sqrt((v ** 2).sum(axis=0))[cut], 2.0, rtol=1e-12)
    assert np.all(v[:, ~cut] == 0.0)
    # only the cells facing -x (normal out of the fluid along +x, i.e. the body's upstream side); incflo
    # compares n . normal with -1 +- the tolerance in radians (its rule, kept as it is)
    tol = np.radians(30.0)
    vf = eb.eb_inflow_velocity(bd["bnorm"], vel_mag=1.0, normal=(-1.0, 0.0, 0.0), normal_tol_deg=30.0)
    kept = (vf ** 2).sum(axis=0) > 0
    assert kept.any() and np.all(bd["bnorm"][0][kept] >= 1.0 - tol - 1e-6)
    assert np.all(bd["bnorm"][0][cut & ~kept] < 1.0 - tol + 1e-6)
    vc = eb.eb_inflow_velocity(bd["bnorm"], velocity=(0.5, 0.0, -1.0))
    assert np.all(vc[0][cut] == 0.5) and np.all(vc[2][cut] == -1.0) and np.all(vc[:, ~cut] == 0.0)
