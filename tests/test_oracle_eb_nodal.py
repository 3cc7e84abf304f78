"""The cut-cell nodal oracle (oracle/eb_nodal.py) and the moments of the cut-cell generator pinned on the
CPU: a full cell's moments give the standard Q1 element, the projection reduces to the single-level
oracle on a regular geometry, cut-cell element matrices are symmetric positive semi-definite with the
constants as null space, and the generator's moments match the volume fractions and centroids."""
import numpy as np

import oracle as O
from incflo_gb300 import eb
from oracle.eb_nodal import EBNodal, element
from tests.helpers import D, N, P, rel_l2, unique_nodes


def _full_moments():
    M = np.zeros((3, 3, 3))
    one = [1.0, 0.0, 1.0 / 12.0]
    for p in range(3):
        for q in range(3):
            for r in range(3):
                M[p, q, r] = one[p] * one[q] * one[r]
    return M


def test_full_cell_is_standard_element():
    h = (0.1, 0.2, 0.3)
    K, G, Gc = element(_full_moments(), h)
    assert np.abs(K - K.T).max() <= 1e-15 and np.abs(K.sum(axis=1)).max() <= 1e-14
    for a in range(8):
        for d in range(3):
            s = 1.0 if (a >> d) & 1 else -1.0
            e, f = [q for q in range(3) if q != d]
            assert abs(G[a, d] - s * h[e] * h[f] / 4) <= 1e-16
            assert abs(Gc[a, d] - s / (4 * h[d])) <= 1e-14
    # diagonal entry of the trilinear stiffness of a cube of side 1: 1/3
    K1, _, _ = element(_full_moments(), (1.0, 1.0, 1.0))
    assert abs(K1[0, 0] - 1.0 / 3.0) <= 1e-15


def test_regular_geometry_matches_single_level_oracle():
    n, ext, bclo, bchi = (8, 6, 4), (1.0, 0.75, 0.5), (P, N, D), (P, N, N)
    h = [ext[d] / n[d] for d in range(3)]
    rng = np.random.default_rng(0)
    sig = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    u = rng.standard_normal((3, n[2], n[1], n[0]))
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    vg = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vg[:, 1:-1, 1:-1, 1:-1] = u
    vn, phi, _, _ = O.nodal_project(g, sig, vg, rtol=1e-14)
    M = np.broadcast_to(_full_moments(), (n[2], n[1], n[0], 3, 3, 3))
    r = EBNodal(n, h, bclo, bchi, M).project(sig, u)
    assert rel_l2(unique_nodes(g, r["phi"]), phi) <= 1e-11
    np.testing.assert_allclose(r["u"], vn[:, 1:-1, 1:-1, 1:-1], rtol=0, atol=1e-11)


def test_cut_cells_psd_with_constant_null_space():
    n, ext = (16, 8, 2), (2.0, 1.0, 0.25)
    M = eb.cylinder_moments(n, (0, 0, 0), ext, (0.7, 0.5, 0.0), 0.2)
    geo = eb.cylinder(n, (0, 0, 0), ext, (0.7, 0.5, 0.0), 0.2)
    np.testing.assert_allclose(M[..., 0, 0, 0], geo["vfrac"], rtol=0, atol=1e-13)
    h = [ext[d] / n[d] for d in range(3)]
    cut = np.argwhere((M[..., 0, 0, 0] > 0) & (M[..., 0, 0, 0] < 1))
    assert len(cut) > 0
    for k, j, i in cut:
        K, G, _ = element(M[k, j, i], h)
        w = np.linalg.eigvalsh(K)
        assert w.min() >= -1e-14 * w.max()
        assert np.abs(K @ np.ones(8)).max() <= 1e-13 * np.abs(K).max()
        assert np.abs(G.sum(axis=0)).max() <= 1e-15  # int grad (sum N) = 0
    # the centroid offsets agree with the generator's (2-D) centroids through the prism
    k, j, i = cut[0]
    cx = M[k, j, i, 1, 0, 0] / M[k, j, i, 0, 0, 0]
    cz = M[k, j, i, 0, 0, 1] / M[k, j, i, 0, 0, 0]
    assert abs(cz) <= 1e-15
    assert abs(cx - geo["fcz"][k, j, i, 0]) <= 1e-9


def test_small_cell_removal_consistent_and_conditions_the_system():
    """eb2.small_volfrac: cells below the threshold become covered in both generators (their faces
    closed), and the singular periodic system loses its near-null sliver modes."""
    n, ext, c, r = (32, 16, 4), (2.0, 1.0, 0.25), (0.9, 0.45, 0.0), 0.23
    h = [ext[d] / n[d] for d in range(3)]
    raw = eb.cylinder_moments(n, (0, 0, 0), ext, c, r)
    M = eb.cylinder_moments(n, (0, 0, 0), ext, c, r, small_volfrac=1e-4)
    geo = eb.cylinder(n, (0, 0, 0), ext, c, r, small_volfrac=1e-4)
    k0 = raw[..., 0, 0, 0]
    small = (k0 > 0) & (k0 < 1e-4)
    assert small.any()
    np.testing.assert_allclose(M[..., 0, 0, 0], geo["vfrac"], rtol=0, atol=1e-13)
    assert (M[small] == 0).all() and (M[~small] == raw[~small]).all()
    k, j, i = np.argwhere(small)[0]
    assert geo["apx"][k, j, i] == 0 and geo["apx"][k, j, i + 1] == 0
    assert geo["apy"][k, j, i] == 0 and geo["apy"][k, j + 1, i] == 0
    P, N = 0, 2
    sig = np.ones((n[2], n[1], n[0]))
    conds = []
    for mom in (raw, M):
        o = EBNodal(n, h, (P, N, P), (P, N, P), mom)
        A, _ = o.assemble(sig, np.zeros((3, n[2], n[1], n[0])))
        ui = np.nonzero(o.active & ~o.fixed)[0]
        w = np.linalg.eigvalsh(A[ui][:, ui].toarray())
        conds.append(w[-1] / w[1])
    assert conds[0] > 1e8 and conds[1] < 1e6


def test_inflow_sides_match_single_level_oracle():
    """Inflow sides (ghost-cell normal velocity on the face) on a regular geometry reduce to the
    single-level oracle's inflow term, on both the low and the high side."""
    I = O.INFLOW
    n, ext, bclo, bchi = (8, 6, 4), (1.0, 0.75, 0.5), (I, N, P), (D, I, P)
    h = [ext[d] / n[d] for d in range(3)]
    rng = np.random.default_rng(1)
    sig = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    vg = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vg[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((3, n[2], n[1], n[0]))
    vg[0, 1:-1, 1:-1, 0] = rng.uniform(0.5, 1.5, (n[2], n[1]))   # x-low inflow ghosts
    vg[1, 1:-1, -1, 1:-1] = rng.uniform(-1.5, -0.5, (n[2], n[0]))  # y-high inflow ghosts
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    vn, phi, _, _ = O.nodal_project(g, sig, vg, rtol=1e-14)
    M = np.broadcast_to(_full_moments(), (n[2], n[1], n[0], 3, 3, 3))
    o = EBNodal(n, h, bclo, bchi, M)
    u = np.ascontiguousarray(vg[:, 1:-1, 1:-1, 1:-1])
    unk = o.active & ~o.fixed  # the C oracle writes 0 on Dirichlet nodes, which are not unknowns
    np.testing.assert_allclose(o.rhs(u, vg)[unk], O.nodal_rhs(g, vg).reshape(-1)[unk], rtol=0, atol=1e-14)
    r = o.project(sig, u, vg)
    assert rel_l2(unique_nodes(g, r["phi"]), phi) <= 1e-11
    np.testing.assert_allclose(r["u"], vn[:, 1:-1, 1:-1, 1:-1], rtol=0, atol=1e-11)


def test_residual_norm_checks_a_solution():
    """residual_norm (the full-size check of a GPU solution) is at round-off for the oracle's own
    solution of a cut-cell channel with inflow and large for a perturbed one."""
    I = O.INFLOW
    n, ext = (32, 8, 4), (4.0, 1.0, 0.5)
    h = [ext[d] / n[d] for d in range(3)]
    M = eb.cylinder_moments(n, (0, 0, 0), ext, (1.0, 0.5, 0.0), 0.125, small_volfrac=1e-4)
    rng = np.random.default_rng(2)
    sig = np.ones((n[2], n[1], n[0]))
    vg = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vg[:, 1:-1, 1:-1, 1:-1] = 1e-3 * rng.uniform(-1, 1, (3, n[2], n[1], n[0]))
    vg[0] += 1.0
    o = EBNodal(n, h, (I, N, P), (D, N, P), M)
    u = np.ascontiguousarray(vg[:, 1:-1, 1:-1, 1:-1])
    r = o.project(sig, u, vg)
    assert o.residual_norm(sig, u, r["phi"], vg) <= 1e-11
    bad = r["phi"] * (1 + 1e-6)
    assert o.residual_norm(sig, u, bad, vg) >= 1e-8


def test_eb_inflow_term_distributes_the_boundary_flux():
    """The EB inflow term of the right-hand side: per cut cell the boundary's outflow F_c spread over the
    eight corners by the trilinear weights at the boundary centroid (they sum to one), so the term adds
    -sum F_c over all nodes; it is linear in the boundary velocity and absent at zero velocity; the
    boundary centroids lie on the circle."""
    n, ext, c, r = (32, 16, 4), (2.0, 1.0, 0.25), (0.7, 0.5), 0.2
    h = [ext[d] / n[d] for d in range(3)]
    M = eb.cylinder_moments(n, (0, 0, 0), ext, (c[0], c[1], 0.0), r, small_volfrac=1e-4)
    bd = eb.cylinder_boundary(n, (0, 0, 0), ext, (c[0], c[1], 0.0), r, small_volfrac=1e-4)
    o = EBNodal(n, h, (N, N, P), (D, N, P), M)
    rng = np.random.default_rng(3)
    u = rng.standard_normal((3, n[2], n[1], n[0]))
    ev = eb.eb_inflow_velocity(bd["bnorm"], vel_mag=1.5)
    b0 = o.rhs(u)
    b1 = o.rhs(u, eb_inflow=(ev, bd["dap"], bd["bcent"]))
    b2 = o.rhs(u, eb_inflow=(2.0 * ev, bd["dap"], bd["bcent"]))
    V = h[0] * h[1] * h[2]
    F = sum(ev[d] * bd["dap"][d] * V / h[d] for d in range(3))
    F[M[..., 0, 0, 0] <= 0] = 0.0
    assert abs((b1 - b0).sum() + F.sum()) <= 1e-12 * np.abs(F).sum()
    np.testing.assert_allclose(b2 - b0, 2.0 * (b1 - b0), rtol=0, atol=1e-13 * np.abs(b1 - b0).max())
    assert np.array_equal(o.rhs(u, eb_inflow=(0.0 * ev, bd["dap"], bd["bcent"])), b0)
    # blowing out of the whole surface at speed 1.5: total source = 1.5 x the boundary area
    area = sum((bd["dap"][d] * V / h[d]) ** 2 for d in range(3)) ** 0.5
    assert abs(-F.sum() - 1.5 * area.sum()) <= 1e-12 * area.sum()
    kk, jj, ii = np.nonzero(area > 0)
    xb = (ii + 0.5 + bd["bcent"][0][kk, jj, ii]) * h[0]
    yb = (jj + 0.5 + bd["bcent"][1][kk, jj, ii]) * h[1]
    rad = np.hypot(xb - c[0], yb - c[1])
    own = rad < r * 1.2  # cells whose face was closed by small-cell removal have no arc of their own
    assert np.abs(rad[own] - r).max() <= 0.02 * r
