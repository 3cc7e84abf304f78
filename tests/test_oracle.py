"""Pins the CPU oracle (oracle/proj_oracle.c) before anything is compared with it.

incflo ships no golden projection outputs and its MLMG (AMReX / AMReX-Hydro) is not vendored, so
the oracle is pinned by: the analytic Taylor-Green pressure of incflo's probtype 1
(src/derive/incflo_error.cpp:33-34) at second order; an independent element-by-element numpy
assembly (Gauss quadrature) of the same finite-element operator, right-hand side and gradient;
and discrete identities (symmetry, null space, D = -G^T).
"""
import itertools

import numpy as np
import pytest

import oracle as O
from incflo_gb300 import synth

P, D, N, I = O.PERIODIC, O.DIRICHLET, O.NEUMANN, O.INFLOW

GAUSS = np.array([-1.0, 1.0]) / np.sqrt(3.0) * 0.5 + 0.5  # 2-point rule on [0,1]


def _q1(xi, a):
    return xi if a else 1.0 - xi


def _dq1(a):
    return 1.0 if a else -1.0


def element_by_quadrature(h):
    """integral over one brick of grad N_a . grad N_b and of grad N_a, by 2x2x2 Gauss quadrature"""
    K = np.zeros((8, 8))
    Gv = np.zeros((8, 3))
    w = h[0] * h[1] * h[2] / 8.0
    corners = [(a & 1, (a >> 1) & 1, (a >> 2) & 1) for a in range(8)]
    for qx, qy, qz in itertools.product(GAUSS, GAUSS, GAUSS):
        grads = []
        for (ax, ay, az) in corners:
            gx = _dq1(ax) / h[0] * _q1(qy, ay) * _q1(qz, az)
            gy = _q1(qx, ax) * _dq1(ay) / h[1] * _q1(qz, az)
            gz = _q1(qx, ax) * _q1(qy, ay) * _dq1(az) / h[2]
            grads.append(np.array([gx, gy, gz]))
        for a in range(8):
            Gv[a] += w * grads[a]
            for b in range(8):
                K[a, b] += w * grads[a] @ grads[b]
    return K, Gv, corners


def assemble_nodal(g: O.Grid, sigma):
    nnz, nny, nnx = g.node_shape
    nnode = nnx * nny * nnz
    K, Gv, corners = element_by_quadrature(g.h)

    def node(i, j, k):
        idx = [i, j, k]
        for d in range(3):
            if g.periodic(d):
                idx[d] %= g.n[d]
        return idx[0] + nnx * (idx[1] + nny * idx[2])

    M = np.zeros((nnode, nnode))
    for ck, cj, ci in itertools.product(range(g.n[2]), range(g.n[1]), range(g.n[0])):
        ids = [node(ci + a, cj + b, ck + c) for (a, b, c) in corners]
        for p in range(8):
            for q in range(8):
                M[ids[p], ids[q]] += sigma[ck, cj, ci] * K[p, q]
    fixed = np.zeros(nnode, bool)
    for k, j, i in itertools.product(range(nnz), range(nny), range(nnx)):
        for d, v in enumerate((i, j, k)):
            if not g.periodic(d) and ((v == 0 and g.bclo[d] == D) or (v == g.n[d] and g.bchi[d] == D)):
                fixed[i + nnx * (j + nny * k)] = True
    return M, fixed, node, Gv, corners


BC_CASES = [
    ((P, P, P), (P, P, P)),
    ((P, P, N), (P, P, N)),
    ((N, D, P), (I, N, P)),
    ((D, N, N), (D, I, D)),
]


@pytest.mark.parametrize("bclo,bchi", BC_CASES)
@pytest.mark.parametrize("n,ext", [((4, 4, 4), (1.0, 1.0, 1.0)), ((4, 6, 2), (1.0, 0.7, 0.5))])
def test_nodal_operator_matches_quadrature_assembly(bclo, bchi, n, ext):
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(7)
    sigma = rng.uniform(0.3, 2.0, g.cell_shape)
    M, fixed, _, _, _ = assemble_nodal(g, sigma)
    x = rng.standard_normal(g.node_shape)
    x.reshape(-1)[fixed] = 0.0
    ref = M @ x.reshape(-1)
    ref[fixed] = 0.0
    out = O.nodal_apply(g, sigma, x).reshape(-1)
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("bclo,bchi", BC_CASES)
def test_nodal_rhs_and_gradient_match_quadrature(bclo, bchi):
    g = O.Grid((4, 5, 3), hi=(1.0, 1.2, 0.9), bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(11)
    vel = rng.standard_normal((3, g.n[2] + 2, g.n[1] + 2, g.n[0] + 2))
    M, fixed, node, Gv, corners = assemble_nodal(g, np.ones(g.cell_shape))
    nnode = M.shape[0]
    ref = np.zeros(nnode)
    for ck, cj, ci in itertools.product(range(g.n[2]), range(g.n[1]), range(g.n[0])):
        u = vel[:, ck + 1, cj + 1, ci + 1]
        for p, (a, b, c) in enumerate(corners):
            ref[node(ci + a, cj + b, ck + c)] += Gv[p] @ u
    # inflow flux: minus integral over the inflow face of (u_bc . n) N_i
    for d in range(3):
        for side, bc in ((0, g.bclo[d]), (1, g.bchi[d])):
            if bc != I:
                continue
            e1, e2 = [e for e in range(3) if e != d]
            area = g.h[e1] * g.h[e2] / 4.0
            for c1, c2 in itertools.product(range(g.n[e1]), range(g.n[e2])):
                cell = [0, 0, 0]
                cell[d] = -1 if side == 0 else g.n[d]
                cell[e1], cell[e2] = c1, c2
                ubc = vel[d, cell[2] + 1, cell[1] + 1, cell[0] + 1]
                un = -ubc if side == 0 else ubc
                for a1, a2 in itertools.product((0, 1), (0, 1)):
                    nd = [0, 0, 0]
                    nd[d] = 0 if side == 0 else g.n[d]
                    nd[e1], nd[e2] = c1 + a1, c2 + a2
                    ref[node(*nd)] -= un * area
    ref[fixed] = 0.0
    out = O.nodal_rhs(g, vel).reshape(-1)
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-13)
    # gradient = cell average of grad(phi_h)
    phi = rng.standard_normal(g.node_shape)
    grad = O.nodal_gradient(g, phi)
    V = g.h[0] * g.h[1] * g.h[2]
    for ck, cj, ci in itertools.product(range(g.n[2]), range(g.n[1]), range(g.n[0])):
        gr = np.zeros(3)
        for p, (a, b, c) in enumerate(corners):
            gr += Gv[p] * phi.reshape(-1)[node(ci + a, cj + b, ck + c)]
        np.testing.assert_allclose(grad[:, ck, cj, ci], gr / V, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("bclo,bchi", BC_CASES)
def test_nodal_symmetry_nullspace_adjoint(bclo, bchi):
    g = O.Grid((6, 4, 8), bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(3)
    sigma = rng.uniform(0.5, 1.5, g.cell_shape)
    st = O.nodal_stencil(g, sigma)
    x, y = rng.standard_normal((2,) + g.node_shape)
    M, fixed, _, _, _ = assemble_nodal(g, sigma)
    x.reshape(-1)[fixed] = 0
    y.reshape(-1)[fixed] = 0
    ax, ay = O.nodal_apply(g, sigma, x), O.nodal_apply(g, sigma, y)
    assert abs((ax * y).sum() - (x * ay).sum()) <= 1e-12 * np.abs(ax * y).sum()
    if not fixed.any():
        np.testing.assert_allclose(O.nodal_apply(g, sigma, np.ones(g.node_shape)), 0.0, atol=1e-12)
        assert np.abs(st.sum(axis=-1)).max() < 1e-12
    # D = -G^T V: <phi, g(u)> = sum_c V u_c . (G phi)_c when no inflow flux enters
    if I not in bclo + bchi:
        vel = np.zeros((3, g.n[2] + 2, g.n[1] + 2, g.n[0] + 2))
        vel[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((3,) + g.cell_shape)
        gu = O.nodal_rhs(g, vel)
        gp = O.nodal_gradient(g, x)
        V = g.h[0] * g.h[1] * g.h[2]
        lhs = (x * gu).sum()
        rhs = V * (vel[:, 1:-1, 1:-1, 1:-1] * gp).sum()
        assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + 1)


def test_taylor_green_pressure_second_order():
    """incflo probtype 1: projecting u_TG + grad p_exact recovers p_exact (incflo_error.cpp:33-34)."""
    errs = []
    for n in (8, 16, 32):
        g = O.Grid((n, n, n), bclo=(P, P, P))
        h = 1.0 / n
        xc = (np.arange(n) + 0.5) * h
        Z, Y, X = np.meshgrid(xc, xc, xc, indexing="ij")
        tp, fp = 2 * np.pi, 4 * np.pi
        vel = np.zeros((3, n + 2, n + 2, n + 2))
        vel[0, 1:-1, 1:-1, 1:-1] = np.sin(tp * X) * np.cos(tp * Y) * np.cos(tp * Z) - 0.25 * fp * np.sin(fp * X)
        vel[1, 1:-1, 1:-1, 1:-1] = -np.cos(tp * X) * np.sin(tp * Y) * np.cos(tp * Z) - 0.25 * fp * np.sin(fp * Y)
        veln, phi, grad, st = O.nodal_project(g, np.ones(g.cell_shape), vel, rtol=1e-12)
        assert st["status"] == 0 and st["rel_resid"] <= 1e-12
        xn = np.arange(n) * h
        Zn, Yn, Xn = np.meshgrid(xn, xn, xn, indexing="ij")
        p = 0.25 * np.cos(fp * Xn) + 0.25 * np.cos(fp * Yn)
        errs.append(np.abs((phi - phi.mean()) - (p - p.mean())).max())
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert (rates > 1.9).all(), (errs, rates)


def assemble_mac(g: O.Grid, beta):
    n = g.n
    N = n[0] * n[1] * n[2]
    M = np.zeros((N, N))
    V = g.h[0] * g.h[1] * g.h[2]

    def cid(i, j, k):
        return i + n[0] * (j + n[1] * k)

    for k, j, i in itertools.product(range(n[2]), range(n[1]), range(n[0])):
        c = cid(i, j, k)
        for d in range(3):
            w = V / g.h[d] ** 2
            for side in (0, 1):
                f = [i, j, k]
                f[d] += side
                fi = list(f)
                if g.periodic(d):
                    fi[d] %= n[d]
                b = beta[d][fi[2], fi[1], fi[0]]
                nb = [i, j, k]
                nb[d] += 1 if side else -1
                if 0 <= nb[d] < n[d] or g.periodic(d):
                    nb[d] %= n[d]
                    M[c, c] += w * b
                    M[c, cid(*nb)] -= w * b
                else:
                    bc = g.bchi[d] if side else g.bclo[d]
                    if bc == D:
                        M[c, c] += 2 * w * b
    return M


@pytest.mark.parametrize("bclo,bchi", [((P, P, P), (P, P, P)), ((P, N, D), (P, I, N)), ((D, D, N), (N, D, D))])
def test_mac_operator_rhs_correction(bclo, bchi):
    g = O.Grid((4, 6, 4), hi=(1.0, 1.5, 0.8), bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(5)
    beta = [rng.uniform(0.2, 2.0, g.face_shape(d)) for d in range(3)]
    for d in range(3):  # periodic: face n is face 0
        if g.periodic(d):
            sl_n = [slice(None)] * 3
            sl_0 = [slice(None)] * 3
            sl_n[2 - d] = -1
            sl_0[2 - d] = 0
            beta[d][tuple(sl_n)] = beta[d][tuple(sl_0)]
    M = assemble_mac(g, beta)
    x = rng.standard_normal(g.cell_shape)
    np.testing.assert_allclose(O.mac_apply(g, beta, x).reshape(-1), M @ x.reshape(-1), rtol=1e-12, atol=1e-12)
    assert np.abs(M - M.T).max() < 1e-12
    # projection: div(u_new) == 0 to solver tolerance
    umac = [rng.standard_normal(g.face_shape(d)) for d in range(3)]
    for d in range(3):
        if g.periodic(d):
            sl_n = [slice(None)] * 3
            sl_0 = [slice(None)] * 3
            sl_n[2 - d] = -1
            sl_0[2 - d] = 0
            umac[d][tuple(sl_n)] = umac[d][tuple(sl_0)]
        else:  # walls / inflow keep their normal velocity: zero it on Neumann faces for solvability
            for side, bc in ((0, g.bclo[d]), (1, g.bchi[d])):
                if bc == N:
                    sl = [slice(None)] * 3
                    sl[2 - d] = 0 if side == 0 else -1
                    umac[d][tuple(sl)] = 0.0
    un, phi, st = O.mac_project(g, beta, umac, rtol=1e-13)
    rhs0 = O.mac_rhs(g, *umac)
    div_after = O.mac_rhs(g, *un)
    singular = D not in bclo + bchi
    if singular:
        div_after -= div_after.mean()
    assert np.abs(div_after).max() <= 1e-10 * np.abs(rhs0).max()


def test_synthetic_inputs_shapes_and_seeds():
    a = synth.variable_density_rt(16)
    b = synth.variable_density_rt(16)
    np.testing.assert_array_equal(a["rho"], b["rho"])
    np.testing.assert_array_equal(a["vel"], b["vel"])
    assert a["rho"].min() >= 1.0 - 1e-12 and a["rho"].max() <= 3.0 + 1e-12
    assert abs(np.sqrt(np.mean(np.sum(a["vel"] ** 2, axis=0))) - 1.0) < 1e-12
    t = synth.taylor_green_noise(8)
    assert t["vel"].shape == (3, 8, 8, 8)
