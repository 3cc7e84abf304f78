"""The ABecLaplacian oracle (oracle/abec.py) pinned on the CPU: a linear potential with Dirichlet values
on the faces is reproduced exactly (the maxorder-2 boundary closure is exact for linear fields), alpha = 0
with zero boundary values matches the MAC oracle's Poisson solve, and the operator is symmetric."""
import numpy as np

import oracle as O
from oracle import abec
from tests.helpers import D, N, P, face_fields, rel_l2


def test_linear_field_exact():
    n, ext = (8, 6, 4), (1.0, 0.75, 0.5)
    h = [ext[d] / n[d] for d in range(3)]
    b = [np.full(s, 1.7) for s in [(4, 6, 9), (4, 7, 8), (5, 6, 8)]]
    phi_g = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2))
    phi_g[:, :, 0] = 0.0  # x = 0 face
    phi_g[:, :, -1] = 2.0 * ext[0]  # x = 1 face
    x = abec.solve(n, h, (D, N, N), (D, N, N), 0.0, 1.0, 1.0, b, np.zeros((n[2], n[1], n[0])), phi_g)
    xc = (np.arange(n[0]) + 0.5) * h[0]
    np.testing.assert_allclose(x, np.broadcast_to(2.0 * xc, x.shape), rtol=0, atol=1e-12)


def test_poisson_matches_mac_oracle():
    n, ext, bclo, bchi = (8, 8, 6), (1.0, 1.0, 0.75), (D, P, N), (N, P, D)
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(3)
    beta = [np.abs(x) + 0.3 for x in face_fields(g, rng, zero_neumann=False)]
    f = rng.standard_normal(g.cell_shape)
    h = [ext[d] / n[d] for d in range(3)]
    V = np.prod(h)
    # MAC oracle: A phi = rhs with A = -V div(beta grad) and its rhs already V-scaled
    phi_or, st = O.mac_solve(g, beta, V * f, rtol=1e-14)
    x = abec.solve(n, h, bclo, bchi, 0.0, 0.0, 1.0, beta, f, np.zeros((n[2] + 2, n[1] + 2, n[0] + 2)))
    assert rel_l2(x, phi_or) <= 1e-11


def test_eta_faces_periodic_and_walls():
    eta = np.arange(2 * 3 * 4, dtype=float).reshape(2, 3, 4)
    fx, fy, fz = abec.eta_to_faces(eta, (True, False, False))
    assert fx.shape == (2, 3, 5) and fy.shape == (2, 4, 4) and fz.shape == (3, 3, 4)
    assert fx[0, 0, 0] == 0.5 * (eta[0, 0, 3] + eta[0, 0, 0]) and fx[0, 0, 4] == fx[0, 0, 0]
    assert fy[0, 0, 1] == eta[0, 0, 1] and fy[0, 3, 1] == eta[0, 2, 1] and fy[0, 1, 1] == 0.5 * (eta[0, 0, 1] + eta[0, 1, 1])
