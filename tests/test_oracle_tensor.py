"""The tensor-diffusion oracle (oracle/tensor.py) pinned on the CPU: exact ghost extrapolation and zero
div tau for linear fields, the continuous operator on quadratic fields away from the boundary, the
scalar ABecLaplacian oracle in the limit of one component varying across a periodic direction, and
solve / apply consistency."""
import numpy as np

from oracle import abec
from oracle import tensor as T

P, D, N = T.PERIODIC, T.DIRICHLET, T.NEUMANN


def _centres(n, h, ghost=True):
    o = 1 if ghost else 0
    xs = [(np.arange(-o, n[d] + o) + 0.5) * h[d] for d in range(3)]
    Z, Y, X = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    return X, Y, Z


def _set_face_values(vel, n, h, field, bclo, bchi):
    """write the face values of `field` into the ghost cells next to the non-periodic sides"""
    X, Y, Z = _centres(n, h)
    for d in range(3):
        for side in (0, 1):
            bcs = bclo if side == 0 else bchi
            if bcs[0][d] == P:
                continue
            pos = [X.copy(), Y.copy(), Z.copy()]
            pos[d][:] = 0.0 if side == 0 else n[d] * h[d]
            val = field(*pos)
            idx = [slice(None)] * 4
            idx[3 - d] = 0 if side == 0 else n[d] + 1
            vel[tuple(idx)] = val[tuple(idx)]


def test_linear_field_ghosts_exact_and_zero_divtau():
    rng = np.random.default_rng(0)
    n, h = (6, 5, 4), (0.3, 0.25, 0.2)
    bclo = [[D, D, P]] * 3
    bchi = [[D, D, P]] * 3
    Amat = rng.standard_normal((3, 3))
    Amat[:, 2] = 0.0
    b = rng.standard_normal(3)

    def field(x, y, z):
        return np.einsum("cd,d...->c...", Amat, np.array([x, y, z])) + b.reshape((3,) + (1,) * x.ndim)

    X, Y, Z = _centres(n, h)
    full = field(X, Y, Z)
    vel = np.zeros_like(full)
    vel[:, 1:-1, 1:-1, 1:-1] = full[:, 1:-1, 1:-1, 1:-1]
    _set_face_values(vel, n, h, field, bclo, bchi)
    u = T.fill_ghosts(vel, bclo, bchi)
    # every ghost, edges and corners included, is the linear field (z is periodic and the field z-free)
    np.testing.assert_allclose(u, full, rtol=0, atol=1e-13)
    eta = [np.ones((n[2], n[1], n[0] + 1)), np.ones((n[2], n[1] + 1, n[0])), np.ones((n[2] + 1, n[1], n[0]))]
    assert np.abs(T.divtau(u, h, eta)).max() <= 1e-12


def test_quadratic_field_matches_continuous_operator_inside():
    """constant eta: div tau = eta (lap u + (1/3) grad div u), exact for quadratics on cells that read
    no ghost cell"""
    rng = np.random.default_rng(1)
    n, h = (7, 6, 5), (0.2, 0.3, 0.25)
    C = rng.standard_normal((3, 3, 3))  # u_c = sum_{d<=e} C[c,d,e] x_d x_e
    C = 0.5 * (C + C.transpose(0, 2, 1))
    X, Y, Z = _centres(n, h)
    pos = np.array([X, Y, Z])
    full = np.einsum("cde,d...,e...->c...", C, pos, pos)
    eta0 = 0.7
    eta = [eta0 * np.ones((n[2], n[1], n[0] + 1)), eta0 * np.ones((n[2], n[1] + 1, n[0])),
           eta0 * np.ones((n[2] + 1, n[1], n[0]))]
    got = T.divtau(full, h, eta)  # full carries exact values in every ghost
    lap = 2.0 * np.einsum("cdd->c", C)
    graddiv = np.array([2.0 * sum(C[d, d, c] for d in range(3)) for c in range(3)])  # d_c (div u)
    want = eta0 * (lap + graddiv / 3.0)
    inner = got[:, 1:-1, 1:-1, 1:-1]
    np.testing.assert_allclose(inner, np.broadcast_to(want[:, None, None, None], inner.shape), rtol=0, atol=1e-10)


def test_one_component_across_periodic_direction_is_the_scalar_solve():
    """u = (0, 0, w(x, y)) periodic in z: the z component solves the scalar ABecLaplacian with b = eta"""
    rng = np.random.default_rng(2)
    n, h = (6, 5, 4), (0.25, 0.2, 0.3)
    bclo = [[D, N, P]] * 3
    bchi = [[N, D, P]] * 3
    rho = rng.uniform(0.5, 2.0, (n[1], n[0]))
    rho = np.broadcast_to(rho, (n[2], n[1], n[0])).copy()
    eta_cc = np.broadcast_to(rng.uniform(0.5, 1.5, (n[1], n[0])), (n[2], n[1], n[0])).copy()
    eta = abec.eta_to_faces(eta_cc, [False, False, True])
    rhs = np.zeros((3, n[2], n[1], n[0]))
    rhs[2] = np.broadcast_to(rng.standard_normal((n[1], n[0])), (n[2], n[1], n[0]))
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    bx = rng.standard_normal((n[1],))
    vel[2, 1:-1, 1:-1, 0] = bx[None, :]          # x-lo Dirichlet face values of w
    by = rng.standard_normal((n[0],))
    vel[2, 1:-1, -1, 1:-1] = by[None, :]         # y-hi Dirichlet face values of w
    dt = 0.3
    u = T.solve(h, bclo, bchi, 1.0, rho, dt, eta, rhs, vel)
    assert np.abs(u[:2]).max() <= 1e-12
    want = abec.solve(n, h, bclo[2], bchi[2], 1.0, rho, dt, eta, rhs[2], vel[2])
    np.testing.assert_allclose(u[2], want, rtol=0, atol=1e-11)


def test_solve_then_apply_gives_back_the_rhs():
    rng = np.random.default_rng(3)
    n, h = (5, 4, 4), (0.2, 0.25, 0.3)
    bclo = [[D, N, P], [D, D, P], [D, N, P]]  # slip wall on y-lo: normal (v) Dirichlet, others Neumann
    bchi = [[N, D, P], [N, D, P], [N, D, P]]
    rho = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    eta_cc = rng.uniform(0.5, 1.5, (n[2], n[1], n[0]))
    eta = abec.eta_to_faces(eta_cc, [False, False, True])
    rhs = rng.standard_normal((3, n[2], n[1], n[0]))
    vel = rng.standard_normal((3, n[2] + 2, n[1] + 2, n[0] + 2))
    u = T.solve(h, bclo, bchi, 1.0, rho, 0.5, eta, rhs, vel)
    full = vel.copy()
    full[:, 1:-1, 1:-1, 1:-1] = u
    np.testing.assert_allclose(T.apply(full, h, bclo, bchi, 1.0, rho, 0.5, eta), rhs, rtol=0, atol=1e-10)


def test_diffuse_tensor_bc_table():
    """incflo::get_diffuse_tensor_bc: walls and mass inflow Dirichlet, pressure sides Neumann, a slip
    wall Dirichlet for the normal component only, periodic kept; [component][direction] per side."""
    from incflo_gb300.diffusion import diffuse_tensor_bc

    lo, hi = diffuse_tensor_bc(("mass_inflow", "slip_wall", "periodic"), ("pressure_outflow", "no_slip_wall", "periodic"))
    for c in range(3):
        assert lo[c][0] == T.DIRICHLET and hi[c][0] == T.NEUMANN
        assert lo[c][1] == (T.DIRICHLET if c == 1 else T.NEUMANN) and hi[c][1] == T.DIRICHLET
        assert lo[c][2] == T.PERIODIC and hi[c][2] == T.PERIODIC
    import pytest

    with pytest.raises(ValueError):
        diffuse_tensor_bc(("mixed", "periodic", "periodic"), ("periodic", "periodic", "periodic"))
