"""The oracle's cell-centred projection pieces on the CPU: MOL face velocities and the full
ApplyCCProjection restatement (divergence-free faces, gp / p_cc bookkeeping)."""
import numpy as np

import oracle as O
from tests.helpers import D, I, N, P


def test_mol_faces_oracle_upwinding():
    """CPU check of the face-velocity restatement: a uniform flow passes through unchanged, a
    divergent pair gives 0, and the upwind side is taken."""
    g = O.Grid((8, 4, 4), bclo=(P, P, P))
    vel = np.zeros((3, 6, 6, 10))
    vel[0] = 0.7
    f = O.mol_extrap_to_faces(g, vel)
    assert np.allclose(f[0], 0.7) and np.allclose(f[1], 0) and np.allclose(f[2], 0)
    vel[0, 1:-1, 1:-1, 1:-1] = np.where(np.arange(8) < 4, -1.0, 1.0)  # diverging at face 4
    f = O.mol_extrap_to_faces(g, vel)
    assert np.allclose(f[0][:, :, 4], 0.0)


def test_cc_projection_oracle_divergence_free_and_consistent():
    g = O.Grid((12, 10, 8), hi=(1.5, 1.25, 1.0), bclo=(I, N, P), bchi=(D, N, P))
    rng = np.random.default_rng(3)
    vel = np.zeros((3, 10, 12, 14))
    vel[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((3,) + g.cell_shape)
    vel[0, 1:-1, 1:-1, 0] = 1.0
    rho = rng.uniform(1.0, 2.0, (10, 12, 14))
    gp0 = np.zeros((3,) + g.cell_shape)
    v, gp, p_cc, um, phi, st = O.cc_projection(g, vel, rho, gp0, np.zeros(g.cell_shape), scaling_factor=0.5)
    assert st["status"] == 0
    assert np.abs(O.mac_rhs(g, *um)).max() < 1e-10
    assert np.array_equal(p_cc, phi)
    # gp = -gphi rho / s and u = u* + gphi  =>  u - u* = -gp s / rho
    du = v[:, 1:-1, 1:-1, 1:-1] - vel[:, 1:-1, 1:-1, 1:-1]
    assert np.allclose(du, -gp * 0.5 / rho[1:-1, 1:-1, 1:-1], atol=1e-12)
