"""Shared helpers of the GPU parity tests: seeded inputs and the oracle's view of the same case."""
import numpy as np
import torch

import oracle as O

P, D, N, I = O.PERIODIC, O.DIRICHLET, O.NEUMANN, O.INFLOW


def nodal_case(n, ext, bclo, bchi, seed=0, sigma_range=(0.3, 2.0)):
    """Random sigma, random velocity with one ghost layer (inflow ghosts hold the inflow value)."""
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(seed)
    sigma = rng.uniform(*sigma_range, g.cell_shape)
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vel[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((3,) + g.cell_shape)
    for d in range(3):
        for side, bc in ((0, bclo[d]), (1, bchi[d])):
            if bc == I:
                sl = [slice(1, -1)] * 3
                sl[2 - d] = 0 if side == 0 else -1
                vel[(d,) + tuple(sl)] = rng.uniform(0.5, 1.5, vel[(d,) + tuple(sl)].shape)
    return g, sigma, vel


def unique_nodes(g, phi_all):
    """GPU nodal arrays hold all nodes 0..n; the oracle keeps the unique ones."""
    nz, ny, nx = g.node_shape
    return phi_all[:nz, :ny, :nx]


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def face_fields(g, rng, zero_neumann=True):
    out = []
    for d in range(3):
        u = rng.standard_normal(g.face_shape(d))
        if g.periodic(d):
            sl_n = [slice(None)] * 3
            sl_0 = [slice(None)] * 3
            sl_n[2 - d] = -1
            sl_0[2 - d] = 0
            u[tuple(sl_n)] = u[tuple(sl_0)]
        elif zero_neumann:
            for side, bc in ((0, g.bclo[d]), (1, g.bchi[d])):
                if bc == N:
                    sl = [slice(None)] * 3
                    sl[2 - d] = 0 if side == 0 else -1
                    u[tuple(sl)] = 0.0
        out.append(u)
    return out
