"""Oracle for the cell-centred ABecLaplacian solve (scalar diffusion) -- test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import this module.

Restates AMReX's MLABecLaplacian as incflo's DiffusionScalarOp::diffuse_scalar uses it
(src/diffusion/DiffusionScalarOp.cpp:150-327): alpha a phi - beta div(b grad phi) = rhs on cells, the
standard 7-point flux form with face coefficients b, Dirichlet sides with the boundary value on the
face and linear extrapolation through it (maxorder 2: the face flux is b (phi_0 - phi_b) / (h / 2)),
homogeneous Neumann sides, periodic wrap. The face b is either given or the face average of a cell
field eta (the adjacent cell on non-periodic sides, incflo_diffusion.cpp:289-343). Assembled with
scipy.sparse and solved directly.

Arrays: cells (nz, ny, nx); faces x (nz, ny, nx+1), ...; phi with one ghost layer (nz+2, ny+2, nx+2)
whose ghost cells on Dirichlet sides hold the boundary values.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

PERIODIC, DIRICHLET, NEUMANN = 0, 1, 2


def eta_to_faces(eta, per):
    nz, ny, nx = eta.shape
    out = []
    for d in range(3):
        ax = 2 - d
        lo = np.take(eta, [0], axis=ax)
        hi = np.take(eta, [eta.shape[ax] - 1], axis=ax)
        if per[d]:
            ext = np.concatenate([hi, eta, lo], axis=ax)
            f = 0.5 * (np.take(ext, range(0, eta.shape[ax] + 1), axis=ax) + np.take(ext, range(1, eta.shape[ax] + 2), axis=ax))
        else:
            inner = 0.5 * (np.take(eta, range(0, eta.shape[ax] - 1), axis=ax) + np.take(eta, range(1, eta.shape[ax]), axis=ax))
            f = np.concatenate([lo, inner, hi], axis=ax)
        out.append(f)
    return out


def solve(n, h, bclo, bchi, alpha, a, beta, b, rhs, phi_g):
    """Returns phi (nz, ny, nx). a: cells or float; b: [bx, by, bz] faces; phi_g: boundary values in its
    ghost cells (and nothing else used)."""
    n = [int(v) for v in n]
    per = [bclo[d] == PERIODIC for d in range(3)]
    N = n[0] * n[1] * n[2]
    V = h[0] * h[1] * h[2]
    a = np.broadcast_to(np.asarray(a, dtype=np.float64), (n[2], n[1], n[0]))

    def cid(i, j, k):
        return i + n[0] * (j + n[1] * k)

    rows, cols, vals = [], [], []
    g = (V * np.asarray(rhs, dtype=np.float64)).reshape(-1).copy()
    for k in range(n[2]):
        for j in range(n[1]):
            for i in range(n[0]):
                c = cid(i, j, k)
                diag = alpha * a[k, j, i] * V
                idx = [i, j, k]
                for d in range(3):
                    w = V / (h[d] * h[d])
                    for side in (0, 1):
                        f = list(idx)
                        f[d] += side
                        bf = beta * b[d][f[2], f[1], f[0]]
                        nb = list(idx)
                        nb[d] += 1 if side else -1
                        if per[d]:
                            nb[d] %= n[d]
                        elif nb[d] < 0 or nb[d] >= n[d]:
                            bc = bchi[d] if side else bclo[d]
                            if bc == DIRICHLET:
                                gh = [v + 1 for v in idx]
                                gh[d] += 1 if side else -1
                                diag += 2.0 * w * bf
                                g[c] += 2.0 * w * bf * phi_g[gh[2], gh[1], gh[0]]
                            continue
                        diag += w * bf
                        rows.append(c)
                        cols.append(cid(*nb))
                        vals.append(-w * bf)
                rows.append(c)
                cols.append(c)
                vals.append(diag)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(N, N))
    x = spla.spsolve(A.tocsc(), g)
    return x.reshape(n[2], n[1], n[0])
