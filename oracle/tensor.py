"""Oracle for the tensor (velocity) diffusion solve -- test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import this module.

Restates what incflo's DiffusionTensorOp asks of AMReX's MLTensorOp (AMReX is not vendored here):
diffuse_velocity (src/diffusion/DiffusionTensorOp.cpp:104-213) solves

    alpha a u - beta div tau = rhs,   tau = eta (grad u + grad u^T) - (2/3) eta (div u) I

with alpha = 1, a = rho, beta = dt, rhs = rho u (the shear-viscosity-only form of MLTensorOp:
setShearViscosity, no bulk viscosity), and compute_divtau (:215-317) applies div tau alone
(setScalars(0, -1)). eta is given on faces (incflo's average_velocity_eta_to_faces,
src/diffusion/incflo_diffusion.cpp:262-286: the face average of the cell field with the domain-side
fix-up). Boundary types are per component and side (get_diffuse_tensor_bc, :106-153): periodic,
Dirichlet (no-slip walls and mass inflow: the value on the face, held in the ghost cell next to it) or
Neumann (outflow, and the tangential components at a slip wall).

Discretisation (cell-centred, flux form): on a face normal to d the normal derivative of every component
is the two-cell difference, the tangential derivative along e the average of the centred differences of
the two cells beside the face. Ghost cells: a Dirichlet side holds 2 u_b - u_inner (linear
extrapolation through the face value, the maxorder-2 stencil), a Neumann side u_inner, a periodic side the
wrapped value. Ghosts are filled direction by direction (x, then y over the x ghosts, then z over both);
beside an edge the face values of a Dirichlet side are continued past the edge (wrapped across a
periodic direction, else extrapolated linearly from the last two faces), so edges and corners follow
from the same rule and a linear field is reproduced exactly. The normal flux of component c through a face normal to d:

    c == d:  eta ((4/3) du_d/dx_d - (2/3) sum_{e != d} du_e/dx_e)
    c != d:  eta (du_c/dx_d + du_d/dx_c)

Arrays: cells (nz, ny, nx); faces x (nz, ny, nx + 1), ...; velocity (3, nz + 2, ny + 2, nx + 2) with one
ghost layer. bclo / bchi: [component][direction].
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

PERIODIC, DIRICHLET, NEUMANN = 0, 1, 2


def fill_ghosts(vel, bclo, bchi):
    """vel: (3, nz+2, ny+2, nx+2), interior and the boundary values in the ghost cells next to each
    Dirichlet face. Returns a copy with every ghost cell (edges and corners included) filled by the
    rule in the module docstring."""
    src = np.array(vel, dtype=np.float64)
    u = src.copy()
    n = [u.shape[3] - 2, u.shape[2] - 2, u.shape[1] - 2]
    for d in range(3):
        ax = 2 - d  # axis of direction d in a (z, y, x) component array
        for side in (0, 1):
            g = 0 if side == 0 else n[d] + 1
            inner = 1 if side == 0 else n[d]
            wrap = n[d] if side == 0 else 1
            for c in range(3):
                bc = (bclo if side == 0 else bchi)[c][d]
                U = u[c]
                gv = np.take(U, g, axis=ax)
                if bc == PERIODIC:
                    val = np.take(U, wrap, axis=ax).copy()
                elif bc == NEUMANN:
                    val = np.take(U, inner, axis=ax).copy()
                else:
                    ub = np.take(src[c], g, axis=ax).copy()
                    # beside an edge (a direction filled before this one) the face values continued
                    # past the edge: wrapped across a periodic direction, else linearly extrapolated
                    for e in range(d):
                        ea = (2 - e) - (1 if (2 - e) > ax else 0)
                        lo = [slice(None), slice(None)]
                        hi = [slice(None), slice(None)]
                        lo[ea], hi[ea] = 0, n[e] + 1
                        if bclo[c][e] == PERIODIC:
                            ub[tuple(lo)] = np.take(ub, n[e], axis=ea)
                            ub[tuple(hi)] = np.take(ub, 1, axis=ea)
                        else:
                            ub[tuple(lo)] = 2.0 * np.take(ub, 1, axis=ea) - np.take(ub, 2, axis=ea)
                            ub[tuple(hi)] = 2.0 * np.take(ub, n[e], axis=ea) - np.take(ub, n[e] - 1, axis=ea)
                    val = 2.0 * ub - np.take(U, inner, axis=ax)
                # directions after d are filled later: only their interior is set here
                keep = np.zeros_like(gv, dtype=bool)
                sl = [slice(None), slice(None)]
                for e in range(3):
                    if e == d:
                        continue
                    ea = (2 - e) - (1 if (2 - e) > ax else 0)
                    sl[ea] = slice(0, n[e] + 2) if e < d else slice(1, n[e] + 1)
                keep[tuple(sl)] = True
                gv = np.where(keep, val, gv)
                idx = [slice(None)] * 3
                idx[ax] = g
                U[tuple(idx)] = gv
    return u


def divtau(u, h, eta):
    """div tau per cell (3, nz, ny, nx) of a ghost-filled velocity; eta = [eta_x, eta_y, eta_z] faces."""
    nz, ny, nx = u.shape[1] - 2, u.shape[2] - 2, u.shape[3] - 2
    n = [nx, ny, nz]
    out = np.zeros((3, nz, ny, nx))
    for d in range(3):
        ax = 3 - d
        # L / R cells of the d-faces, interior in the other directions
        def cells(shift_d, e=None, se=0):
            sl = [slice(None), slice(1, nz + 1), slice(1, ny + 1), slice(1, nx + 1)]
            sl[ax] = slice(shift_d, shift_d + n[d] + 1)
            if e is not None:
                a2 = 3 - e
                sl[a2] = slice(1 + se, 1 + se + n[e])
            return u[tuple(sl)]
        UL, UR = cells(0), cells(1)
        N = (UR - UL) / h[d]  # (3, face shape): normal derivative of every component
        T = {}
        for e in range(3):
            if e == d:
                continue
            T[e] = ((cells(0, e, 1) - cells(0, e, -1)) + (cells(1, e, 1) - cells(1, e, -1))) / (4.0 * h[e])
        ef = eta[d]
        for c in range(3):
            if c == d:
                flux = ef * ((4.0 / 3.0) * N[d] - (2.0 / 3.0) * sum(T[e][e] for e in range(3) if e != d))
            else:
                flux = ef * (N[c] + T[c][d])
            sl_hi = [slice(None)] * 3
            sl_lo = [slice(None)] * 3
            sl_hi[2 - d] = slice(1, n[d] + 1)
            sl_lo[2 - d] = slice(0, n[d])
            out[c] += (flux[tuple(sl_hi)] - flux[tuple(sl_lo)]) / h[d]
    return out


def apply(vel, h, bclo, bchi, alpha, a, beta, eta):
    """alpha a u - beta div tau per cell (3, nz, ny, nx); vel with the boundary values in its ghosts."""
    u = fill_ghosts(vel, bclo, bchi)
    inner = u[:, 1:-1, 1:-1, 1:-1]
    return alpha * np.asarray(a) * inner - beta * divtau(u, h, eta)


def solve(h, bclo, bchi, alpha, a, beta, eta, rhs, vel):
    """u (3, nz, ny, nx) with alpha a u - beta div tau = rhs; vel's ghost cells hold the boundary
    values (its interior is not used). Assembled by probing (small grids only)."""
    vel = np.array(vel, dtype=np.float64)
    nz, ny, nx = vel.shape[1] - 2, vel.shape[2] - 2, vel.shape[3] - 2
    N = 3 * nx * ny * nz
    base = vel.copy()
    base[:, 1:-1, 1:-1, 1:-1] = 0.0
    b0 = apply(base, h, bclo, bchi, alpha, a, beta, eta).reshape(-1)
    cols = []
    probe = np.zeros_like(vel)
    for q in range(N):
        probe[:] = 0.0
        c, rem = divmod(q, nx * ny * nz)
        k, rem = divmod(rem, nx * ny)
        j, i = divmod(rem, nx)
        probe[c, k + 1, j + 1, i + 1] = 1.0
        col = apply(probe, h, bclo, bchi, alpha, a, beta, eta).reshape(-1)
        nzr = np.nonzero(col)[0]
        cols.append((nzr, col[nzr]))
    rows = np.concatenate([r for r, _ in cols])
    vals = np.concatenate([v for _, v in cols])
    cidx = np.concatenate([np.full(len(r), q) for q, (r, _) in enumerate(cols)])
    A = sp.csc_matrix((vals, (rows, cidx)), shape=(N, N))
    x = spla.spsolve(A, np.asarray(rhs, dtype=np.float64).reshape(-1) - b0)
    return x.reshape(3, nz, ny, nx)
