"""Oracle for the cut-cell (embedded-boundary) nodal projection -- test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import this module.

What it restates: Hydro::NodalProjector with MLNodeLaplacian on an EB geometry, as incflo's
ApplyNodalProjection uses it (src/projection/incflo_apply_nodal_projection.cpp:95-267 with the EB
factory of the level). AMReX is not vendored; the discretisation is the Q1 finite-element one restricted
to the fluid: every cell contributes sigma_c int_{fluid part} grad N_a . grad N_b to the operator and
int_{fluid part} u_c . grad N_a to the right-hand side, with the integrals taken exactly from the cell's
second moments of the fluid region (the EB factory's volume moments, as MLNodeLaplacian builds its
integral arrays from them); the embedded boundary carries no flux (no EB inflow); nodes that touch no
fluid are not unknowns (phi = 0). The velocity correction takes grad phi of the trilinear interpolant
at the fluid centroid of each cell (the cell centre for regular cells, the usual cell-average gradient).

Moments: M[..., p, q, r] = int xi^p eta^q zeta^r dV / V over the fluid part of the cell, in the cell's
normalised coordinates [-1/2, 1/2]^3 (incflo_gb300.eb.cylinder_moments). Arrays: cells (nz, ny, nx),
nodes (nz+1, ny+1, nx+1) on all positions (periodic duplicates filled), velocity (3, nz, ny, nx).
"""
from __future__ import annotations

import itertools

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

PERIODIC, DIRICHLET, NEUMANN = 0, 1, 2


def _sgn(a, d):
    return 1.0 if (a >> d) & 1 else -1.0


def element(M, h):
    """Stiffness K (8 x 8), int grad N (8 x 3) over the fluid part and grad N at the fluid centroid
    (8 x 3) of one cell with moments M (3, 3, 3) and spacing h."""
    V = h[0] * h[1] * h[2]
    K = np.zeros((8, 8))
    G = np.zeros((8, 3))
    for a in range(8):
        for d in range(3):
            e, f = [q for q in range(3) if q != d]
            # int prod_{e != d} (1/2 + s_e xi_e): coefficients (1/2, s) in each of e, f
            acc = 0.0
            for pe, ce in ((0, 0.5), (1, _sgn(a, e))):
                for pf, cf in ((0, 0.5), (1, _sgn(a, f))):
                    idx = [0, 0, 0]
                    idx[e], idx[f] = pe, pf
                    acc += ce * cf * M[idx[0], idx[1], idx[2]]
            G[a, d] = _sgn(a, d) / h[d] * V * acc
        for b in range(8):
            s = 0.0
            for d in range(3):
                e, f = [q for q in range(3) if q != d]
                ce = (0.25, 0.5 * (_sgn(a, e) + _sgn(b, e)), _sgn(a, e) * _sgn(b, e))
                cf = (0.25, 0.5 * (_sgn(a, f) + _sgn(b, f)), _sgn(a, f) * _sgn(b, f))
                acc = 0.0
                for pe in range(3):
                    for pf in range(3):
                        idx = [0, 0, 0]
                        idx[e], idx[f] = pe, pf
                        acc += ce[pe] * cf[pf] * M[idx[0], idx[1], idx[2]]
                s += _sgn(a, d) * _sgn(b, d) / (h[d] * h[d]) * V * acc
            K[a, b] = s
    vol = M[0, 0, 0]
    cen = np.array([M[1, 0, 0], M[0, 1, 0], M[0, 0, 1]]) / vol if vol > 0 else np.zeros(3)
    Gc = np.zeros((8, 3))
    for a in range(8):
        fac = [0.5 + _sgn(a, d) * cen[d] for d in range(3)]
        for d in range(3):
            e, f = [q for q in range(3) if q != d]
            Gc[a, d] = _sgn(a, d) / h[d] * fac[e] * fac[f]
    return K, G, Gc


class EBNodal:
    def __init__(self, n, h, bclo, bchi, moments):
        self.n = [int(v) for v in n]
        self.h = [float(v) for v in h]
        self.bclo, self.bchi = list(bclo), list(bchi)
        self.per = [b == PERIODIC for b in self.bclo]
        self.M = np.asarray(moments, dtype=np.float64)
        self.kap = self.M[..., 0, 0, 0]
        self.nu = [self.n[d] if self.per[d] else self.n[d] + 1 for d in range(3)]
        self.singular = not any((not self.per[d]) and (self.bclo[d] == DIRICHLET or self.bchi[d] == DIRICHLET)
                                for d in range(3))
        self._elements()

    def _node(self, i, j, k):
        v = [i, j, k]
        for d in range(3):
            if self.per[d]:
                v[d] %= self.n[d]
        return v[0] + self.nu[0] * (v[1] + self.nu[1] * v[2])

    def _fixed(self, i, j, k):
        for d, v in enumerate((i, j, k)):
            if self.per[d]:
                continue
            if (v == 0 and self.bclo[d] == DIRICHLET) or (v == self.n[d] and self.bchi[d] == DIRICHLET):
                return True
        return False

    def _elements(self):
        cache = {}
        self.cells = []
        n = self.n
        for k, j, i in itertools.product(range(n[2]), range(n[1]), range(n[0])):
            if self.kap[k, j, i] <= 0.0:
                continue
            key = self.M[k, j, i].tobytes()
            if key not in cache:
                cache[key] = element(self.M[k, j, i], self.h)
            nodes = [self._node(i + (a & 1), j + ((a >> 1) & 1), k + (a >> 2)) for a in range(8)]
            fixed = [self._fixed(i + (a & 1), j + ((a >> 1) & 1), k + (a >> 2)) for a in range(8)]
            self.cells.append(((i, j, k), nodes, fixed, cache[key]))
        N = self.nu[0] * self.nu[1] * self.nu[2]
        self.active = np.zeros(N, bool)
        self.fixed = np.zeros(N, bool)
        for _, nodes, fixed, _ in self.cells:
            for a in range(8):
                self.active[nodes[a]] = True
                self.fixed[nodes[a]] |= fixed[a]

    def assemble(self, sigma, u):
        N = self.nu[0] * self.nu[1] * self.nu[2]
        rows, cols, vals = [], [], []
        b = np.zeros(N)
        for (i, j, k), nodes, fixed, (K, G, _) in self.cells:
            s = sigma[k, j, i]
            for a in range(8):
                b[nodes[a]] += float(G[a] @ u[:, k, j, i])
                for c in range(8):
                    rows.append(nodes[a])
                    cols.append(nodes[c])
                    vals.append(s * K[a, c])
        A = sp.csr_matrix((vals, (rows, cols)), shape=(N, N))
        return A, b

    def project(self, sigma, u):
        """Returns dict(phi (all node positions), u (projected), grad (3, nz, ny, nx), b)."""
        A, b = self.assemble(sigma, u)
        unk = np.nonzero(self.active & ~self.fixed)[0]
        Aa = A[unk][:, unk].tocsc()
        ba = b[unk]
        if self.singular:
            w = np.zeros(len(self.active))
            for (i, j, k), nodes, fixed, _ in self.cells:
                for a in range(8):
                    w[nodes[a]] += self.kap[k, j, i] / 8.0
            wu = w[unk]
            ba = ba - wu * ba.sum() / wu.sum()
            Ab = sp.bmat([[Aa, sp.csc_matrix(wu.reshape(-1, 1))], [sp.csc_matrix(wu.reshape(1, -1)), None]]).tocsc()
            x = spla.spsolve(Ab, np.concatenate([ba, [0.0]]))[:len(unk)]
        else:
            x = spla.spsolve(Aa, ba)
        phi_u = np.zeros(len(self.active))
        phi_u[unk] = x
        n = self.n
        phi = np.zeros((n[2] + 1, n[1] + 1, n[0] + 1))
        for k, j, i in itertools.product(range(n[2] + 1), range(n[1] + 1), range(n[0] + 1)):
            phi[k, j, i] = phi_u[self._node(i, j, k)]
        grad = np.zeros((3, n[2], n[1], n[0]))
        un = np.array(u, dtype=np.float64, copy=True)
        for (i, j, k), nodes, fixed, (_, _, Gc) in self.cells:
            g = Gc.T @ phi_u[nodes]
            grad[:, k, j, i] = g
            un[:, k, j, i] -= sigma[k, j, i] * g
        return {"phi": phi, "u": un, "grad": grad, "b": b, "unknowns": unk}
