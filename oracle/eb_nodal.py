"""Oracle for the cut-cell (embedded-boundary) nodal projection -- test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import this module.

What it restates: Hydro::NodalProjector with MLNodeLaplacian on an EB geometry, as incflo's
ApplyNodalProjection uses it (src/projection/incflo_apply_nodal_projection.cpp:95-267 with the EB
factory of the level). AMReX is not vendored; the discretisation is the Q1 finite-element one restricted
to the fluid: every cell contributes sigma_c int_{fluid part} grad N_a . grad N_b to the operator and
int_{fluid part} u_c . grad N_a to the right-hand side, with the integrals taken exactly from the cell's
second moments of the fluid region (the EB factory's volume moments, as MLNodeLaplacian builds its
integral arrays from them); the embedded boundary carries no flux unless an EB inflow velocity is given
(setEBInflowVelocity, src/projection/incflo_apply_nodal_projection.cpp:196-201): then the weak form's
boundary term -int_EB (u_eb . n) N_a dA is added per cut cell as -F_c N_a(x_b), F_c = u_eb . int_EB n dA
the boundary's outflow (area vector from the area fractions, eb.cylinder_boundary's dap) and x_b the
boundary centroid (the EB factory's bcent), the one-point rule on the cell's boundary face; nodes that touch no
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

PERIODIC, DIRICHLET, NEUMANN, INFLOW = 0, 1, 2, 3


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
    """The cut-cell nodal system of one box. Inflow sides (code 3) are natural boundaries like Neumann
    sides; their right-hand-side term comes from the ghost cells of the velocity passed to project()
    (regular ghost cells across the face, normal component only, as the plain oracle's or_nodal_rhs
    takes them)."""

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
        """Unknown index of node (i, j, k) (scalars or integer arrays; periodic positions wrapped)."""
        v = [np.asarray(i), np.asarray(j), np.asarray(k)]
        for d in range(3):
            if self.per[d]:
                v[d] = v[d] % self.n[d]
        return v[0] + self.nu[0] * (v[1] + self.nu[1] * v[2])

    def _fixed(self, i, j, k):
        """Whether node (i, j, k) sits on a Dirichlet side (arrays accepted)."""
        out = np.zeros(np.broadcast(np.asarray(i), np.asarray(j), np.asarray(k)).shape, bool)
        for d, v in enumerate((np.asarray(i), np.asarray(j), np.asarray(k))):
            if self.per[d]:
                continue
            if self.bclo[d] == DIRICHLET:
                out |= v == 0
            if self.bchi[d] == DIRICHLET:
                out |= v == self.n[d]
        return out

    def _elements(self):
        n = self.n
        kk, jj, ii = np.nonzero(self.kap > 0.0)
        self.cell_k, self.cell_j, self.cell_i = kk, jj, ii
        Mc = self.M[kk, jj, ii].reshape(len(kk), 27)
        keys, inv = np.unique(Mc, axis=0, return_inverse=True)
        els = [element(key.reshape(3, 3, 3), self.h) for key in keys]
        self.Ku = np.array([e[0] for e in els]).reshape(-1, 8, 8)
        self.Gu = np.array([e[1] for e in els]).reshape(-1, 8, 3)
        self.Gcu = np.array([e[2] for e in els]).reshape(-1, 8, 3)
        self.inv = np.asarray(inv).reshape(-1)
        a = np.arange(8)
        ci, cj, ck = ii[:, None] + (a & 1), jj[:, None] + ((a >> 1) & 1), kk[:, None] + (a >> 2)
        self.ids = self._node(ci, cj, ck)
        fixed_c = self._fixed(ci, cj, ck)
        N = self.nu[0] * self.nu[1] * self.nu[2]
        self.active = np.zeros(N, bool)
        self.active[self.ids.reshape(-1)] = True
        self.fixed = np.zeros(N, bool)
        self.fixed[self.ids[fixed_c]] = True

    def _inflow_rhs(self, b, u_ghost):
        """Inflow sides: each ghost cell across the face adds its normal velocity times the regular
        element's int dN/dn (+-h_e h_f / 4) to the four face nodes it touches (or_nodal_rhs's term)."""
        n, h = self.n, self.h
        for d in range(3):
            for side, bc in ((0, self.bclo[d]), (1, self.bchi[d])):
                if bc != INFLOW:
                    continue
                e, f = [q for q in range(3) if q != d]  # e < f, so the slice's array axes are (f, e)
                sl = [slice(1, -1)] * 3
                sl[2 - d] = 0 if side == 0 else n[d] + 1
                vals = u_ghost[(d,) + tuple(sl)]
                tf, te = np.meshgrid(np.arange(n[f]), np.arange(n[e]), indexing="ij")
                w = (1.0 if side == 0 else -1.0) * h[e] * h[f] / 4.0
                for de in (0, 1):
                    for df in (0, 1):
                        idx = [None, None, None]
                        idx[d] = np.full(te.shape, 0 if side == 0 else n[d])
                        idx[e] = te + de
                        idx[f] = tf + df
                        node = self._node(idx[0], idx[1], idx[2])
                        np.add.at(b, node.reshape(-1), (w * vals).reshape(-1))

    def _eb_inflow_rhs(self, b, eb_inflow):
        """eb_inflow = (eb_vel, dap, bcent), each (3, nz, ny, nx): b_a -= F_c N_a(x_b) on every fluid
        cell with a boundary face, F_c = sum_d u_d dap_d V / h_d."""
        ev, dap, bc = (np.asarray(a, dtype=np.float64) for a in eb_inflow)
        k, j, i = self.cell_k, self.cell_j, self.cell_i
        V = self.h[0] * self.h[1] * self.h[2]
        F = sum(ev[d][k, j, i] * dap[d][k, j, i] * (V / self.h[d]) for d in range(3))
        N = self.nu[0] * self.nu[1] * self.nu[2]
        a = np.arange(8)
        w = np.ones((len(k), 8))
        for d in range(3):
            s = np.where((a >> d) & 1, 1.0, -1.0)
            w *= 0.5 + s[None, :] * bc[d][k, j, i][:, None]
        b -= np.bincount(self.ids.reshape(-1), weights=(F[:, None] * w).reshape(-1), minlength=N)

    def assemble(self, sigma, u, u_ghost=None, eb_inflow=None):
        """Sparse operator A (all node positions, unknowns and not) and right-hand side b."""
        N = self.nu[0] * self.nu[1] * self.nu[2]
        s = sigma[self.cell_k, self.cell_j, self.cell_i]
        rows = np.repeat(self.ids, 8, axis=1).reshape(-1)
        cols = np.tile(self.ids, (1, 8)).reshape(-1)
        vals = (s[:, None, None] * self.Ku[self.inv]).reshape(-1)
        A = sp.csr_matrix((vals, (rows, cols)), shape=(N, N))
        b = self.rhs(u, u_ghost, eb_inflow)
        return A, b

    def rhs(self, u, u_ghost=None, eb_inflow=None):
        N = self.nu[0] * self.nu[1] * self.nu[2]
        uc = u[:, self.cell_k, self.cell_j, self.cell_i]  # (3, ncell)
        contrib = np.einsum("cad,dc->ca", self.Gu[self.inv], uc)
        b = np.bincount(self.ids.reshape(-1), weights=contrib.reshape(-1), minlength=N)
        if u_ghost is not None:
            self._inflow_rhs(b, u_ghost)
        if eb_inflow is not None:
            self._eb_inflow_rhs(b, eb_inflow)
        return b

    def apply(self, sigma, phi_u, chunk=1 << 17):
        """A phi over all node positions, matrix-free (phi_u indexed like the unknowns)."""
        N = self.nu[0] * self.nu[1] * self.nu[2]
        y = np.zeros(N)
        s = sigma[self.cell_k, self.cell_j, self.cell_i]
        for c0 in range(0, len(s), chunk):
            sl = slice(c0, c0 + chunk)
            ids = self.ids[sl]
            kx = np.einsum("cab,cb->ca", self.Ku[self.inv[sl]], phi_u[ids]) * s[sl, None]
            y += np.bincount(ids.reshape(-1), weights=kx.reshape(-1), minlength=N)
        return y

    def dual_volume(self):
        """Fluid volume of each node's dual cell (kappa V / 8 from every cell around it)."""
        N = self.nu[0] * self.nu[1] * self.nu[2]
        V = self.h[0] * self.h[1] * self.h[2]
        w = self.kap[self.cell_k, self.cell_j, self.cell_i] * V / 8.0
        return np.bincount(self.ids.reshape(-1), weights=np.repeat(w, 8), minlength=N)

    def to_unknowns(self, phi_all):
        """A node array over all positions (nz+1, ny+1, nx+1) as the unknown-indexed vector."""
        n = self.n
        out = np.zeros(self.nu[0] * self.nu[1] * self.nu[2])
        k, j, i = np.meshgrid(np.arange(self.nu[2]), np.arange(self.nu[1]), np.arange(self.nu[0]), indexing="ij")
        out[self._node(i, j, k).reshape(-1)] = phi_all[:self.nu[2], :self.nu[1], :self.nu[0]].reshape(-1)
        del n
        return out

    def residual_norm(self, sigma, u, phi_all, u_ghost=None, eb_inflow=None):
        """max |b - A phi| / (fluid dual volume) over the unknowns, relative to the same norm of b
        (after the consistency shift on singular systems): a check of a solution at any size."""
        b = self.rhs(u, u_ghost, eb_inflow)
        w = self.dual_volume()
        unk = self.active & ~self.fixed
        if self.singular:
            b[unk] -= w[unk] * b[unk].sum() / w[unk].sum()
        r = b - self.apply(sigma, self.to_unknowns(phi_all))
        bn = np.max(np.abs(b[unk]) / w[unk])
        return float(np.max(np.abs(r[unk]) / w[unk]) / bn) if bn > 0 else 0.0

    def project(self, sigma, u, u_ghost=None, eb_inflow=None):
        """Returns dict(phi (all node positions), u (projected), grad (3, nz, ny, nx), b)."""
        A, b = self.assemble(sigma, u, u_ghost, eb_inflow)
        unk = np.nonzero(self.active & ~self.fixed)[0]
        Aa = A[unk][:, unk].tocsc()
        ba = b[unk]
        if self.singular:
            wu = (self.dual_volume() / (self.h[0] * self.h[1] * self.h[2]))[unk]
            ba = ba - wu * ba.sum() / wu.sum()
            Ab = sp.bmat([[Aa, sp.csc_matrix(wu.reshape(-1, 1))], [sp.csc_matrix(wu.reshape(1, -1)), None]]).tocsc()
            x = spla.spsolve(Ab, np.concatenate([ba, [0.0]]))[:len(unk)]
        else:
            x = spla.spsolve(Aa, ba)
        phi_u = np.zeros(len(self.active))
        phi_u[unk] = x
        n = self.n
        k, j, i = np.meshgrid(np.arange(n[2] + 1), np.arange(n[1] + 1), np.arange(n[0] + 1), indexing="ij")
        phi = phi_u[self._node(i, j, k)]
        grad = np.zeros((3, n[2], n[1], n[0]))
        un = np.array(u, dtype=np.float64, copy=True)
        g = np.einsum("cad,ca->dc", self.Gcu[self.inv], phi_u[self.ids])
        s = sigma[self.cell_k, self.cell_j, self.cell_i]
        for d in range(3):
            grad[d, self.cell_k, self.cell_j, self.cell_i] = g[d]
            un[d, self.cell_k, self.cell_j, self.cell_i] -= s * g[d]
        return {"phi": phi, "u": un, "grad": grad, "b": b, "unknowns": unk}
