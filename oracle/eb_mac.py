"""Oracle for the cut-cell (embedded-boundary) MAC projection -- test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import this module.

What it restates: Hydro::MacProjector with AMReX's MLEBABecLap operator, as incflo sets it up for an
EB geometry (src/incflo.cpp:286-292 with MLMG::Location::FaceCentroid for umac and beta,
src/convection/incflo_compute_MAC_projected_velocities.cpp:82-90, 272-299). AMReX is not vendored, so
the discretisation follows the published cut-cell finite-volume method (Johansen & Colella 1998;
Schwartz, Barad, Colella & Ligocki 2015) with the conventions AMReX documents for MLEBABecLap:

  * unknowns at cell centres of cells with volume fraction kappa > 0; covered cells hold phi = 0;
  * the flux through face f is ap_f * area * beta_f * (dphi/dn at the face centroid); the normal
    derivative at the centroid is the bilinear interpolation of the face-centre differences
    (phi_R - phi_L) / h of face f and of its neighbours f1, f2, f12 shifted by one cell towards the
    centroid in the two tangential directions, with weights |fc_t| (the centroid offset in cell
    widths); a neighbour face enters only when it is open (ap > 0), and the corner face f12 only when
    it and both f1 and f2 are open (otherwise the second direction's weight drops to 0);
  * no interpolation on domain-boundary faces; the embedded boundary itself is homogeneous Neumann
    for phi; with an EB inflow velocity (MacProjector::setEBInflowVelocity,
    src/convection/incflo_compute_MAC_projected_velocities.cpp:274-281) its flux out of the fluid,
    u_eb . (int_EB n dA) = sum_d u_eb,d (ap_lo - ap_hi) area_d (the divergence theorem over the cut
    cell's closed surface), is part of the divergence: b_c -= that flux;
  * operator (scaled by kappa V, which is how both sides are stored here):
        (A phi)_c = - sum_d [F_hi - F_lo],     b_c = - sum_d area_d (ap_hi u_hi - ap_lo u_lo)
    and the correction u_f -= beta_f * dphi/dn(centroid) on every open face;
  * the stopping norm is the reference operator's own max norm, |r_c| / (kappa_c V);
  * singular systems (no Dirichlet side): b_c -= kappa_c sum(b) / sum(kappa), phi gauge
    sum(kappa phi) = 0.

The system is assembled with scipy.sparse and solved directly, so the oracle carries no iteration
error. Array conventions as in oracle/__init__.py: cells (nz, ny, nx), x faces (nz, ny, nx+1), ...
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

PERIODIC, DIRICHLET, NEUMANN, INFLOW = 0, 1, 2, 3


class EBMac:
    def __init__(self, n, h, bclo, bchi, vfrac, ap, fc, beta):
        """n, h: (3,) cells and spacing; bclo/bchi: boundary types; vfrac: cells; ap[d], beta[d]:
        face arrays of direction d; fc[d]: (face shape) + (2,) centroid offsets (tangential
        directions in increasing order)."""
        self.n = [int(v) for v in n]
        self.h = [float(v) for v in h]
        self.bclo, self.bchi = list(bclo), list(bchi)
        self.per = [b == PERIODIC for b in self.bclo]
        self.kap = np.asarray(vfrac, dtype=np.float64)
        self.ap = [np.asarray(a, dtype=np.float64) for a in ap]
        self.fc = [np.asarray(f, dtype=np.float64) for f in fc]
        self.beta = [np.asarray(b, dtype=np.float64) for b in beta]
        self.V = self.h[0] * self.h[1] * self.h[2]
        self.area = [self.V / self.h[d] for d in range(3)]
        self.w = [self.V / (self.h[d] * self.h[d]) for d in range(3)]
        self.ncell = self.n[0] * self.n[1] * self.n[2]
        self.active = self.kap.reshape(-1) > 0.0
        self.singular = not any((not self.per[d]) and (self.bclo[d] == DIRICHLET or self.bchi[d] == DIRICHLET)
                                for d in range(3))
        self._faces()

    # ----------------------------------------------------------------------------------- helpers
    def cid(self, i, j, k):
        return i + self.n[0] * (j + self.n[1] * k)

    def _face_terms(self, d, f):
        """Interior face f = (i, j, k) of direction d (f[d] in 1..n-1, or 0..n-1 periodic): list of
        (weight, L cell, R cell, beta) whose weighted sum of beta (phi_R - phi_L) is the flux
        derivative times h_d at the centroid. Boundary faces get the face-centre term only."""
        n, per = self.n, self.per
        i, j, k = f
        a = self.ap[d][k, j, i]

        def cells(g):
            L = list(g)
            L[d] -= 1
            R = list(g)
            if per[d]:
                L[d] %= n[d]
                R[d] %= n[d]
            return L, R

        L, R = cells(f)
        terms = [(1.0, L, R, self.beta[d][k, j, i])]
        if not (0.0 < a < 1.0):
            return terms
        tang = [t for t in range(3) if t != d]
        off = self.fc[d][k, j, i]

        def shifted(g, t, s):
            g = list(g)
            g[t] += s
            if per[t]:
                g[t] %= n[t]
            elif g[t] < 0 or g[t] >= n[t]:
                return None
            return g

        def open_(g):
            return g is not None and self.ap[d][g[2], g[1], g[0]] > 0.0

        s1 = 1 if off[0] >= 0 else -1
        s2 = 1 if off[1] >= 0 else -1
        f1 = shifted(f, tang[0], s1)
        f2 = shifted(f, tang[1], s2)
        w1 = abs(off[0]) if open_(f1) else 0.0
        w2 = abs(off[1]) if open_(f2) else 0.0
        f12 = shifted(f1, tang[1], s2) if f1 is not None else None
        if w1 > 0.0 and w2 > 0.0 and not open_(f12):
            w2 = 0.0
        terms = [((1 - w1) * (1 - w2), L, R, self.beta[d][k, j, i])]
        for wt, g in ((w1 * (1 - w2), f1), ((1 - w1) * w2, f2), (w1 * w2, f12)):
            if wt != 0.0:
                gl, gr = cells(g)
                terms.append((wt, gl, gr, self.beta[d][g[2], g[1], g[0]]))
        return terms

    def _faces(self):
        """Face list: (d, (i,j,k), kind, terms) with kind 0 interior, 1 Dirichlet low, 2 Dirichlet high."""
        self.faces = []
        n = self.n
        for d in range(3):
            fn = list(n)
            fn[d] += 1
            for k in range(fn[2]):
                for j in range(fn[1]):
                    for i in range(fn[0]):
                        f = (i, j, k)
                        a = self.ap[d][k, j, i]
                        if a <= 0.0:
                            continue
                        fi = f[d]
                        if self.per[d]:
                            if fi == n[d]:
                                continue  # the periodic image of face 0
                            self.faces.append((d, f, 0, self._face_terms(d, f)))
                        elif fi == 0 or fi == n[d]:
                            bc = self.bclo[d] if fi == 0 else self.bchi[d]
                            if bc == DIRICHLET:
                                self.faces.append((d, f, 1 if fi == 0 else 2, None))
                        else:
                            self.faces.append((d, f, 0, self._face_terms(d, f)))

    # ---------------------------------------------------------------------------------- assembly
    def matrix(self):
        rows, cols, vals = [], [], []
        n = self.n
        for d, f, kind, terms in self.faces:
            a = self.ap[d][f[2], f[1], f[0]]
            if kind:
                # Dirichlet boundary face: ghost phi = -phi_inside (phi = 0 on the face)
                c = list(f)
                if kind == 2:
                    c[d] -= 1
                ci = self.cid(*c)
                beta = self.beta[d][f[2], f[1], f[0]]
                rows.append(ci)
                cols.append(ci)
                vals.append(2.0 * a * self.w[d] * beta)
                continue
            L = list(f)
            L[d] -= 1
            if self.per[d]:
                L[d] %= n[d]
            cL, cR = self.cid(*L), self.cid(*f)
            # flux F (positive from L to R along +d) = a w sum wt beta (phi_gR - phi_gL)
            for wt, gl, gr, beta in terms:
                c = a * self.w[d] * wt * beta
                il, ir = self.cid(*gl), self.cid(*gr)
                # (A phi)_cR gets -F ... no: (A phi)_c = -(F_hi - F_lo): cell R has this face low (+F),
                # cell L has it high (-F)
                for row, sgn in ((cR, 1.0), (cL, -1.0)):
                    rows += [row, row]
                    cols += [ir, il]
                    vals += [sgn * c, -sgn * c]
        A = sp.csr_matrix((vals, (rows, cols)), shape=(self.ncell, self.ncell))
        return A

    def eb_flux(self, eb_vel):
        """Flux of the EB inflow velocity (3, nz, ny, nx) out of each cell's fluid through its
        embedded boundary: sum_d u_d (ap_d(low) - ap_d(high)) area_d."""
        n = self.n
        f = np.zeros((n[2], n[1], n[0]))
        for d in range(3):
            sl_lo = [slice(None)] * 3
            sl_hi = [slice(None)] * 3
            sl_lo[2 - d] = slice(0, n[d])
            sl_hi[2 - d] = slice(1, n[d] + 1)
            f += np.asarray(eb_vel[d]) * (self.ap[d][tuple(sl_lo)] - self.ap[d][tuple(sl_hi)]) * self.area[d]
        f[self.kap <= 0.0] = 0.0
        return f

    def rhs(self, umac, eb_vel=None):
        """b = -sum_d area (ap_hi u_hi - ap_lo u_lo) on face-centroid velocities, minus the EB inflow
        flux when an EB velocity is given."""
        n = self.n
        b = np.zeros((n[2], n[1], n[0]))
        for d in range(3):
            fl = self.ap[d] * umac[d] * self.area[d]
            sl_lo = [slice(None)] * 3
            sl_hi = [slice(None)] * 3
            sl_lo[2 - d] = slice(0, n[d])
            sl_hi[2 - d] = slice(1, n[d] + 1)
            hi = fl[tuple(sl_hi)].copy()
            if self.per[d]:
                sl0 = [slice(None)] * 3
                sl0[2 - d] = slice(n[d] - 1, n[d])
                src = [slice(None)] * 3
                src[2 - d] = slice(0, 1)
                hi[tuple(sl0)] = fl[tuple(src)]
            b -= hi - fl[tuple(sl_lo)]
        if eb_vel is not None:
            b -= self.eb_flux(eb_vel)
        b = b.reshape(-1)
        b[~self.active] = 0.0
        return b

    def norm(self, r):
        act = self.active
        kv = self.kap.reshape(-1)[act] * self.V
        return float(np.max(np.abs(r[act]) / kv)) if act.any() else 0.0

    def solve(self, b):
        """Direct solve; singular systems are made consistent and gauged as the module says."""
        A = self.matrix()
        act = np.nonzero(self.active)[0]
        kap = self.kap.reshape(-1)
        b = np.array(b, dtype=np.float64)
        if self.singular:
            b[act] -= kap[act] * b[act].sum() / kap[act].sum()
        Aa = A[act][:, act]
        ba = b[act]
        if self.singular:
            m = len(act)
            kv = kap[act]
            Aa = sp.bmat([[Aa, sp.csr_matrix(kv.reshape(-1, 1))], [sp.csr_matrix(kv.reshape(1, -1)), None]]).tocsc()
            ba = np.concatenate([ba, [0.0]])
            x = spla.spsolve(Aa, ba)[:m]
        else:
            x = spla.spsolve(Aa.tocsc(), ba)
        phi = np.zeros(self.ncell)
        phi[act] = x
        return phi, b

    def grad_face(self, phi):
        """beta dphi/dn at the centroid of every open face (0 elsewhere), face arrays per direction."""
        n = self.n
        out = []
        for d in range(3):
            fn = list(n)
            fn[d] += 1
            out.append(np.zeros((fn[2], fn[1], fn[0])))
        for d, f, kind, terms in self.faces:
            if kind:
                c = list(f)
                if kind == 2:
                    c[d] -= 1
                v = phi[self.cid(*c)]
                beta = self.beta[d][f[2], f[1], f[0]]
                g = (0.0 - v) / (0.5 * self.h[d]) if kind == 2 else (v - 0.0) / (0.5 * self.h[d])
                out[d][f[2], f[1], f[0]] = beta * g
                continue
            acc = 0.0
            for wt, gl, gr, beta in terms:
                acc += wt * beta * (phi[self.cid(*gr)] - phi[self.cid(*gl)]) / self.h[d]
            out[d][f[2], f[1], f[0]] = acc
            if self.per[d] and f[d] == 0:
                g = list(f)
                g[d] = n[d]
                out[d][g[2], g[1], g[0]] = acc
        return out

    def project(self, umac, eb_vel=None):
        """Returns (corrected face velocities, phi (nz, ny, nx), rhs after the singular fix)."""
        b = self.rhs(umac, eb_vel)
        phi, b = self.solve(b)
        gf = self.grad_face(phi)
        u = [np.array(x, dtype=np.float64, copy=True) for x in umac]
        for d in range(3):
            u[d] = u[d] - gf[d]
        return u, phi.reshape(self.n[2], self.n[1], self.n[0]), b

    def divergence(self, umac, eb_vel=None):
        """Max over fluid cells of |sum ap u area (+ EB flux)| / (kappa V): the discrete EB divergence."""
        return self.norm(self.rhs(umac, eb_vel))
