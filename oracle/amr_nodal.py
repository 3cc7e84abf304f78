"""Oracle for the two-level (AMR) composite nodal projection -- test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import this module.

What it restates: incflo::ApplyNodalProjection over finest_level = 1
(src/projection/incflo_apply_nodal_projection.cpp:95-267): one Hydro::NodalProjector over both levels
(:187-192), MLNodeLaplacian's composite solve (:215), phi and grad phi per level (:218-219). AMReX is not
vendored; the composite discretisation is the conforming Q1 finite-element one on the composite mesh
(the Almgren-Bell-Szymczak nodal projection with coarse-fine synchronisation):

  * leaf cells: fine cells inside the fine boxes (ratio 2) and coarse cells not covered by them;
    sigma and u per leaf cell;
  * unknowns: coarse nodes not covered by the fine region, fine nodes strictly inside it; a fine node
    on the coarse-fine interface at a coarse node position is that coarse node; the other interface
    nodes hang: their value is the bilinear (linear on edges) interpolation of the coarse nodes of the
    coarse face they lie on;
  * equations: A phi = b with A = P^T (sum over leaf cells of sigma_c K_c) P and b = P^T (sum over leaf
    cells of int u . grad N), P the map from unknowns to leaf-cell corner values (the hanging-node
    constraint); Dirichlet nodes hold 0; periodic directions wrap; singular systems (no Dirichlet side)
    are made consistent and gauged to a volume-weighted mean of zero over the unknowns;
  * outputs: phi on every coarse node (a covered node takes the fine value at its position) and on every
    fine node of the region; a singular system's phi is shifted so that the coarse level's node-volume
    weighted mean is zero; grad phi per level is the cell average of the nodal differences of that
    level's phi (as on one level); u -= sigma grad phi on each level.

Arrays (numpy, C order, last axis x): coarse cells (nz, ny, nx), fine cells (2nz, 2ny, 2nx) over the
whole domain with a boolean fine-cell mask; nodes (nz+1, ny+1, nx+1) / (2nz+1, ...) on all positions
(periodic duplicates filled). Velocities (3, ...) per cell without ghosts; inflow boundaries are not
supported here.
"""
from __future__ import annotations

import itertools

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

PERIODIC, DIRICHLET, NEUMANN = 0, 1, 2


def _element(h):
    """Q1 stiffness (8 x 8) and int grad N (8 x 3) of a box cell; local node a = ax + 2 ay + 4 az."""
    M = [np.array([[2.0, 1.0], [1.0, 2.0]]) * hd / 6.0 for hd in h]
    S = [np.array([[1.0, -1.0], [-1.0, 1.0]]) / hd for hd in h]
    K = (np.kron(M[2], np.kron(M[1], S[0])) + np.kron(M[2], np.kron(S[1], M[0]))
         + np.kron(S[2], np.kron(M[1], M[0])))
    G = np.zeros((8, 3))
    for a in range(8):
        sel = (a & 1, (a >> 1) & 1, (a >> 2) & 1)
        for d in range(3):
            e, f = [q for q in range(3) if q != d]
            G[a, d] = (1.0 if sel[d] else -1.0) * h[e] * h[f] / 4.0
    return K, G


class CompositeNodal:
    def __init__(self, n, h, bclo, bchi, fine_mask):
        """n, h: coarse cells and spacing; fine_mask: bool (2nz, 2ny, 2nx), True on fine leaf cells
        (a union of 2x2x2 blocks, i.e. whole coarse cells)."""
        self.n = [int(v) for v in n]
        self.h = [float(v) for v in h]
        self.hf = [v / 2.0 for v in self.h]
        self.nf = [2 * v for v in self.n]
        self.bclo, self.bchi = list(bclo), list(bchi)
        self.per = [b == PERIODIC for b in self.bclo]
        fm = np.asarray(fine_mask, dtype=bool)
        assert fm.shape == (self.nf[2], self.nf[1], self.nf[0])
        blk = fm.reshape(self.n[2], 2, self.n[1], 2, self.n[0], 2)
        self.covered = blk.all(axis=(1, 3, 5))
        assert np.array_equal(self.covered, blk.any(axis=(1, 3, 5))), "fine cells must fill whole coarse cells"
        self.fmask = fm
        self.singular = not any((not self.per[d]) and (self.bclo[d] == DIRICHLET or self.bchi[d] == DIRICHLET)
                                for d in range(3))
        self._classify()

    # ------------------------------------------------------------------------------ geometry
    def _wrap(self, idx, nn, d):
        if self.per[d]:
            return idx % nn
        return idx

    def _node_cells_in(self, mask, ncell, node):
        """(count of in-domain cells around node, count of those with mask True)."""
        tot = inn = 0
        for dz, dy, dx in itertools.product((-1, 0), repeat=3):
            c = [node[0] + dx, node[1] + dy, node[2] + dz]
            ok = True
            for d in range(3):
                if self.per[d]:
                    c[d] %= ncell[d]
                elif c[d] < 0 or c[d] >= ncell[d]:
                    ok = False
            if not ok:
                continue
            tot += 1
            inn += bool(mask[c[2], c[1], c[0]])
        return tot, inn

    def _dirichlet(self, node, nn):
        for d in range(3):
            if self.per[d]:
                continue
            if (node[d] == 0 and self.bclo[d] == DIRICHLET) or (node[d] == nn[d] and self.bchi[d] == DIRICHLET):
                return True
        return False

    def _classify(self):
        n, nf = self.n, self.nf
        # unique node index ranges (periodic: 0..n-1)
        self.nuc = [n[d] if self.per[d] else n[d] + 1 for d in range(3)]
        self.nuf = [nf[d] if self.per[d] else nf[d] + 1 for d in range(3)]
        self.fclass = {}  # fine node -> 'in', 'al' (aligned interface), 'hg' (hanging)
        for k, j, i in itertools.product(range(self.nuf[2]), range(self.nuf[1]), range(self.nuf[0])):
            tot, inn = self._node_cells_in(self.fmask, nf, (i, j, k))
            if inn == 0:
                continue
            if inn == tot:
                self.fclass[(i, j, k)] = "in"
            elif i % 2 == 0 and j % 2 == 0 and k % 2 == 0:
                self.fclass[(i, j, k)] = "al"
            else:
                self.fclass[(i, j, k)] = "hg"
        self.dof = {}
        cnt = 0
        self.cdof = {}
        for k, j, i in itertools.product(range(self.nuc[2]), range(self.nuc[1]), range(self.nuc[0])):
            if self.fclass.get((2 * i % self.nuf[0] if self.per[0] else 2 * i,
                                2 * j % self.nuf[1] if self.per[1] else 2 * j,
                                2 * k % self.nuf[2] if self.per[2] else 2 * k)) == "in":
                continue  # covered coarse node
            if self._dirichlet((i, j, k), n):
                continue
            self.cdof[(i, j, k)] = cnt
            cnt += 1
        self.fdof = {}
        for m, c in self.fclass.items():
            if c == "in" and not self._dirichlet(m, nf):
                self.fdof[m] = cnt
                cnt += 1
        self.ndof = cnt

    def fine_map(self, m):
        """list of (dof, weight) giving the value at fine node m (unique index)."""
        c = self.fclass.get(m)
        if c == "in":
            return [(self.fdof[m], 1.0)] if m in self.fdof else []
        if c is None:
            raise KeyError(m)
        odd = [d for d in range(3) if m[d] % 2]
        out = []
        for sel in itertools.product(*[(-1, 1) if d in odd else (0,) for d in range(3)]):
            I = tuple(self._wrap((m[d] + sel[d]) // 2, self.nuc[d], d) if self.per[d] else (m[d] + sel[d]) // 2
                      for d in range(3))
            w = 0.5 ** len(odd)
            if I in self.cdof:
                out.append((self.cdof[I], w))
            elif not self._dirichlet(I, self.n):
                raise RuntimeError(f"hanging node {m} interpolates from a non-unknown coarse node {I}")
        return out

    def coarse_map(self, I):
        if I in self.cdof:
            return [(self.cdof[I], 1.0)]
        if self._dirichlet(I, self.n):
            return []
        raise KeyError(I)

    # ------------------------------------------------------------------------------ assembly
    def _cell_nodes(self, c, ncell, nun):
        out = []
        for a in range(8):
            sel = (a & 1, (a >> 1) & 1, (a >> 2) & 1)
            out.append(tuple((c[d] + sel[d]) % nun[d] if self.per[d] else c[d] + sel[d] for d in range(3)))
        return out

    def assemble(self, sig_c, sig_f, u_c=None, u_f=None):
        Kc, Gc = _element(self.h)
        Kf, Gf = _element(self.hf)
        rows, cols, vals = [], [], []
        b = np.zeros(self.ndof)

        def add(maps, K, G, s, u):
            for a in range(8):
                for p, wp in maps[a]:
                    if u is not None:
                        b[p] += wp * float(G[a] @ u)
                    for bb in range(8):
                        for q, wq in maps[bb]:
                            rows.append(p)
                            cols.append(q)
                            vals.append(wp * wq * s * K[a, bb])

        n, nf = self.n, self.nf
        for k, j, i in itertools.product(range(n[2]), range(n[1]), range(n[0])):
            if self.covered[k, j, i]:
                continue
            maps = [self.coarse_map(I) for I in self._cell_nodes((i, j, k), n, self.nuc)]
            add(maps, Kc, Gc, sig_c[k, j, i], None if u_c is None else u_c[:, k, j, i])
        for k, j, i in itertools.product(range(nf[2]), range(nf[1]), range(nf[0])):
            if not self.fmask[k, j, i]:
                continue
            maps = [self.fine_map(m) for m in self._cell_nodes((i, j, k), nf, self.nuf)]
            add(maps, Kf, Gf, sig_f[k, j, i], None if u_f is None else u_f[:, k, j, i])
        A = sp.csr_matrix((vals, (rows, cols)), shape=(self.ndof, self.ndof))
        return A, b

    def volumes(self):
        """volume (dual cell) of every unknown: the leaf-cell volume shared by its corners."""
        vol = np.zeros(self.ndof)
        Vc = np.prod(self.h) / 8.0
        Vf = np.prod(self.hf) / 8.0
        n, nf = self.n, self.nf
        for k, j, i in itertools.product(range(n[2]), range(n[1]), range(n[0])):
            if self.covered[k, j, i]:
                continue
            for I in self._cell_nodes((i, j, k), n, self.nuc):
                for p, w in self.coarse_map(I):
                    vol[p] += w * Vc
        for k, j, i in itertools.product(range(nf[2]), range(nf[1]), range(nf[0])):
            if not self.fmask[k, j, i]:
                continue
            for m in self._cell_nodes((i, j, k), nf, self.nuf):
                for p, w in self.fine_map(m):
                    vol[p] += w * Vf
        return vol

    # ------------------------------------------------------------------------------ solve
    def solve(self, sig_c, sig_f, u_c, u_f):
        A, b = self.assemble(sig_c, sig_f, u_c, u_f)
        if self.singular:
            vol = self.volumes()
            b = b - vol * b.sum() / vol.sum()
            Aa = sp.bmat([[A, sp.csr_matrix(vol.reshape(-1, 1))], [sp.csr_matrix(vol.reshape(1, -1)), None]]).tocsc()
            x = spla.spsolve(Aa, np.concatenate([b, [0.0]]))[:self.ndof]
        else:
            x = spla.spsolve(A.tocsc(), b)
        return x, A, b

    def node_fields(self, x):
        """phi on all coarse nodes (nz+1, ny+1, nx+1) and all fine nodes (2nz+1, ...), NaN outside the
        fine region; periodic duplicates filled."""
        n, nf = self.n, self.nf
        pc = np.zeros((n[2] + 1, n[1] + 1, n[0] + 1))
        pf = np.full((nf[2] + 1, nf[1] + 1, nf[0] + 1), np.nan)

        def val(maps):
            return sum(w * x[p] for p, w in maps)

        for k, j, i in itertools.product(range(n[2] + 1), range(n[1] + 1), range(n[0] + 1)):
            I = tuple(v % self.nuc[d] if self.per[d] else v for d, v in enumerate((i, j, k)))
            if I in self.cdof or self._dirichlet(I, n):
                pc[k, j, i] = val(self.coarse_map(I))
            else:  # covered: the fine value at the same position
                m = tuple((2 * I[d]) % self.nuf[d] if self.per[d] else 2 * I[d] for d in range(3))
                pc[k, j, i] = val(self.fine_map(m))
        for k, j, i in itertools.product(range(nf[2] + 1), range(nf[1] + 1), range(nf[0] + 1)):
            m = tuple(v % self.nuf[d] if self.per[d] else v for d, v in enumerate((i, j, k)))
            if m in self.fclass:
                pf[k, j, i] = val(self.fine_map(m))
        return pc, pf

    @staticmethod
    def gradient(phi, h):
        """cell gradient (3, nz, ny, nx) of a nodal field on all positions."""
        g = np.zeros((3,) + tuple(s - 1 for s in phi.shape))
        p = phi
        g[0] = ((p[:-1, :-1, 1:] - p[:-1, :-1, :-1]) + (p[:-1, 1:, 1:] - p[:-1, 1:, :-1])
                + (p[1:, :-1, 1:] - p[1:, :-1, :-1]) + (p[1:, 1:, 1:] - p[1:, 1:, :-1])) / (4 * h[0])
        g[1] = ((p[:-1, 1:, :-1] - p[:-1, :-1, :-1]) + (p[:-1, 1:, 1:] - p[:-1, :-1, 1:])
                + (p[1:, 1:, :-1] - p[1:, :-1, :-1]) + (p[1:, 1:, 1:] - p[1:, :-1, 1:])) / (4 * h[1])
        g[2] = ((p[1:, :-1, :-1] - p[:-1, :-1, :-1]) + (p[1:, :-1, 1:] - p[:-1, :-1, 1:])
                + (p[1:, 1:, :-1] - p[:-1, 1:, :-1]) + (p[1:, 1:, 1:] - p[:-1, 1:, 1:])) / (4 * h[2])
        return g

    def project(self, sig_c, sig_f, u_c, u_f):
        """Returns dict(phi_c, phi_f, gphi_c, gphi_f, u_c, u_f (projected copies), x, A, b)."""
        x, A, b = self.solve(sig_c, sig_f, u_c, u_f)
        pc, pf = self.node_fields(x)
        if self.singular:
            # gauge: node-volume weighted mean of the coarse level's phi over its unique nodes is zero
            uq = pc[:self.nuc[2], :self.nuc[1], :self.nuc[0]]
            w = np.ones_like(uq)
            for d in range(3):
                if not self.per[d]:
                    sl = [slice(None)] * 3
                    for e in (0, -1):
                        sl[2 - d] = e
                        w[tuple(sl)] *= 0.5
            c = float((w * uq).sum() / w.sum())
            pc = pc - c
            pf = pf - c
        gc = self.gradient(pc, self.h)
        gf = self.gradient(np.nan_to_num(pf), self.hf)
        gf[:, ~self.fmask] = 0.0
        uc = u_c - sig_c[None] * gc
        uf = np.where(self.fmask[None], u_f - sig_f[None] * gf, u_f)
        return dict(phi_c=pc, phi_f=pf, gphi_c=gc, gphi_f=gf, u_c=uc, u_f=uf, x=x, A=A, b=b)
