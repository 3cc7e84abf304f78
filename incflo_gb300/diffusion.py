"""Implicit scalar diffusion on the GPU: the MLABecLaplacian + MLMG solve behind
DiffusionScalarOp::diffuse_scalar (src/diffusion/DiffusionScalarOp.cpp:150-327), through the C ABI
(gbp_abec_*). One single-box level; Dirichlet sides take their values from the ghost cells of phi."""
from __future__ import annotations

import ctypes

import torch

from . import _abi as A
from .projection import Geometry, LinOpBCType, _Plan, _ref, array4


class ABecLaplacian:
    """amrex::MLABecLaplacian (alpha a phi - beta div(b grad phi)) for one level, solved by MLMG's
    replacement: setDomainBC / setScalars / setACoeffs / setBCoeffs / setLevelBC / solve."""

    def __init__(self, geom: Geometry, options: A.Options | None = None, stream=None):
        self.geom = geom
        self.options = options or A.default_options(A.GBP_MAC)
        self.stream = stream
        self.plan = None
        self.alpha, self.beta = 0.0, 1.0
        self.a = 0.0
        self.b = 1.0
        self.eta = None
        self.phi = None
        self.ng_phi = 1
        self.bc_lo = self.bc_hi = None

    def setDomainBC(self, lo, hi):  # noqa: N802
        self.bc_lo = tuple(LinOpBCType.get(v, v) for v in lo)
        self.bc_hi = tuple(LinOpBCType.get(v, v) for v in hi)
        self.plan = None

    def setScalars(self, alpha, beta):  # noqa: N802
        self.alpha, self.beta = float(alpha), float(beta)

    def setACoeffs(self, lev, a):  # noqa: N802
        """a: cell tensor (nz, ny, nx) or a float."""
        if lev != 0:
            raise ValueError("single level only")
        self.a = a

    def setBCoeffs(self, lev, b):  # noqa: N802
        """b: [bx, by, bz] face tensors or a float."""
        if lev != 0:
            raise ValueError("single level only")
        self.b, self.eta = b, None

    def setBCoeffsFromEta(self, lev, eta):  # noqa: N802
        """setBCoeffs(average_scalar_eta_to_faces(eta)): face average of the cell field eta."""
        if lev != 0:
            raise ValueError("single level only")
        self.eta = eta

    def setLevelBC(self, lev, phi, ng=1):  # noqa: N802
        """phi: cell tensor with ng ghost layers; its ghost cells on Dirichlet sides hold the boundary values."""
        if lev != 0:
            raise ValueError("single level only")
        self.phi, self.ng_phi = phi, ng

    def _push(self):
        if self.plan is None:
            if self.bc_lo is None:
                raise RuntimeError("setDomainBC must be called before solve")
            self.plan = _Plan(self.geom, A.GBP_MAC, self.bc_lo, self.bc_hi, self.options, self.stream)
        else:
            self.plan.set_options(self.options)
        L = A.load()
        a_t = self.a if isinstance(self.a, torch.Tensor) else None
        a0 = 0.0 if a_t is not None else float(self.a)
        if self.eta is not None:
            A.check(L.gbp_abec_set_coeffs_eta(self.plan.ptr, self.alpha, _ref(array4(a_t)) if a_t is not None else None,
                                              a0, self.beta, _ref(array4(self.eta))), "gbp_abec_set_coeffs_eta")
        elif isinstance(self.b, (list, tuple)):
            b = [array4(x) for x in self.b]
            A.check(L.gbp_abec_set_coeffs(self.plan.ptr, self.alpha, _ref(array4(a_t)) if a_t is not None else None,
                                          a0, self.beta, _ref(b[0]), _ref(b[1]), _ref(b[2]), 0.0),
                    "gbp_abec_set_coeffs")
        else:
            A.check(L.gbp_abec_set_coeffs(self.plan.ptr, self.alpha, _ref(array4(a_t)) if a_t is not None else None,
                                          a0, self.beta, None, None, None, float(self.b)), "gbp_abec_set_coeffs")

    def solve(self, phi=None, rhs=None, rtol=1e-11, atol=1e-14):
        """MLMG::solve(phi, rhs, rtol, atol): phi (set by setLevelBC if None) is the initial guess and output."""
        if phi is not None:
            self.phi = phi
        self.options.rtol = float(rtol)
        self.options.atol = float(atol)
        self._push()
        st = A.Stats()
        A.check(A.load().gbp_abec_solve(self.plan.ptr, _ref(array4(rhs)), _ref(array4(self.phi, self.ng_phi)),
                                        ctypes.byref(st)), "gbp_abec_solve")
        return st.as_dict()


def diffuse_scalar(geom: Geometry, bc_lo, bc_hi, tracer, density, eta, dt, iconserv, options=None, stream=None):
    """DiffusionScalarOp::diffuse_scalar for one level: for each component c of tracer (ncomp, nz+2,
    ny+2, nx+2 with one ghost layer holding the Dirichlet values), solve
    (a - dt div(eta_c grad)) tracer_c = a tracer_c with a = density if iconserv[c] else 1, b = the face
    average of eta_c (ncomp, nz, ny, nx), in place. Returns the per-component stats."""
    op = ABecLaplacian(geom, options=options, stream=stream)
    op.setDomainBC(bc_lo, bc_hi)
    op.setScalars(1.0, dt)
    out = []
    for c in range(tracer.shape[0]):
        phi = tracer[c]
        interior = phi[1:-1, 1:-1, 1:-1]
        if iconserv[c]:
            op.setACoeffs(0, density)
            rhs = (density * interior).contiguous()
        else:
            op.setACoeffs(0, 1.0)
            rhs = interior.contiguous()
        op.setBCoeffsFromEta(0, eta[c].contiguous())
        op.setLevelBC(0, phi, 1)
        out.append(op.solve(rhs=rhs, rtol=op.options.rtol, atol=op.options.atol))
    return out
