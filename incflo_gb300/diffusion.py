"""Implicit scalar diffusion on the GPU: the MLABecLaplacian + MLMG solve behind
DiffusionScalarOp::diffuse_scalar (src/diffusion/DiffusionScalarOp.cpp:150-327), through the C ABI
(gbp_abec_*). One single-box level; Dirichlet sides take their values from the ghost cells of phi."""
from __future__ import annotations

import ctypes

import torch

from . import _abi as A
from .projection import Geometry, LinOpBCType, _Plan, _ref, _stream_ptr, array4


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


def diffuse_tensor_bc(bc_type_lo, bc_type_hi):
    """incflo::get_diffuse_tensor_bc (src/diffusion/incflo_diffusion.cpp:106-153): per direction the
    incflo boundary type of the low and high side ("periodic", "no_slip_wall", "slip_wall",
    "mass_inflow", "direction_dependent", "pressure_inflow", "pressure_outflow") to the solver's
    per-component types, [component][direction] for each side."""
    def side(types):
        out = [[A.BC_PERIODIC] * 3 for _ in range(3)]
        for d, t in enumerate(types):
            for c in range(3):
                if t == "periodic":
                    v = A.BC_PERIODIC
                elif t in ("pressure_inflow", "pressure_outflow"):
                    v = A.BC_NEUMANN
                elif t in ("mass_inflow", "direction_dependent", "no_slip_wall"):
                    v = A.BC_DIRICHLET
                elif t == "slip_wall":
                    v = A.BC_DIRICHLET if c == d else A.BC_NEUMANN
                else:
                    raise ValueError(f"get_diffuse_tensor_bc: undefined BC type {t!r}")
                out[c][d] = v
        return out
    return side(bc_type_lo), side(bc_type_hi)


class TensorOp:
    """amrex::MLTensorOp as DiffusionTensorOp drives it, for one single-box level:
    alpha a u - beta div tau = rhs, tau = eta (grad u + grad u^T) - (2/3) eta (div u) I.
    setDomainBC takes per-component types ([component][direction] per side, diffuse_tensor_bc), then
    setScalars / setACoeffs / setShearViscosity / setLevelBC and solve (MLMG::solve) or apply (div tau)."""

    def __init__(self, geom: Geometry, options: A.Options | None = None, stream=None):
        self.geom = geom
        self.options = options or A.default_options(A.GBP_MAC)
        self.stream = stream
        self.ptr = None
        self.bc_lo = self.bc_hi = None
        self.alpha, self.beta = 1.0, 1.0
        self.a = 1.0
        self.eta = 1.0
        self.eta_faces = False
        self.vel = None
        self._dirty = True

    def __del__(self):
        if getattr(self, "ptr", None) is not None:
            A.load().gbp_tensor_destroy(self.ptr)
            self.ptr = None

    def setDomainBC(self, lo, hi):  # noqa: N802
        self.bc_lo = [[int(v) for v in comp] for comp in lo]
        self.bc_hi = [[int(v) for v in comp] for comp in hi]
        if self.ptr is not None:
            A.load().gbp_tensor_destroy(self.ptr)
            self.ptr = None

    def setScalars(self, alpha, beta):  # noqa: N802
        self.alpha, self.beta = float(alpha), float(beta)
        self._dirty = True

    def setACoeffs(self, lev, a):  # noqa: N802
        if lev != 0:
            raise ValueError("single level only")
        self.a = a
        self._dirty = True

    def setShearViscosity(self, lev, eta):  # noqa: N802
        """eta: [eta_x, eta_y, eta_z] face tensors, a cell tensor (averaged to the faces as
        average_velocity_eta_to_faces does) or a float."""
        if lev != 0:
            raise ValueError("single level only")
        self.eta = eta
        self._dirty = True

    def setLevelBC(self, lev, vel):  # noqa: N802
        """vel (3, nz+2, ny+2, nx+2): the ghost cells next to Dirichlet faces hold the face values."""
        if lev != 0:
            raise ValueError("single level only")
        self.vel = vel

    def _push(self):
        L = A.load()
        if self.ptr is None:
            if self.bc_lo is None:
                raise RuntimeError("setDomainBC must be called first")
            lo = (ctypes.c_int * 9)(*[self.bc_lo[c][d] for c in range(3) for d in range(3)])
            hi = (ctypes.c_int * 9)(*[self.bc_hi[c][d] for c in range(3) for d in range(3)])
            h = ctypes.c_void_p()
            A.check(L.gbp_tensor_create(ctypes.byref(self.geom.c()), lo, hi, ctypes.byref(self.options),
                                        _stream_ptr(self.stream), ctypes.byref(h)), "gbp_tensor_create")
            self.ptr = h
            self._dirty = True
        else:
            A.check(L.gbp_tensor_set_options(self.ptr, ctypes.byref(self.options)), "gbp_tensor_set_options")
        if not self._dirty:
            return
        a_t = self.a if isinstance(self.a, torch.Tensor) else None
        a0 = 0.0 if a_t is not None else float(self.a)
        a_ref = _ref(array4(a_t)) if a_t is not None else None
        if isinstance(self.eta, (list, tuple)):
            e = [array4(x) for x in self.eta]
            rc = L.gbp_tensor_set_coeffs(self.ptr, self.alpha, a_ref, a0, self.beta, None, _ref(e[0]), _ref(e[1]),
                                         _ref(e[2]), 0.0)
        elif isinstance(self.eta, torch.Tensor):
            rc = L.gbp_tensor_set_coeffs(self.ptr, self.alpha, a_ref, a0, self.beta, _ref(array4(self.eta)), None,
                                         None, None, 0.0)
        else:
            rc = L.gbp_tensor_set_coeffs(self.ptr, self.alpha, a_ref, a0, self.beta, None, None, None, None,
                                         float(self.eta))
        A.check(rc, "gbp_tensor_set_coeffs")
        self._dirty = False

    def solve(self, vel=None, rhs=None, rtol=1e-11, atol=1e-14):
        """MLMG::solve(velocity, rhs, rtol, atol): vel (setLevelBC's if None) is the initial guess and the output."""
        if vel is not None:
            self.vel = vel
        self.options.rtol = float(rtol)
        self.options.atol = float(atol)
        self._push()
        st = A.Stats()
        A.check(A.load().gbp_tensor_solve(self.ptr, _ref(array4(rhs)), _ref(array4(self.vel, 1)), ctypes.byref(st)),
                "gbp_tensor_solve")
        return st.as_dict()

    def apply(self, divtau, vel=None):
        """divtau (3, nz, ny, nx) = div tau of vel (MLMG::apply with setScalars(0, -1))."""
        if vel is not None:
            self.vel = vel
        self._push()
        A.check(A.load().gbp_tensor_apply(self.ptr, _ref(array4(self.vel, 1)), _ref(array4(divtau))),
                "gbp_tensor_apply")
        return divtau


def diffuse_velocity(geom: Geometry, bc_lo, bc_hi, velocity, density, eta, dt, options=None, stream=None):
    """DiffusionTensorOp::diffuse_velocity for one level: (rho - dt div tau) u = rho u, with eta the cell
    viscosity averaged to the faces. velocity (3, nz+2, ny+2, nx+2) is solved in place (its ghost cells
    hold the Dirichlet values); bc_lo / bc_hi per component ([component][direction])."""
    op = TensorOp(geom, options=options, stream=stream)
    op.setDomainBC(bc_lo, bc_hi)
    op.setScalars(1.0, dt)
    op.setACoeffs(0, density)
    op.setShearViscosity(0, eta)
    op.setLevelBC(0, velocity)
    rhs = (density[None] * velocity[:, 1:-1, 1:-1, 1:-1]).contiguous()
    return op.solve(rhs=rhs, rtol=op.options.rtol, atol=op.options.atol)


def compute_divtau(geom: Geometry, bc_lo, bc_hi, velocity, density, eta, advect_momentum=True, options=None,
                   stream=None):
    """DiffusionTensorOp::compute_divtau for one level: div tau of velocity, divided by rho when the
    momentum is not advected (:302-316). Returns a (3, nz, ny, nx) tensor."""
    op = TensorOp(geom, options=options, stream=stream)
    op.setDomainBC(bc_lo, bc_hi)
    op.setScalars(1.0, 1.0)
    op.setACoeffs(0, 1.0)
    op.setShearViscosity(0, eta)
    out = torch.empty((3, velocity.shape[1] - 2, velocity.shape[2] - 2, velocity.shape[3] - 2),
                      dtype=torch.float64, device=velocity.device)
    op.apply(out, velocity)
    if not advect_momentum:
        out /= density[None]
    return out
