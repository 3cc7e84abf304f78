"""Host-side mirror of the reference's projection interface, over the C ABI.

Classes and methods keep the names and argument meaning of the AMReX-Hydro projectors that incflo
drives, so code written against them reads the same:

  NodalProjector   Hydro::NodalProjector as used in incflo::ApplyNodalProjection
                   (src/projection/incflo_apply_nodal_projection.cpp:181-219)
  MacProjector     Hydro::MacProjector as used in incflo::compute_MAC_projected_velocities
                   (src/convection/incflo_compute_MAC_projected_velocities.cpp:93-133, 272-299)
  apply_nodal_projection   incflo::ApplyNodalProjection(density, time, scaling_factor,
                   incremental) for one level (:29-93 plus :95-267), fused on the device.

Fields are CUDA float64 torch tensors (torch is only the allocator here). Layout, last axis x:
  cell fields   (ncomp, nz+2g, ny+2g, nx+2g) or (nz+2g, ny+2g, nx+2g); ``ng`` gives g
  nodal fields  (nz+1, ny+1, nx+1)
  face fields   x: (nz, ny, nx+1), y: (nz, ny+1, nx), z: (nz+1, ny, nx)
Errors raise ProjectionError (status code + message); nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import torch

from . import _abi as A
from ._abi import BC_DIRICHLET, BC_INFLOW, BC_NEUMANN, BC_PERIODIC, BC_ROBIN  # noqa: F401

LinOpBCType = {
    "Periodic": BC_PERIODIC,
    "Dirichlet": BC_DIRICHLET,
    "Neumann": BC_NEUMANN,
    "inflow": BC_INFLOW,
    "Robin": BC_ROBIN,
}


@dataclass
class Geometry:
    """amrex::Geometry of one single-box level: cell counts and physical extent."""

    n_cell: tuple
    prob_lo: tuple = (0.0, 0.0, 0.0)
    prob_hi: tuple = (1.0, 1.0, 1.0)

    def c(self) -> A.Geometry:
        g = A.Geometry()
        for d in range(3):
            g.n_cell[d] = int(self.n_cell[d])
            g.prob_lo[d] = float(self.prob_lo[d])
            g.prob_hi[d] = float(self.prob_hi[d])
        return g

    @property
    def dx(self):
        return tuple((self.prob_hi[d] - self.prob_lo[d]) / self.n_cell[d] for d in range(3))


@dataclass
class LPInfo:
    """amrex::LPInfo: only the coarsening depth matters to this solver."""

    max_coarsening_level: int = 100

    def setMaxCoarseningLevel(self, n):  # noqa: N802 (reference name)
        self.max_coarsening_level = int(n)
        return self


def array4(t: torch.Tensor, ng: int = 0, lo=None) -> A.Array4:
    """Describe a CUDA float64 tensor as an amrex::Array4-like view for the C ABI."""
    if not isinstance(t, torch.Tensor) or t.dtype != torch.float64 or not t.is_cuda:
        raise TypeError("fields must be CUDA float64 tensors")
    if t.dim() not in (3, 4):
        raise ValueError("fields are 3-D (one component) or 4-D (components first)")
    a = A.Array4()
    a.data = t.data_ptr()
    shape = t.shape[-3:]
    lo = (-ng, -ng, -ng) if lo is None else lo
    for d in range(3):
        a.lo[d] = int(lo[d])
        a.hi[d] = int(lo[d]) + int(shape[2 - d]) - 1
    if t.stride(-1) != 1:
        raise ValueError("the x axis (last) must be contiguous")
    a.jstride = t.stride(-2)
    a.kstride = t.stride(-3)
    a.ncomp = int(t.shape[0]) if t.dim() == 4 else 1
    a.nstride = t.stride(0) if t.dim() == 4 else 0
    return a


def _ref(a):
    return ctypes.byref(a) if a is not None else None


def _stream_ptr(stream):
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


class _Plan:
    def __init__(self, geom: Geometry, kind: int, bc_lo, bc_hi, options: A.Options, stream=None):
        A.load()
        self.geom = geom
        self.kind = kind
        self.options = options
        self.ptr = ctypes.c_void_p()
        lo = (ctypes.c_int * 3)(*[int(v) for v in bc_lo])
        hi = (ctypes.c_int * 3)(*[int(v) for v in bc_hi])
        A.check(A.load().gbp_plan_create(ctypes.byref(geom.c()), kind, lo, hi, ctypes.byref(options),
                                         _stream_ptr(stream), ctypes.byref(self.ptr)), "gbp_plan_create")
        self.bc_lo, self.bc_hi = tuple(bc_lo), tuple(bc_hi)

    def set_options(self, options: A.Options):
        self.options = options
        A.check(A.load().gbp_plan_set_options(self.ptr, ctypes.byref(options)), "gbp_plan_set_options")

    def device_bytes(self) -> int:
        return int(A.load().gbp_plan_device_bytes(self.ptr))

    def __del__(self):
        try:
            if self.ptr:
                A.load().gbp_plan_destroy(self.ptr)
                self.ptr = ctypes.c_void_p()
        except Exception:
            pass


def make_options(kind: int, **kw) -> A.Options:
    """Options from keyword overrides; keys are the inputs-file keys (mg_rtol, maxiter, precision ...)."""
    o = A.default_options(kind)
    for k, v in kw.items():
        A.check(A.load().gbp_options_set(ctypes.byref(o), k.encode(), str(v).encode()), f"option {k}")
    return o


def options_from_inputs(kind: int, text: str, prefix=None) -> A.Options:
    """Parse ParmParse-style inputs text for the nodal_proj.* (or mac_proj.*) keys."""
    o = A.default_options(kind)
    prefix = prefix or ("nodal_proj" if kind == A.GBP_NODAL else "mac_proj")
    A.check(A.load().gbp_options_parse(ctypes.byref(o), prefix.encode(), text.encode()), "gbp_options_parse")
    return o


# ---------------------------------------------------------------------------------- nodal
class NodalProjector:
    """Hydro::NodalProjector(vel, sigma, geom, info) for one level.

    ``sigma`` is a cell tensor (nz, ny, nx) or a float (constant-density form). The plan (the
    multigrid hierarchy) is cached per geometry/boundary set and reused across projectors.
    """

    _plans: dict = {}

    def __init__(self, vel, sigma, geom: Geometry, info: LPInfo | None = None, ng: int = 1,
                 options: A.Options | None = None, stream=None):
        self.vel = vel
        self.sigma = sigma
        self.geom = geom
        self.info = info or LPInfo()
        self.ng = ng
        self.options = options or A.default_options(A.GBP_NODAL)
        self.options.max_coarsening_level = self.info.max_coarsening_level
        self.stream = stream
        self.bc_lo = self.bc_hi = None
        self.phi = None
        self.gradphi = None
        self.stats = None
        self.surrogate = None
        self.surrogate_level = 1
        self.mask = None

    def setDomainBC(self, lo, hi):  # noqa: N802 (reference name)
        self.bc_lo = tuple(LinOpBCType.get(b, b) for b in lo)
        self.bc_hi = tuple(LinOpBCType.get(b, b) for b in hi)

    def setOversetMask(self, mask):  # noqa: N802 (getLinOp().setOversetMask(lev, mask))
        """Nodal int32 tensor (nz+1, ny+1, nx+1): 0 = phi held at 0 (the Dirichlet part of a mixed
        boundary, incflo::make_nodalBC_mask), nonzero = solve. None removes it."""
        self.mask = mask

    def setSurrogate(self, surrogate, level: int = 1):  # noqa: N802 (no reference counterpart)
        """Learned warm start for zero-guess solves (incflo_gb300.surrogate.Surrogate), evaluated on
        multigrid level ``level``; None detaches it."""
        self.surrogate = surrogate
        self.surrogate_level = int(level)

    def _plan(self) -> _Plan:
        if self.bc_lo is None:
            raise RuntimeError("setDomainBC must be called before project")
        key = (tuple(self.geom.n_cell), tuple(self.geom.prob_lo), tuple(self.geom.prob_hi), self.bc_lo,
               self.bc_hi, self.options.max_coarsening_level, torch.cuda.current_device())
        plan = NodalProjector._plans.get(key)
        if plan is None:
            plan = _Plan(self.geom, A.GBP_NODAL, self.bc_lo, self.bc_hi, self.options, self.stream)
            NodalProjector._plans[key] = plan
        else:
            plan.set_options(self.options)
        return plan

    def project(self, rtol=None, atol=None, phi_guess: torch.Tensor | None = None):
        if rtol is not None:
            self.options.rtol = float(rtol)
        if atol is not None:
            self.options.atol = float(atol)
        plan = self._plan()
        L = A.load()
        if isinstance(self.sigma, torch.Tensor):
            A.check(L.gbp_nodal_set_sigma(plan.ptr, _ref(array4(self.sigma)), 0.0), "gbp_nodal_set_sigma")
        else:
            A.check(L.gbp_nodal_set_sigma(plan.ptr, None, float(self.sigma)), "gbp_nodal_set_sigma")
        # plans are shared between projectors of one geometry: (re)state the mask (when it changed)
        # and the warm start every call
        m = self.mask
        if getattr(plan, "mask_ref", None) is not m:
            if m is not None:
                if m.dtype != torch.int32 or not m.is_cuda or m.stride(-1) != 1:
                    raise TypeError("the overset mask is a CUDA int32 tensor, x contiguous")
                ia = A.IArray4()
                ia.data = m.data_ptr()
                ia.hi[0], ia.hi[1], ia.hi[2] = m.shape[2] - 1, m.shape[1] - 1, m.shape[0] - 1
                ia.jstride, ia.kstride = m.stride(1), m.stride(0)
                A.check(L.gbp_nodal_set_overset_mask(plan.ptr, ctypes.byref(ia)), "gbp_nodal_set_overset_mask")
            else:
                A.check(L.gbp_nodal_set_overset_mask(plan.ptr, None), "gbp_nodal_set_overset_mask")
            plan.mask_ref = m
        s = self.surrogate
        A.check(L.gbp_plan_set_surrogate(plan.ptr, s.ptr if s is not None else None, self.surrogate_level,
                                         int(s is not None)), "gbp_plan_set_surrogate")
        n = self.geom.n_cell
        dev = self.vel.device
        if phi_guess is not None:
            self.phi = phi_guess
        elif self.phi is None:
            self.phi = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device=dev)
        if self.gradphi is None:
            self.gradphi = torch.zeros((3, n[2], n[1], n[0]), dtype=torch.float64, device=dev)
        st = A.Stats()
        A.check(L.gbp_nodal_project(plan.ptr, _ref(array4(self.vel, self.ng)), _ref(array4(self.phi)),
                                    _ref(array4(self.gradphi)), int(phi_guess is not None), ctypes.byref(st)),
                "gbp_nodal_project")
        self.stats = st.as_dict()
        return self.stats

    def getPhi(self):  # noqa: N802
        return self.phi

    def getGradPhi(self):  # noqa: N802
        return self.gradphi

    def enforceInOutSolvability(self, dd_lo, dd_hi):  # noqa: N802
        """HydroUtils::enforceInOutSolvability on this projector's velocity (whose boundary ghost
        cells hold the boundary values) for the direction_dependent faces marked in dd_lo / dd_hi
        (incflo_apply_nodal_projection.cpp:166-179). Returns (inflow, outflow) before scaling."""
        plan = self._plan()
        io = (ctypes.c_double * 2)()
        A.check(A.load().gbp_enforce_inout_solvability(plan.ptr, _ref(array4(self.vel, self.ng)),
                                                       (ctypes.c_int * 3)(*dd_lo), (ctypes.c_int * 3)(*dd_hi), io),
                "gbp_enforce_inout_solvability")
        return io[0], io[1]


def _set_plan_eb(plan, eb_moments):
    """attach (or remove) cut cells on a cached nodal plan when they changed"""
    key = None if eb_moments is None else (eb_moments.data_ptr(), tuple(eb_moments.shape), eb_moments._version)
    if getattr(plan, "_eb_key", None) == key:
        return
    A.check(A.load().gbp_nodal_set_eb(plan.ptr, _ref(array4(eb_moments)) if eb_moments is not None else None),
            "gbp_nodal_set_eb")
    plan._eb_key = key


def apply_nodal_projection(geom: Geometry, bc_lo, bc_hi, vel, density, gp, p_nd, *, time=0.0, dt=1.0,
                           prev_dt=1.0, scaling_factor=1.0, incremental=False, set_inflow_bc=True,
                           vel_old=None, rho0=1.0, ng=1, options: A.Options | None = None, stream=None,
                           constant_density=False, surrogate=None, surrogate_level=1, eb_moments=None,
                           eb_inflow=None):
    """incflo::ApplyNodalProjection for one level, fused on the device; returns the stats dict.
    ``surrogate`` (incflo_gb300.surrogate.Surrogate) enables the learned warm start on multigrid level
    ``surrogate_level``; ``eb_moments`` (27, nz, ny, nx) the cut cells of an embedded boundary
    (incflo_gb300.eb.cylinder_moments, components p + 3q + 9r); ``eb_inflow`` = (eb_vel, dap, bcent),
    each (3, nz, ny, nx), the velocity on the embedded boundary with the boundary's area vector and
    centroid (incflo_gb300.eb.cylinder_boundary / eb_inflow_velocity; setEBInflowVelocity)."""
    options = options or A.default_options(A.GBP_NODAL)
    key = (tuple(geom.n_cell), tuple(geom.prob_lo), tuple(geom.prob_hi), tuple(bc_lo), tuple(bc_hi),
           options.max_coarsening_level, torch.cuda.current_device())
    plan = NodalProjector._plans.get(key)
    if plan is None:
        plan = _Plan(geom, A.GBP_NODAL, bc_lo, bc_hi, options, stream)
        NodalProjector._plans[key] = plan
    else:
        plan.set_options(options)
    A.check(A.load().gbp_plan_set_surrogate(plan.ptr, surrogate.ptr if surrogate is not None else None,
                                            int(surrogate_level), int(surrogate is not None)),
            "gbp_plan_set_surrogate")
    _set_plan_eb(plan, eb_moments)
    if eb_inflow is not None:
        ev, dap, bc = (array4(t) for t in eb_inflow)
        A.check(A.load().gbp_nodal_set_eb_inflow(plan.ptr, _ref(ev), _ref(dap), _ref(bc)), "gbp_nodal_set_eb_inflow")
    elif eb_moments is not None:
        A.check(A.load().gbp_nodal_set_eb_inflow(plan.ptr, None, None, None), "gbp_nodal_set_eb_inflow")
    st = A.Stats()
    rho_a = None if constant_density else array4(density, 0)
    A.check(A.load().gbp_apply_nodal_projection(
        plan.ptr, _ref(array4(vel, ng)), _ref(array4(vel_old, 0)) if vel_old is not None else None, _ref(rho_a),
        float(rho0), _ref(array4(gp)), _ref(array4(p_nd)) if p_nd is not None else None, float(time), float(dt),
        float(prev_dt), float(scaling_factor), int(incremental), int(set_inflow_bc), ctypes.byref(st)),
        "gbp_apply_nodal_projection")
    return st.as_dict()


def _fab_ptrs(arrays, keep):
    """array of nbox pointers to gbp_array4 (the C ABI's per-FAB argument); arrays: list of Array4"""
    arr = (A.Array4 * len(arrays))(*arrays)
    ptrs = (ctypes.POINTER(A.Array4) * len(arrays))(*[ctypes.pointer(arr[b]) for b in range(len(arrays))])
    keep.append((arr, ptrs))
    return ptrs


def _box_table(boxes):
    """boxes: [((lo_x, lo_y, lo_z), (hi_x, hi_y, hi_z)), ...] of valid cells -> 6 ints per box"""
    flat = [int(v) for lo, hi in boxes for v in (*lo, *hi)]
    return (ctypes.c_int * len(flat))(*flat)


def fab_array4(t, box, ng=0, nodal=False):
    """A FAB tensor of box ((lo), (hi)) with ng ghost cells (nodal: nodes lo..hi+1, no ghosts)."""
    lo = box[0]
    return array4(t, 0, lo=tuple(int(v) - (0 if nodal else ng) for v in lo))


def apply_nodal_projection_boxes(geom: Geometry, bc_lo, bc_hi, boxes, vel, density, gp, p_nd, *, time=0.0, dt=1.0,
                                 prev_dt=1.0, scaling_factor=1.0, incremental=False, set_inflow_bc=True,
                                 vel_old=None, rho0=1.0, ng=1, options: A.Options | None = None, stream=None,
                                 constant_density=False):
    """incflo::ApplyNodalProjection for one level held in several boxes (the MultiFab's FABs): boxes =
    [(lo, hi), ...] valid cells tiling the domain; vel (ng ghost cells), density, gp, vel_old: one tensor
    per box; p_nd: one nodal tensor per box (nodes lo..hi+1). Returns the stats dict."""
    options = options or A.default_options(A.GBP_NODAL)
    key = (tuple(geom.n_cell), tuple(geom.prob_lo), tuple(geom.prob_hi), tuple(bc_lo), tuple(bc_hi),
           options.max_coarsening_level, torch.cuda.current_device())
    plan = NodalProjector._plans.get(key)
    if plan is None:
        plan = _Plan(geom, A.GBP_NODAL, bc_lo, bc_hi, options, stream)
        NodalProjector._plans[key] = plan
    else:
        plan.set_options(options)
    _set_plan_eb(plan, None)
    A.check(A.load().gbp_plan_set_surrogate(plan.ptr, None, 1, 0), "gbp_plan_set_surrogate")
    keep = []
    nb = len(boxes)

    def fabs(ts, g=0, nodal=False):
        if ts is None:
            return None
        if len(ts) != nb:
            raise ValueError("one tensor per box is required")
        return _fab_ptrs([fab_array4(t, boxes[b], g, nodal) for b, t in enumerate(ts)], keep)

    st = A.Stats()
    A.check(A.load().gbp_apply_nodal_projection_boxes(
        plan.ptr, nb, _box_table(boxes), fabs(vel, ng), fabs(vel_old), None if constant_density else fabs(density),
        float(rho0), fabs(gp), fabs(p_nd, 0, True), float(time), float(dt), float(prev_dt), float(scaling_factor),
        int(incremental), int(set_inflow_bc), ctypes.byref(st)), "gbp_apply_nodal_projection_boxes")
    return st.as_dict()


class AmrNodalProjector:
    """incflo::ApplyNodalProjection over two levels (finest_level = 1, refinement ratio 2): the composite
    nodal solve of one NodalProjector over both levels. ``fine_boxes``: the fine level's BoxArray as
    [(lo, hi)] of fine cells (inclusive, whole coarse cells). Fields per level: the coarse ones as
    tensors over the coarse cells (nodes for p_nd), the fine ones as lists of per-box tensors over each
    box's cells (nodes lo..hi+1 for p_nd); components first for velocities and gp."""

    def __init__(self, geom: Geometry, bc_lo, bc_hi, fine_boxes, options: A.Options | None = None, stream=None):
        L = A.load()
        self.geom = geom
        self.boxes = [(tuple(int(v) for v in lo), tuple(int(v) for v in hi)) for lo, hi in fine_boxes]
        self.options = options or A.default_options(A.GBP_NODAL)
        flat = (ctypes.c_int * (6 * len(self.boxes)))(*[v for lo, hi in self.boxes for v in (*lo, *hi)])
        self.ptr = ctypes.c_void_p()
        A.check(L.gbp_amr_create(ctypes.byref(geom.c()), (ctypes.c_int * 3)(*[int(v) for v in bc_lo]),
                                 (ctypes.c_int * 3)(*[int(v) for v in bc_hi]), flat, len(self.boxes),
                                 ctypes.byref(self.options), _stream_ptr(stream), ctypes.byref(self.ptr)),
                "gbp_amr_create")

    def set_options(self, options: A.Options):
        self.options = options
        A.check(A.load().gbp_amr_set_options(self.ptr, ctypes.byref(options)), "gbp_amr_set_options")

    def device_bytes(self) -> int:
        return int(A.load().gbp_amr_device_bytes(self.ptr))

    def _boxes4(self, tensors):
        """(keep-alive, argument): the C ABI takes an array of nbox pointers to gbp_array4."""
        if tensors is None:
            return None, None
        if len(tensors) != len(self.boxes):
            raise ValueError("one tensor per fine box is required")
        arr = (A.Array4 * len(self.boxes))()
        for b, t in enumerate(tensors):
            arr[b] = array4(t, 0, lo=self.boxes[b][0])
        ptrs = (ctypes.POINTER(A.Array4) * len(self.boxes))(*[ctypes.pointer(arr[b]) for b in range(len(self.boxes))])
        return (arr, ptrs), ptrs

    def apply(self, vel_c, density_c, gp_c, p_c, vel_f, density_f, gp_f, p_f, *, scaling_factor=1.0,
              incremental=False, vel_old_c=None, vel_old_f=None, rho0=1.0, constant_density=False):
        keep = []

        def bx(t):
            a, p = self._boxes4(t)
            keep.append(a)
            return p

        st = A.Stats()
        rho_c = None if constant_density else array4(density_c, 0)
        A.check(A.load().gbp_amr_apply_nodal_projection(
            self.ptr, _ref(array4(vel_c)), _ref(array4(vel_old_c)) if vel_old_c is not None else None, _ref(rho_c),
            _ref(array4(gp_c)), _ref(array4(p_c)) if p_c is not None else None, bx(vel_f), bx(vel_old_f),
            None if constant_density else bx(density_f), bx(gp_f), bx(p_f), float(rho0), float(scaling_factor),
            int(incremental), ctypes.byref(st)), "gbp_amr_apply_nodal_projection")
        return st.as_dict()

    def __del__(self):
        try:
            if self.ptr:
                A.load().gbp_amr_destroy(self.ptr)
                self.ptr = ctypes.c_void_p()
        except Exception:
            pass


def apply_cc_projection(geom: Geometry, bc_lo, bc_hi, vel, density, gp, p_cc, umac, *, time=0.0, dt=1.0,
                        prev_dt=1.0, scaling_factor=1.0, incremental=False, set_inflow_bc=True, vel_old=None,
                        rho0=1.0, ng=1, ng_rho=1, options: A.Options | None = None, stream=None,
                        constant_density=False):
    """incflo::ApplyCCProjection for one level (non-EB), on the device; umac = [ux, uy, uz] face tensors
    receive the projected face velocities. density has ``ng_rho`` ghost layers. Returns the stats dict."""
    options = options or A.default_options(A.GBP_MAC)
    key = ("cc", tuple(geom.n_cell), tuple(geom.prob_lo), tuple(geom.prob_hi), tuple(bc_lo), tuple(bc_hi),
           options.max_coarsening_level, torch.cuda.current_device())
    plan = MacProjector._cc_plans.get(key)
    if plan is None:
        plan = _Plan(geom, A.GBP_MAC, bc_lo, bc_hi, options, stream)
        MacProjector._cc_plans[key] = plan
    else:
        plan.set_options(options)
    st = A.Stats()
    rho_a = None if constant_density else array4(density, ng_rho)
    u = [array4(x) for x in umac]
    A.check(A.load().gbp_apply_cc_projection(
        plan.ptr, _ref(array4(vel, ng)), _ref(array4(vel_old, 0)) if vel_old is not None else None, _ref(rho_a),
        float(rho0), _ref(array4(gp)), _ref(array4(p_cc)) if p_cc is not None else None, _ref(u[0]), _ref(u[1]),
        _ref(u[2]), float(time), float(dt), float(prev_dt), float(scaling_factor), int(incremental),
        int(set_inflow_bc), ctypes.byref(st)), "gbp_apply_cc_projection")
    return st.as_dict()


def average_down(fine: torch.Tensor, crse: torch.Tensor, ratio=(2, 2, 2), crse_lo=None, crse_hi=None, stream=None,
                 fine_lo=(0, 0, 0), crse_box_lo=(0, 0, 0)):
    """amrex::average_down of a cell field (components first, or one component): crse[box] = mean of its
    fine cells. Index spaces: fine_lo / crse_box_lo are the global indices of each tensor's first
    element; the coarse box defaults to the coarsened fine extent."""
    fa = array4(fine, 0, lo=fine_lo)
    ca = array4(crse, 0, lo=crse_box_lo)
    nc = fine.shape[0] if fine.dim() == 4 else 1
    if crse_lo is None:
        crse_lo = [fa.lo[d] // ratio[d] for d in range(3)]
        crse_hi = [(fa.hi[d] + 1) // ratio[d] - 1 for d in range(3)]
    A.check(A.load().gbp_average_down(_ref(fa), _ref(ca), (ctypes.c_int * 3)(*ratio), nc,
                                      (ctypes.c_int * 3)(*crse_lo), (ctypes.c_int * 3)(*crse_hi), _stream_ptr(stream)),
            "gbp_average_down")


def nodal_divergence(geom: Geometry, bc_lo, bc_hi, vel, ng=1, use_inflow=True, out=None, stream=None):
    """Nodal divergence of vel as the projection sees it (strong form, consistent for singular
    boundary sets). Returns (max |div|, out) with out a nodal (nz+1, ny+1, nx+1) tensor."""
    key = (tuple(geom.n_cell), tuple(geom.prob_lo), tuple(geom.prob_hi), tuple(bc_lo), tuple(bc_hi), 100,
           torch.cuda.current_device())
    plan = NodalProjector._plans.get(key)
    if plan is None:
        plan = _Plan(geom, A.GBP_NODAL, bc_lo, bc_hi, A.default_options(A.GBP_NODAL), stream)
        NodalProjector._plans[key] = plan
    n = geom.n_cell
    if out is None:
        out = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device=vel.device)
    m = ctypes.c_double()
    A.check(A.load().gbp_nodal_divergence(plan.ptr, _ref(array4(vel, ng)), int(use_inflow), _ref(array4(out)),
                                          ctypes.byref(m)), "gbp_nodal_divergence")
    return m.value, out


# ------------------------------------------------------------------------------------ MAC
class MacProjector:
    """Hydro::MacProjector(geom) for one level: initProjector / updateCoeffs / setUMAC / project."""

    _cc_plans: dict = {}

    def __init__(self, geom: Geometry, options: A.Options | None = None, stream=None):
        self.geom = geom
        self.options = options or A.default_options(A.GBP_MAC)
        self.stream = stream
        self.plan = None
        self.bc_lo = self.bc_hi = None
        self.beta = None
        self.umac = None
        self.stats = None
        self.robin = None
        self.eb = None
        self.eb_vel = None

    def needInitialization(self):  # noqa: N802
        return self.plan is None

    def initProjector(self, info: LPInfo | None = None, beta=None):  # noqa: N802
        """beta: [bx, by, bz] face tensors, or a float (the constant-density form dt/rho0)."""
        if info is not None:
            self.options.max_coarsening_level = info.max_coarsening_level
        self.beta = beta
        self.plan = None

    def setDomainBC(self, lo, hi):  # noqa: N802
        self.bc_lo = tuple(LinOpBCType.get(b, b) for b in lo)
        self.bc_hi = tuple(LinOpBCType.get(b, b) for b in hi)
        self.plan = None

    def setLevelBC(self, lev, levelbcdata=None, robinbc_a=None, robinbc_b=None, robinbc_f=None):  # noqa: N802
        """Robin data of the Robin sides: cell tensors (nz+2, ny+2, nx+2) with one ghost layer, read in
        the ghost cells next to each Robin face (a phi + b dphi/dn = f, f = 0)."""
        if lev != 0 or levelbcdata is not None:
            raise ValueError("single level only; Dirichlet values are zero")
        self.robin = (robinbc_a, robinbc_b, robinbc_f)
        self._push_robin()

    def _push_robin(self):
        if self.plan is None or self.robin is None:
            return
        a, b, f = self.robin
        A.check(A.load().gbp_mac_set_robin(self.plan.ptr, _ref(array4(a, 1)), _ref(array4(b, 1)),
                                           _ref(array4(f, 1)) if f is not None else None), "gbp_mac_set_robin")

    def setEB(self, vfrac, areafrac, facecent):  # noqa: N802
        """Cut cells of an embedded boundary (what the reference takes from the EB factory of its
        MultiFabs): vfrac (nz, ny, nx); areafrac = [x (nz, ny, nx+1), y, z] face tensors; facecent =
        [x (2, nz, ny, nx+1), y, z]: centroid offsets in cell widths along the two tangential
        directions in increasing order (AMReX's fcx / fcy / fcz). vfrac None removes the EB."""
        self.eb = None if vfrac is None else (vfrac, list(areafrac), list(facecent))
        self.eb_vel = None
        self._push_eb()
        self._push_beta()
        self._push_robin()

    def setEBInflowVelocity(self, lev, eb_vel):  # noqa: N802 (reference name)
        """The velocity on the embedded boundary (3, nz, ny, nx) of level `lev` (0 only); None removes
        it. Its flux out of each cut cell is part of the divergence of the next projections."""
        if lev != 0:
            raise ValueError("single-level MAC projector: lev must be 0")
        self.eb_vel = eb_vel
        self._push_eb_inflow()

    def _push_eb_inflow(self):
        if self.plan is None:
            return
        ev = getattr(self, "eb_vel", None)
        A.check(A.load().gbp_mac_set_eb_inflow(self.plan.ptr, _ref(array4(ev)) if ev is not None else None),
                "gbp_mac_set_eb_inflow")

    def _push_eb(self):
        if self.plan is None:
            return
        L = A.load()
        if self.eb is None:
            A.check(L.gbp_mac_set_eb(self.plan.ptr, None, None, None, None, None, None, None), "gbp_mac_set_eb")
            return
        v, ap, fc = self.eb
        a = [array4(x) for x in ap]
        f = [array4(x) for x in fc]
        A.check(L.gbp_mac_set_eb(self.plan.ptr, _ref(array4(v)), _ref(a[0]), _ref(a[1]), _ref(a[2]), _ref(f[0]),
                                 _ref(f[1]), _ref(f[2])), "gbp_mac_set_eb")

    def updateCoeffs(self, beta):  # noqa: N802
        self.beta = beta
        self._push_beta()

    def updateBeta(self, beta):  # noqa: N802
        self.beta = float(beta)
        self._push_beta()

    def setUMAC(self, umac):  # noqa: N802
        self.umac = list(umac)

    def enforceInOutSolvability(self, dd_lo, dd_hi):  # noqa: N802
        """HydroUtils::enforceInOutSolvability on the face velocities given to setUMAC
        (incflo_compute_MAC_projected_velocities.cpp:266-270). Returns (inflow, outflow)."""
        self._ensure()
        u = [array4(x) for x in self.umac]
        io = (ctypes.c_double * 2)()
        A.check(A.load().gbp_mac_enforce_inout_solvability(self.plan.ptr, _ref(u[0]), _ref(u[1]), _ref(u[2]),
                                                           (ctypes.c_int * 3)(*dd_lo), (ctypes.c_int * 3)(*dd_hi),
                                                           io), "gbp_mac_enforce_inout_solvability")
        return io[0], io[1]

    def _ensure(self):
        if self.plan is None:
            if self.bc_lo is None:
                raise RuntimeError("setDomainBC must be called before project")
            self.plan = _Plan(self.geom, A.GBP_MAC, self.bc_lo, self.bc_hi, self.options, self.stream)
            self._push_eb()
            self._push_eb_inflow()
            self._push_beta()
            self._push_robin()
        else:
            self.plan.set_options(self.options)

    def _push_beta(self):
        if self.plan is None or self.beta is None:  # None: set on the plan from the density already
            return
        L = A.load()
        if isinstance(self.beta, (list, tuple)):
            b = [array4(x) for x in self.beta]
            A.check(L.gbp_mac_set_beta(self.plan.ptr, _ref(b[0]), _ref(b[1]), _ref(b[2]), 0.0), "gbp_mac_set_beta")
        else:
            A.check(L.gbp_mac_set_beta(self.plan.ptr, None, None, None, float(self.beta)), "gbp_mac_set_beta")

    def project(self, rtol=None, atol=None, phi: torch.Tensor | None = None, phi_guess=True, ng_phi=0):
        """project(rtol, atol) or project(phi, rtol, atol): phi (cells) is the initial guess and output."""
        if rtol is not None:
            self.options.rtol = float(rtol)
        if atol is not None:
            self.options.atol = float(atol)
        self._ensure()
        u = [array4(x) for x in self.umac]
        st = A.Stats()
        pa = array4(phi, ng_phi) if phi is not None else None
        A.check(A.load().gbp_mac_project(self.plan.ptr, _ref(u[0]), _ref(u[1]), _ref(u[2]), _ref(pa),
                                         int(phi is not None and phi_guess), ctypes.byref(st)), "gbp_mac_project")
        self.stats = st.as_dict()
        return self.stats

    def setBetaFromDensityBoxes(self, boxes, rho, dt, ng=1):  # noqa: N802 (multi-box average_cellcenter_to_face)
        """beta = dt / (face average of rho) from one density tensor per box (ng ghost cells, read across
        Dirichlet sides)."""
        self._ensure()
        keep = []
        ptrs = _fab_ptrs([fab_array4(t, boxes[b], ng) for b, t in enumerate(rho)], keep)
        A.check(A.load().gbp_mac_set_beta_from_density_boxes(self.plan.ptr, len(boxes), _box_table(boxes), ptrs,
                                                             float(dt)), "gbp_mac_set_beta_from_density_boxes")
        self.beta = None  # set on the plan; not pushed again

    def projectBoxes(self, boxes, umac, phi=None, phi_guess=True, rtol=None, atol=None):  # noqa: N802
        """project() on a level held in several boxes: umac = [[ux, uy, uz] per box] (faces lo..hi+1 in
        their direction), phi = one cell tensor per box or None."""
        if rtol is not None:
            self.options.rtol = float(rtol)
        if atol is not None:
            self.options.atol = float(atol)
        self._ensure()
        keep = []
        u = [_fab_ptrs([fab_array4(umac[b][d], boxes[b]) for b in range(len(boxes))], keep) for d in range(3)]
        ph = None if phi is None else _fab_ptrs([fab_array4(t, boxes[b]) for b, t in enumerate(phi)], keep)
        st = A.Stats()
        A.check(A.load().gbp_mac_project_boxes(self.plan.ptr, len(boxes), _box_table(boxes), u[0], u[1], u[2], ph,
                                               int(phi is not None and phi_guess), ctypes.byref(st)),
                "gbp_mac_project_boxes")
        self.stats = st.as_dict()
        return self.stats

    def getFluxes(self, fluxes, phi, ng_phi=0):  # noqa: N802 (reference name)
        """MacProjector::getFluxes(fluxes, phi, loc): fluxes[d] = -beta grad phi on the faces of
        direction d (face centroids of cut faces), the correction project() applies to umac."""
        self._ensure()
        f = [array4(x) for x in fluxes]
        A.check(A.load().gbp_mac_get_fluxes(self.plan.ptr, _ref(array4(phi, ng_phi)), _ref(f[0]), _ref(f[1]),
                                            _ref(f[2])), "gbp_mac_get_fluxes")
        return fluxes
