"""CPU oracle for the projection hot path -- test infrastructure only.

Parity status: parity unpinned (the reference's MLMG lives in AMReX / AMReX-Hydro, which are
not vendored with incflo, and incflo ships no golden projection outputs). The C restatement in
``proj_oracle.c`` is pinned instead by incflo's analytic Taylor-Green pressure
(src/derive/incflo_error.cpp:33-34), by an independent numpy assembly of the same element
matrices, and by discrete identities; see tests/test_oracle.py.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline may import this module.

Array conventions (numpy, C order, so the LAST axis is x):
  node arrays  shape (nnz, nny, nnx), nn = n in a periodic direction, n+1 otherwise
  cell arrays  shape (nz, ny, nx)
  velocity     shape (3, nz+2, ny+2, nx+2): one ghost layer, read only on inflow faces
  face arrays  x: (nz, ny, nx+1), y: (nz, ny+1, nx), z: (nz+1, ny, nx)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

PERIODIC, DIRICHLET, NEUMANN, INFLOW = 0, 1, 2, 3

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libproj_oracle.so")
_lib = None


class _Grid(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int * 3),
        ("h", ctypes.c_double * 3),
        ("bclo", ctypes.c_int * 3),
        ("bchi", ctypes.c_int * 3),
        ("mask", ctypes.c_void_p),
    ]


def build() -> str:
    """Compile the oracle with its Makefile (gcc + OpenMP) and return the library path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(_HERE, "proj_oracle.c")
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER(_Grid)
        d = ctypes.c_void_p
        L.or_nodal_dims.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
        L.or_nodal_volume.argtypes = [P, d]
        L.or_nodal_stencil.argtypes = [P, d, d]
        L.or_nodal_apply.argtypes = [P, d, d, d]
        L.or_nodal_rhs.argtypes = [P, d, d]
        L.or_nodal_gradient.argtypes = [P, d, d]
        L.or_nodal_resid_norm.argtypes = [P, d, d, d, d]
        L.or_nodal_resid_norm.restype = ctypes.c_double
        L.or_nodal_solve.argtypes = [P, d, d, d, ctypes.c_double, ctypes.c_double, ctypes.c_int, d]
        L.or_nodal_project.argtypes = [P, d, d, d, d, ctypes.c_double, ctypes.c_double, ctypes.c_int, d]
        L.or_mac_rhs.argtypes = [P, d, d, d, d]
        L.or_mac_apply.argtypes = [P, d, d, d, d, d]
        L.or_mac_correct.argtypes = [P, d, d, d, d, d, d, d]
        L.or_mac_solve.argtypes = [P, d, d, d, d, d, ctypes.c_double, ctypes.c_double, ctypes.c_int, d]
        L.or_mac_project.argtypes = [P, d, d, d, d, d, d, d, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_int, d]
        L.or_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


class Grid:
    """Single-box domain: n cells, extent [lo, hi], boundary codes per side."""

    def __init__(self, n, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), bclo=(0, 0, 0), bchi=None, mask=None):
        self.n = tuple(int(v) for v in n)
        self.lo = tuple(float(v) for v in lo)
        self.hi = tuple(float(v) for v in hi)
        self.h = tuple((self.hi[d] - self.lo[d]) / self.n[d] for d in range(3))
        self.bclo = tuple(int(v) for v in bclo)
        self.bchi = tuple(int(v) for v in (bchi if bchi is not None else bclo))
        for d in range(3):
            if (self.bclo[d] == PERIODIC) != (self.bchi[d] == PERIODIC):
                raise ValueError("periodic must be set on both sides")
        # overset mask (nodal): unique nodes (node_shape), 0 = phi fixed at 0 (incflo's mixed BCs)
        self.mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        if self.mask is not None and self.mask.shape != self.node_shape:
            raise ValueError("mask must have the unique-node shape")
        self._c = _Grid((ctypes.c_int * 3)(*self.n), (ctypes.c_double * 3)(*self.h),
                        (ctypes.c_int * 3)(*self.bclo), (ctypes.c_int * 3)(*self.bchi),
                        self.mask.ctypes.data if self.mask is not None else None)

    def periodic(self, d):
        return self.bclo[d] == PERIODIC

    @property
    def node_shape(self):
        nn = [self.n[d] if self.periodic(d) else self.n[d] + 1 for d in range(3)]
        return (nn[2], nn[1], nn[0])

    @property
    def cell_shape(self):
        return (self.n[2], self.n[1], self.n[0])

    def face_shape(self, d):
        s = [self.n[2], self.n[1], self.n[0]]
        s[2 - d] += 1
        return tuple(s)

    @property
    def ref(self):
        return ctypes.byref(self._c)


def num_threads() -> int:
    return lib().or_num_threads()


# ---------------------------------------------------------------------------------- nodal
def nodal_volume(g: Grid):
    v = np.zeros(g.node_shape)
    lib().or_nodal_volume(g.ref, _p(v))
    return v


def nodal_stencil(g: Grid, sigma):
    st = np.zeros(g.node_shape + (27,))
    lib().or_nodal_stencil(g.ref, _p(np.ascontiguousarray(sigma, dtype=np.float64)), _p(st))
    return st


def nodal_apply(g: Grid, sigma, phi):
    out = np.zeros(g.node_shape)
    lib().or_nodal_apply(g.ref, _p(np.ascontiguousarray(sigma, dtype=np.float64)),
                         _p(np.ascontiguousarray(phi, dtype=np.float64)), _p(out))
    return out


def nodal_rhs(g: Grid, vel_g):
    out = np.zeros(g.node_shape)
    lib().or_nodal_rhs(g.ref, _p(np.ascontiguousarray(vel_g, dtype=np.float64)), _p(out))
    return out


def nodal_gradient(g: Grid, phi):
    out = np.zeros((3,) + g.cell_shape)
    lib().or_nodal_gradient(g.ref, _p(np.ascontiguousarray(phi, dtype=np.float64)), _p(out))
    return out


def nodal_resid_norm(g: Grid, sigma, rhs, phi):
    bn = ctypes.c_double(0.0)
    rn = lib().or_nodal_resid_norm(g.ref, _p(np.ascontiguousarray(sigma, dtype=np.float64)),
                                   _p(np.ascontiguousarray(rhs, dtype=np.float64)),
                                   _p(np.ascontiguousarray(phi, dtype=np.float64)),
                                   ctypes.cast(ctypes.byref(bn), ctypes.c_void_p))
    return rn, bn.value


def nodal_solve(g: Grid, sigma, rhs, phi0=None, rtol=1e-13, atol=0.0, maxiter=400):
    phi = np.zeros(g.node_shape) if phi0 is None else np.array(phi0, dtype=np.float64, copy=True)
    stats = np.zeros(4)
    st = lib().or_nodal_solve(g.ref, _p(np.ascontiguousarray(sigma, dtype=np.float64)),
                              _p(np.ascontiguousarray(rhs, dtype=np.float64)), _p(phi),
                              rtol, atol, maxiter, _p(stats))
    return phi, {"status": st, "iters": int(stats[0]), "rel_resid": stats[1],
                 "rhs_norm": stats[2], "initial_rel_resid": stats[3]}


def nodal_project(g: Grid, sigma, vel_g, rtol=1e-13, atol=0.0, maxiter=400):
    """Full nodal projection on copies: returns (vel_new, phi, gradphi, stats)."""
    vel = np.array(vel_g, dtype=np.float64, copy=True, order="C")
    phi = np.zeros(g.node_shape)
    grad = np.zeros((3,) + g.cell_shape)
    stats = np.zeros(4)
    st = lib().or_nodal_project(g.ref, _p(np.ascontiguousarray(sigma, dtype=np.float64)), _p(vel),
                                _p(phi), _p(grad), rtol, atol, maxiter, _p(stats))
    return vel, phi, grad, {"status": st, "iters": int(stats[0]), "rel_resid": stats[1],
                            "rhs_norm": stats[2]}


# ------------------------------------------------------------------------------------ MAC
def mac_rhs(g: Grid, ux, uy, uz):
    out = np.zeros(g.cell_shape)
    lib().or_mac_rhs(g.ref, _p(np.ascontiguousarray(ux, dtype=np.float64)),
                     _p(np.ascontiguousarray(uy, dtype=np.float64)),
                     _p(np.ascontiguousarray(uz, dtype=np.float64)), _p(out))
    return out


def mac_apply(g: Grid, beta, phi):
    out = np.zeros(g.cell_shape)
    b = [np.ascontiguousarray(x, dtype=np.float64) for x in beta]
    lib().or_mac_apply(g.ref, _p(b[0]), _p(b[1]), _p(b[2]),
                       _p(np.ascontiguousarray(phi, dtype=np.float64)), _p(out))
    return out


def mac_solve(g: Grid, beta, rhs, phi0=None, rtol=1e-13, atol=0.0, maxiter=400):
    phi = np.zeros(g.cell_shape) if phi0 is None else np.array(phi0, dtype=np.float64, copy=True)
    b = [np.ascontiguousarray(x, dtype=np.float64) for x in beta]
    stats = np.zeros(4)
    st = lib().or_mac_solve(g.ref, _p(b[0]), _p(b[1]), _p(b[2]),
                            _p(np.ascontiguousarray(rhs, dtype=np.float64)), _p(phi),
                            rtol, atol, maxiter, _p(stats))
    return phi, {"status": st, "iters": int(stats[0]), "rel_resid": stats[1],
                 "rhs_norm": stats[2], "initial_rel_resid": stats[3]}


def mac_project(g: Grid, beta, umac, phi0=None, rtol=1e-13, atol=0.0, maxiter=400):
    """Full MAC projection on copies: returns (umac_new, phi, stats)."""
    u = [np.array(x, dtype=np.float64, copy=True, order="C") for x in umac]
    b = [np.ascontiguousarray(x, dtype=np.float64) for x in beta]
    phi = np.zeros(g.cell_shape) if phi0 is None else np.array(phi0, dtype=np.float64, copy=True)
    stats = np.zeros(4)
    st = lib().or_mac_project(g.ref, _p(b[0]), _p(b[1]), _p(b[2]), _p(u[0]), _p(u[1]), _p(u[2]),
                              _p(phi), int(phi0 is not None), rtol, atol, maxiter, _p(stats))
    return u, phi, {"status": st, "iters": int(stats[0]), "rel_resid": stats[1],
                    "rhs_norm": stats[2]}


def _inout_faces(g: Grid, dd_lo, dd_hi, getter):
    """Yield (d, side, view) for every marked face; view is a writable array of normal velocities."""
    for d in range(3):
        for side, on in ((0, dd_lo[d]), (1, dd_hi[d])):
            if on:
                yield d, side, getter(d, side)


def _inout_scale(g: Grid, faces):
    """HydroUtils::enforceInOutSolvability (AMReX-Hydro, not vendored; called by incflo at
    src/projection/incflo_apply_nodal_projection.cpp:166-179 and
    src/convection/incflo_compute_MAC_projected_velocities.cpp:266-270): the flux into the domain
    over the marked faces (area x normal velocity, positive = inflow) is split into inflow and
    outflow; every outflow velocity is multiplied by inflow / outflow so the net flux is zero."""
    faces = list(faces)
    inflow = outflow = 0.0
    for d, side, v in faces:
        area = g.h[(d + 1) % 3] * g.h[(d + 2) % 3]
        into = -v if side else v
        inflow += area * into[into > 0].sum()
        outflow -= area * into[into < 0].sum()
    if outflow > 0.0:
        alpha = inflow / outflow
        for d, side, v in faces:
            into = -v if side else v
            v[into < 0] *= alpha
    return inflow, outflow


def enforce_inout_solvability(g: Grid, vel, dd_lo, dd_hi):
    """Cell velocity (3, nz+2, ny+2, nx+2) whose boundary ghost cells hold the boundary values;
    returns (scaled copy, inflow, outflow)."""
    v = np.array(vel, dtype=np.float64, copy=True)

    def getter(d, side):
        sl = [slice(1, -1)] * 3
        sl[2 - d] = -1 if side else 0
        return v[(d,) + tuple(sl)]

    # views share memory with v, so scaling them scales v
    inflow, outflow = _inout_scale(g, _inout_faces(g, dd_lo, dd_hi, getter))
    return v, inflow, outflow


def mac_enforce_inout_solvability(g: Grid, umac, dd_lo, dd_hi):
    """Face velocities (x: (nz, ny, nx+1), ...): scales the boundary faces 0 / n; returns
    (scaled copies, inflow, outflow)."""
    u = [np.array(x, dtype=np.float64, copy=True) for x in umac]

    def getter(d, side):
        sl = [slice(None)] * 3
        sl[2 - d] = -1 if side else 0
        return u[d][tuple(sl)]

    inflow, outflow = _inout_scale(g, _inout_faces(g, dd_lo, dd_hi, getter))
    return u, inflow, outflow


def mol_extrap_to_faces(g: Grid, vel, use_inflow=True):
    """Normal velocity on faces from cell velocity, the method-of-lines face extrapolation incflo's
    ApplyCCProjection uses (MOL::ExtrapVelToFaces, AMReX-Hydro, not vendored; called at
    src/projection/incflo_apply_cc_projection.cpp:350-353), restated: each cell's value is
    extrapolated to its faces with a monotonised-central slope, the two face states are upwinded by
    their average (zero when they diverge or the average is below 1e-10 in magnitude). Boundaries:
    periodic faces wrap; wall (Neumann) faces carry 0; inflow faces carry the ghost-cell value
    (0 when use_inflow is false); outflow (Dirichlet) faces take the adjacent interior value; cells
    next to a non-periodic boundary use a zero slope.

    vel: (3, nz+2, ny+2, nx+2); returns [ux (nz, ny, nx+1), uy (nz, ny+1, nx), uz (nz+1, ny, nx)]."""
    small = 1e-10
    out = []
    for d in range(3):
        ax = 2 - d
        n = g.n[d]
        q = np.moveaxis(vel[d][1:-1, 1:-1, 1:-1], ax, -1)  # (..., n) interior values along d
        if g.periodic(d):
            qm, qp = np.roll(q, 1, axis=-1), np.roll(q, -1, axis=-1)
        else:
            qm = np.concatenate([q[..., :1], q[..., :-1]], axis=-1)
            qp = np.concatenate([q[..., 1:], q[..., -1:]], axis=-1)
        dl, dr, dc = 2.0 * (q - qm), 2.0 * (qp - q), 0.5 * (qp - qm)
        slope = np.minimum(np.minimum(np.abs(dl), np.abs(dr)), np.abs(dc))
        slope = np.where(dl * dr > 0.0, np.where(dc > 0.0, slope, -slope), 0.0)
        if not g.periodic(d):
            slope[..., 0] = 0.0
            slope[..., -1] = 0.0
        right_of_face = q - 0.5 * slope   # state just right of face i (cell i)
        left_of_face = q + 0.5 * slope    # state just left of face i+1 (cell i)
        f = np.zeros(q.shape[:-1] + (n + 1,))
        # interior faces 1..n-1 (and the periodic face 0 == n)
        um = left_of_face[..., :-1]
        up = right_of_face[..., 1:]
        avg = 0.5 * (um + up)
        val = np.where(avg >= small, um, np.where(avg <= -small, up, 0.0))
        val = np.where((um < 0.0) & (up > 0.0), 0.0, val)
        f[..., 1:n] = val
        if g.periodic(d):
            um, up = left_of_face[..., -1], right_of_face[..., 0]
            avg = 0.5 * (um + up)
            v = np.where(avg >= small, um, np.where(avg <= -small, up, 0.0))
            v = np.where((um < 0.0) & (up > 0.0), 0.0, v)
            f[..., 0] = v
            f[..., n] = v
        else:
            for side, bc in ((0, g.bclo[d]), (1, g.bchi[d])):
                k = n if side else 0
                if bc == DIRICHLET:
                    f[..., k] = q[..., -1 if side else 0]
                elif bc == INFLOW and use_inflow:
                    gsl = [slice(1, -1)] * 3
                    gsl[ax] = -1 if side else 0
                    f[..., k] = vel[d][tuple(gsl)]  # the boundary ghost cell holds the inflow value
                else:
                    f[..., k] = 0.0
        out.append(np.ascontiguousarray(np.moveaxis(f, -1, ax)))
    return out


def cc_projection(g: Grid, vel, rho, gp, p_cc, *, vel_old=None, rho0=1.0, constant_density=False, time=0.0,
                  dt=1.0, prev_dt=1.0, scaling_factor=1.0, incremental=False, use_inflow=True, rtol=1e-13):
    """incflo::ApplyCCProjection for one level, non-EB (src/projection/incflo_apply_cc_projection.cpp:199-487):
    gp add-back (:214-238), U^n subtraction for incremental / small-dt (:241-249), MOL face velocities
    (:350-353), MAC projection with beta = s / rho_face, rho_face the arithmetic mean of the two cells
    (:276-323, :366), fluxes -beta grad phi averaged to cells (:392-399), then u += gphi, p_cc = phi
    (+= when incremental), gp = -gphi rho / s (-= when incremental) (:401-463), U^n added back (:471-477).

    vel (3, nz+2, ny+2, nx+2) with inflow ghosts; rho (nz+2, ny+2, nx+2) with ghosts (the ghost across
    a Dirichlet face is used); gp (3, nz, ny, nx); p_cc (nz, ny, nx). Returns new copies
    (vel, gp, p_cc, umac, phi, stats)."""
    v = np.array(vel, dtype=np.float64, copy=True)
    gp = np.array(gp, dtype=np.float64, copy=True)
    p_cc = np.array(p_cc, dtype=np.float64, copy=True)
    s = scaling_factor
    small_dt = time > 0.0 and dt < 0.1 * prev_dt
    sub_old = small_dt or incremental
    rc = np.full(g.cell_shape, rho0) if constant_density else rho[1:-1, 1:-1, 1:-1]
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))
    if not incremental:
        v[inner] += gp * (s / rc)
    if sub_old:
        v[inner] -= vel_old
    umac = mol_extrap_to_faces(g, v, use_inflow=use_inflow and not sub_old)
    if constant_density:
        beta = [np.full(g.face_shape(d), s / rho0) for d in range(3)]
    else:
        beta = []
        for d in range(3):
            ax = 2 - d
            core = [slice(1, -1)] * 3
            core[ax] = slice(None)
            r = np.moveaxis(rho[tuple(core)], ax, -1)  # (..., n+2) with both ghosts along d
            if g.periodic(d):
                rr = r[..., 1:-1]
                r = np.concatenate([rr[..., -1:], rr, rr[..., :1]], axis=-1)
            rf = 0.5 * (r[..., :-1] + r[..., 1:])
            beta.append(np.ascontiguousarray(np.moveaxis(s / rf, -1, ax)))
    unew, phi, st = mac_project(g, beta, umac, rtol=rtol)
    gphi = np.empty((3,) + g.cell_shape)
    for d in range(3):
        ax = 2 - d
        F = np.moveaxis(unew[d] - umac[d], ax, -1)
        gphi[d] = np.moveaxis(0.5 * (F[..., :-1] + F[..., 1:]), -1, ax)
    v[inner] += gphi
    if incremental:
        p_cc += phi
        gp -= gphi * rc / s
    else:
        p_cc = phi.copy()
        gp = -gphi * rc / s
    if sub_old:
        v[inner] += vel_old
    return v, gp, p_cc, unew, phi, st
