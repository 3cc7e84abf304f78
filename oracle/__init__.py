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

    def __init__(self, n, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), bclo=(0, 0, 0), bchi=None):
        self.n = tuple(int(v) for v in n)
        self.lo = tuple(float(v) for v in lo)
        self.hi = tuple(float(v) for v in hi)
        self.h = tuple((self.hi[d] - self.lo[d]) / self.n[d] for d in range(3))
        self.bclo = tuple(int(v) for v in bclo)
        self.bchi = tuple(int(v) for v in (bchi if bchi is not None else bclo))
        for d in range(3):
            if (self.bclo[d] == PERIODIC) != (self.bchi[d] == PERIODIC):
                raise ValueError("periodic must be set on both sides")
        self._c = _Grid((ctypes.c_int * 3)(*self.n), (ctypes.c_double * 3)(*self.h),
                        (ctypes.c_int * 3)(*self.bclo), (ctypes.c_int * 3)(*self.bchi))

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
