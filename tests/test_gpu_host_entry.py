"""The host-buffer entry point gbp_apply_nodal_projection_host (the end-to-end path: uploads, the
projection and the copy-out of velocity, gp and p_nd by z-slabs behind the correction) against the
device-resident gbp_apply_nodal_projection on the same inputs: identical results (the same kernels on
the same data), for several slab counts, with and without p_nd; and against the oracle."""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
from incflo_gb300 import Geometry, _abi, apply_nodal_projection, make_options
from incflo_gb300.projection import _Plan
from tests.helpers import N, P, rel_l2

pytestmark = pytest.mark.gpu


def _case(n, seed=3):
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    vel = rng.standard_normal((3, n[2], n[1], n[0]))
    gp = 0.1 * rng.standard_normal((3, n[2], n[1], n[0]))
    return rho, vel, gp


@pytest.mark.parametrize("n", [(32, 24, 40), (16, 16, 8), (24, 20, 130)])
@pytest.mark.parametrize("with_pnd", [True, False])
def test_host_entry_matches_device_path(gpu_lib, n, with_pnd):
    bclo, bchi = (P, P, N), (P, P, N)
    ext = (n[0] / 32, n[1] / 32, n[2] / 32)  # isotropic cells
    rho, vel, gp = _case(n)
    geom = Geometry(n, (0, 0, 0), ext)
    opts = make_options(0, precision="mixed", mg_rtol=1e-11, mg_atol=0.0)
    # device-resident path
    vt = torch.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2), dtype=torch.float64, device="cuda")
    vt[:, 1:-1, 1:-1, 1:-1] = torch.from_numpy(vel)
    gt = torch.from_numpy(gp).cuda()
    pt = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device="cuda")
    st = apply_nodal_projection(geom, bclo, bchi, vt, torch.from_numpy(rho).cuda(), gt, pt, set_inflow_bc=False,
                                options=opts)
    assert st["status"] == 0
    # host path, pinned buffers
    lib = _abi.load()
    plan = _Plan(geom, _abi.GBP_NODAL, bclo, bchi, opts)
    vh = torch.from_numpy(np.ascontiguousarray(vel)).pin_memory()
    rh = torch.from_numpy(np.ascontiguousarray(rho)).pin_memory()
    gh = torch.from_numpy(np.ascontiguousarray(gp)).pin_memory()
    ph = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64).pin_memory()
    sth = _abi.Stats()
    rc = lib.gbp_apply_nodal_projection_host(plan.ptr, vh.data_ptr(), rh.data_ptr(), 1.0, gh.data_ptr(),
                                             ph.data_ptr() if with_pnd else None, 1.0, 0, ctypes.byref(sth))
    _abi.check(rc, "gbp_apply_nodal_projection_host")
    assert sth.status == 0 and sth.vcycles == st["vcycles"]
    np.testing.assert_array_equal(vh.numpy(), vt.cpu().numpy()[:, 1:-1, 1:-1, 1:-1])
    np.testing.assert_array_equal(gh.numpy(), gt.cpu().numpy())
    if with_pnd:
        np.testing.assert_array_equal(ph.numpy(), pt.cpu().numpy())


def test_host_entry_matches_oracle(gpu_lib):
    n, ext = (16, 16, 16), (1.0, 1.0, 1.0)
    bclo, bchi = (P, P, N), (P, P, N)
    rho, vel, gp = _case(n, seed=4)
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    vg = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vg[:, 1:-1, 1:-1, 1:-1] = vel + gp / rho[None]  # the gp add-back: u + sigma gp, sigma = 1 / rho
    vel_or, phi_or, _, st_or = O.nodal_project(g, 1.0 / rho, vg, rtol=1e-13)
    assert st_or["status"] == 0
    lib = _abi.load()
    plan = _Plan(Geometry(n, (0, 0, 0), ext), _abi.GBP_NODAL, bclo, bchi,
                 make_options(0, precision="mixed", mg_rtol=1e-12, mg_atol=0.0))
    vh = torch.from_numpy(np.ascontiguousarray(vel)).pin_memory()
    rh = torch.from_numpy(np.ascontiguousarray(rho)).pin_memory()
    gh = torch.from_numpy(np.ascontiguousarray(gp)).pin_memory()
    ph = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64).pin_memory()
    sth = _abi.Stats()
    _abi.check(lib.gbp_apply_nodal_projection_host(plan.ptr, vh.data_ptr(), rh.data_ptr(), 1.0, gh.data_ptr(),
                                                   ph.data_ptr(), 1.0, 0, ctypes.byref(sth)), "host entry")
    un = vh.numpy()
    want = vel_or[:, 1:-1, 1:-1, 1:-1]
    assert np.abs(un - want).max() <= 1e-9 * np.abs(want).max()
