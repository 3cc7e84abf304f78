"""Tensor (velocity) diffusion on the GPU against the oracle (oracle/tensor.py, a direct sparse solve of
the same discretisation): a channel between no-slip walls (one moving), inflow / outflow with a slip
wall, and a box of no-slip walls with random face values (edges and corners); velocity relative L2
<= 1e-9 in the FP64 and FP32-in-FP64 forms; div tau (compute_divtau) to 1e-12; diffuse_velocity and
the incflo boundary-type table."""
import numpy as np
import pytest
import torch

from incflo_gb300 import Geometry, make_options
from incflo_gb300.diffusion import TensorOp, compute_divtau, diffuse_tensor_bc, diffuse_velocity
from oracle import abec
from oracle import tensor as T
from tests.helpers import cuda, rel_l2

pytestmark = pytest.mark.gpu

CASES = {
    "channel": ((12, 10, 6), (1.2, 1.0, 0.6),
                ("periodic", "no_slip_wall", "periodic"), ("periodic", "no_slip_wall", "periodic")),
    "inflow-outflow-slip": ((12, 8, 6), (1.5, 1.0, 0.75),
                            ("mass_inflow", "slip_wall", "periodic"), ("pressure_outflow", "no_slip_wall", "periodic")),
    "box": ((8, 8, 8), (1.0, 1.0, 1.0),
            ("no_slip_wall", "no_slip_wall", "no_slip_wall"), ("no_slip_wall", "no_slip_wall", "no_slip_wall")),
}


def _case(name, seed=5):
    n, ext, tlo, thi = CASES[name]
    h = [ext[d] / n[d] for d in range(3)]
    bclo, bchi = diffuse_tensor_bc(tlo, thi)
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    eta_cc = rng.uniform(0.01, 0.05, (n[2], n[1], n[0]))
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vel[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((3, n[2], n[1], n[0]))
    for d in range(3):
        for side, bcs in ((0, bclo), (1, bchi)):
            for c in range(3):
                if bcs[c][d] != T.DIRICHLET:
                    continue
                sl = [c, slice(1, -1), slice(1, -1), slice(1, -1)]
                sl[3 - d] = -1 if side else 0
                vel[tuple(sl)] = rng.uniform(-1.0, 1.0, vel[tuple(sl)].shape)
    return n, ext, h, bclo, bchi, rho, eta_cc, vel


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(CASES))
def test_tensor_solve_matches_oracle(gpu_lib, name, precision):
    n, ext, h, bclo, bchi, rho, eta_cc, vel = _case(name)
    dt = 0.5
    per = [bclo[0][d] == T.PERIODIC for d in range(3)]
    eta = abec.eta_to_faces(eta_cc, per)
    rhs = rho[None] * vel[:, 1:-1, 1:-1, 1:-1]
    ref = T.solve(h, bclo, bchi, 1.0, rho, dt, eta, rhs, vel)
    op = TensorOp(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision=precision))
    op.setDomainBC(bclo, bchi)
    op.setScalars(1.0, dt)
    op.setACoeffs(0, cuda(rho))
    op.setShearViscosity(0, cuda(eta_cc))
    vt = cuda(vel)
    st = op.solve(vt, cuda(np.ascontiguousarray(rhs)), rtol=1e-12, atol=0.0)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    got = vt.cpu().numpy()
    assert rel_l2(got[:, 1:-1, 1:-1, 1:-1], ref) <= 1e-9
    # ghost cells (the boundary values) are left as given
    mask = np.ones(vel.shape, bool)
    mask[:, 1:-1, 1:-1, 1:-1] = False
    assert np.array_equal(got[mask], vel[mask])


@pytest.mark.parametrize("name", list(CASES))
def test_divtau_matches_oracle(gpu_lib, name):
    n, ext, h, bclo, bchi, rho, eta_cc, vel = _case(name, seed=6)
    per = [bclo[0][d] == T.PERIODIC for d in range(3)]
    eta = abec.eta_to_faces(eta_cc, per)
    want = T.divtau(T.fill_ghosts(vel, bclo, bchi), h, eta)
    got = compute_divtau(Geometry(n, (0, 0, 0), ext), bclo, bchi, cuda(vel), cuda(rho), cuda(eta_cc)).cpu().numpy()
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    got2 = compute_divtau(Geometry(n, (0, 0, 0), ext), bclo, bchi, cuda(vel), cuda(rho), cuda(eta_cc),
                          advect_momentum=False).cpu().numpy()
    np.testing.assert_allclose(got2, want / rho[None], rtol=1e-12, atol=1e-14)


def test_diffuse_velocity_and_face_viscosity(gpu_lib):
    n, ext, h, bclo, bchi, rho, eta_cc, vel = _case("inflow-outflow-slip", seed=7)
    dt = 0.25
    per = [bclo[0][d] == T.PERIODIC for d in range(3)]
    eta = abec.eta_to_faces(eta_cc, per)
    ref = T.solve(h, bclo, bchi, 1.0, rho, dt, eta, rho[None] * vel[:, 1:-1, 1:-1, 1:-1], vel)
    vt = cuda(vel)
    st = diffuse_velocity(Geometry(n, (0, 0, 0), ext), bclo, bchi, vt, cuda(rho), cuda(eta_cc), dt,
                          options=make_options(1, precision="mixed", mg_rtol=1e-12, mg_atol=0.0))
    assert st["status"] == 0
    assert rel_l2(vt.cpu().numpy()[:, 1:-1, 1:-1, 1:-1], ref) <= 1e-9
    # the same viscosity given on the faces
    op = TensorOp(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision="fp64"))
    op.setDomainBC(bclo, bchi)
    op.setScalars(1.0, dt)
    op.setACoeffs(0, cuda(rho))
    op.setShearViscosity(0, [cuda(np.ascontiguousarray(e)) for e in eta])
    vt2 = cuda(vel)
    op.solve(vt2, cuda(np.ascontiguousarray(rho[None] * vel[:, 1:-1, 1:-1, 1:-1])), rtol=1e-12, atol=0.0)
    assert rel_l2(vt2.cpu().numpy()[:, 1:-1, 1:-1, 1:-1], ref) <= 1e-9
