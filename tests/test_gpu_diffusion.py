"""Cell-centred ABecLaplacian solve (implicit scalar diffusion) on the GPU against the oracle
(oracle/abec.py, direct sparse solve): conservative and non-conservative tracers, inhomogeneous
Dirichlet values from the ghost cells, Neumann and periodic sides, the Poisson limit alpha = 0;
phi relative L2 <= 1e-9, FP64 and FP32-in-FP64 forms; and diffuse_scalar over two components."""
import numpy as np
import pytest
import torch

from incflo_gb300 import Geometry, make_options
from incflo_gb300.diffusion import ABecLaplacian, diffuse_scalar
from oracle import abec
from tests.helpers import D, N, P, cuda, rel_l2

pytestmark = pytest.mark.gpu

CASES = {
    "conservative-dirichlet": ((16, 12, 8), (1.0, 0.75, 0.5), (D, P, N), (N, P, D), 1.0, True),
    "periodic": ((16, 16, 8), (1.0, 1.0, 0.5), (P, P, P), (P, P, P), 1.0, False),
    "poisson-dirichlet": ((16, 8, 8), (1.0, 0.5, 0.5), (D, N, N), (D, N, N), 0.0, False),
}


def _case(name, seed=9):
    n, ext, bclo, bchi, alpha, cons = CASES[name]
    h = [ext[d] / n[d] for d in range(3)]
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    eta = rng.uniform(0.01, 0.05, (n[2], n[1], n[0]))
    phi = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2))
    phi[1:-1, 1:-1, 1:-1] = rng.standard_normal((n[2], n[1], n[0]))
    for d in range(3):
        for side, bc in ((0, bclo[d]), (1, bchi[d])):
            if bc == D:
                sl = [slice(1, -1)] * 3
                sl[2 - d] = -1 if side else 0
                phi[tuple(sl)] = rng.uniform(0.5, 1.5, phi[tuple(sl)].shape)
    return n, ext, h, bclo, bchi, alpha, cons, rho, eta, phi


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(CASES))
def test_abec_solve_matches_oracle(gpu_lib, name, precision):
    n, ext, h, bclo, bchi, alpha, cons, rho, eta, phi = _case(name)
    dt = 0.05
    a = rho if cons else 1.0
    rhs = (rho if cons else 1.0) * phi[1:-1, 1:-1, 1:-1]
    per = [bclo[d] == P for d in range(3)]
    b = abec.eta_to_faces(eta, per)
    ref = abec.solve(n, h, bclo, bchi, alpha, a, dt, b, rhs, phi)
    op = ABecLaplacian(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision=precision))
    op.setDomainBC(bclo, bchi)
    op.setScalars(alpha, dt)
    op.setACoeffs(0, cuda(rho) if cons else 1.0)
    op.setBCoeffsFromEta(0, cuda(eta))
    pt = cuda(phi)
    st = op.solve(pt, cuda(np.ascontiguousarray(rhs)), rtol=1e-12, atol=0.0)
    assert st["status"] == 0
    got = pt.cpu().numpy()
    assert rel_l2(got[1:-1, 1:-1, 1:-1], ref) <= 1e-9
    # the boundary values in the ghost cells are left as given
    assert np.array_equal(got[:, :, 0], phi[:, :, 0])


def test_abec_face_coefficients_given(gpu_lib):
    """setBCoeffs with face arrays (instead of eta) gives the same solve."""
    n, ext, h, bclo, bchi, alpha, cons, rho, eta, phi = _case("conservative-dirichlet")
    b = abec.eta_to_faces(eta, [bclo[d] == P for d in range(3)])
    ref = abec.solve(n, h, bclo, bchi, 1.0, rho, 0.05, b, rho * phi[1:-1, 1:-1, 1:-1], phi)
    op = ABecLaplacian(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision="fp64"))
    op.setDomainBC(bclo, bchi)
    op.setScalars(1.0, 0.05)
    op.setACoeffs(0, cuda(rho))
    op.setBCoeffs(0, [cuda(x) for x in b])
    pt = cuda(phi)
    op.solve(pt, cuda(np.ascontiguousarray(rho * phi[1:-1, 1:-1, 1:-1])), rtol=1e-12, atol=0.0)
    assert rel_l2(pt.cpu().numpy()[1:-1, 1:-1, 1:-1], ref) <= 1e-9


def test_diffuse_scalar_two_components(gpu_lib):
    n, ext, h, bclo, bchi, alpha, cons, rho, eta, phi = _case("conservative-dirichlet")
    rng = np.random.default_rng(2)
    tr = np.stack([phi, phi + 0.1 * rng.standard_normal(phi.shape)])
    etas = np.stack([eta, 2.0 * eta])
    dt = 0.02
    refs = []
    for c, cons_c in enumerate((1, 0)):
        b = abec.eta_to_faces(etas[c], [bclo[d] == P for d in range(3)])
        a = rho if cons_c else 1.0
        refs.append(abec.solve(n, h, bclo, bchi, 1.0, a, dt, b, a * tr[c][1:-1, 1:-1, 1:-1], tr[c]))
    tt = cuda(tr)
    opts = make_options(1, precision="mixed", mg_rtol=1e-12, mg_atol=0.0)
    stats = diffuse_scalar(Geometry(n, (0, 0, 0), ext), bclo, bchi, tt, cuda(rho), cuda(etas), dt, (1, 0),
                           options=opts)
    assert all(s["status"] == 0 for s in stats)
    got = tt.cpu().numpy()
    for c in range(2):
        assert rel_l2(got[c][1:-1, 1:-1, 1:-1], refs[c]) <= 1e-9
