"""incflo::ApplyCCProjection on the GPU (through the C ABI) against the oracle's restatement:
the same MOL face velocities, MAC solve and cell updates; phi-dependent outputs within 1e-9 of scale
(both solves converge to 1e-12 / 1e-13 relative), face divergence removed to solver tolerance."""
import numpy as np
import pytest
import torch

import oracle as O
from incflo_gb300 import Geometry, apply_cc_projection, make_options
from tests.helpers import D, I, N, P

pytestmark = pytest.mark.gpu

CASES = [
    # n, extent, bclo, bchi, constant density, incremental
    ((16, 16, 16), (1.0, 1.0, 1.0), (P, P, P), (P, P, P), True, False),
    ((16, 12, 10), (1.0, 0.75, 0.625), (P, N, N), (P, N, N), False, False),
    ((12, 10, 8), (1.5, 1.25, 1.0), (I, N, P), (D, N, P), False, False),
    ((16, 16, 8), (1.0, 1.0, 0.5), (P, P, N), (P, P, N), False, True),
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[2]}-{c[3]}-{'c' if c[4] else 'v'}{'-inc' if c[5] else ''}"
                                             for c in CASES])
def test_cc_projection_matches_oracle(gpu_lib, case):
    n, ext, bclo, bchi, const, incr = case
    g = O.Grid(n, hi=ext, bclo=bclo, bchi=bchi)
    rng = np.random.default_rng(5)
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vel[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((3,) + g.cell_shape)
    for d in range(3):
        for side, bc in ((0, bclo[d]), (1, bchi[d])):
            if bc == I:
                sl = [slice(1, -1)] * 3
                sl[2 - d] = -1 if side else 0
                vel[(d,) + tuple(sl)] = rng.uniform(0.5, 1.5, vel[(d,) + tuple(sl)].shape) * (-1 if side else 1)
    rho = rng.uniform(1.0, 3.0, (n[2] + 2, n[1] + 2, n[0] + 2))
    gp = rng.standard_normal((3,) + g.cell_shape) * 0.1
    p_cc = rng.standard_normal(g.cell_shape) * 0.1
    vel_old = rng.standard_normal((3,) + g.cell_shape) if incr else None
    s, rho0 = 0.5, 2.0
    ref = O.cc_projection(g, vel, rho, gp, p_cc, vel_old=vel_old, rho0=rho0, constant_density=const,
                          scaling_factor=s, incremental=incr, use_inflow=True, rtol=1e-13)
    rv, rgp, rp, ru, rphi, rst = ref
    assert rst["status"] == 0
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    vt, gpt, pt, rt = t(vel), t(gp), t(p_cc), t(rho)
    umac = [torch.zeros(g.face_shape(d), dtype=torch.float64, device="cuda") for d in range(3)]
    st = apply_cc_projection(Geometry(n, (0, 0, 0), ext), bclo, bchi, vt, rt, gpt, pt, umac,
                             scaling_factor=s, incremental=incr, set_inflow_bc=True,
                             vel_old=t(vel_old) if incr else None, rho0=rho0, constant_density=const,
                             options=make_options(1, mg_rtol=1e-12, mg_atol=0.0))
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    for got, want in ((vt.cpu().numpy()[:, 1:-1, 1:-1, 1:-1], rv[:, 1:-1, 1:-1, 1:-1]),
                      (gpt.cpu().numpy(), rgp), (pt.cpu().numpy(), rp)):
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-9 * max(np.abs(want).max(), 1e-30))
    for d in range(3):
        np.testing.assert_allclose(umac[d].cpu().numpy(), ru[d], rtol=0, atol=1e-9 * np.abs(ru[d]).max())
    div = O.mac_rhs(g, *[u.cpu().numpy() for u in umac])
    assert np.abs(div).max() <= 1e-9 * np.abs(O.mac_rhs(g, *O.mol_extrap_to_faces(g, vel))).max() + 1e-12
