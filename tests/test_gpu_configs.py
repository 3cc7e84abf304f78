"""Parity on the benchmark configurations themselves, at their own sizes, against the FP64 oracle.

  cfg1  64^3 Taylor-Green + U(-1e-2, 1e-2) noise on [0, 2pi]^3, triply periodic, rho = 1: the nodal
        projection of the cell velocity and the MAC projection of its face average, plain FP64 and
        the mixed form, to incflo's MLMG tolerances (rtol 1e-11, atol 1e-14).
  cfg2  256^3 variable density (rho 1 -> 3 tanh interface, k^-2 random velocity), periodic x / y,
        walls in z: the nodal projection (sigma = 1 / rho) and the MAC projection (beta = 1 / rho on
        faces, arithmetic face average as average_cellcenter_to_face), both forms.

The bar: phi relative L2 <= 1e-9 against the oracle solved to 1e-13, corrected velocities within
1e-9 of their scale, post-projection max|div u| no worse than the oracle's (the nodal projection is
approximate: its leftover divergence is the discretisation's, equal for both to a relative 1e-6).
The mixed form is also run at the benchmark's tolerance (1e-10) and its phi error against the oracle
is bounded and printed (the figure quoted for each configuration).
"""
import numpy as np
import pytest
import torch

import oracle as O
from incflo_gb300 import Geometry, MacProjector, NodalProjector, make_options, synth
from tests.helpers import cuda, rel_l2, unique_nodes

pytestmark = pytest.mark.gpu

_CACHE = {}


def cell_to_faces(vel, per):
    """Face velocities from cell velocities: the arithmetic average of the two cells (wrapped in a
    periodic direction, so the duplicate face n equals face 0); wall faces carry 0."""
    out = []
    for d in range(3):
        u, ax = vel[d], 2 - d
        n = u.shape[ax]
        f = 0.5 * (np.take(u, np.arange(-1, n), axis=ax, mode="wrap") + np.take(u, np.arange(0, n + 1), axis=ax,
                                                                               mode="wrap"))
        if not per[d]:
            for end in (0, n):
                sl = [slice(None)] * 3
                sl[ax] = end
                f[tuple(sl)] = 0.0
        out.append(np.ascontiguousarray(f))
    return out


def rho_to_faces(rho, per):
    """Arithmetic face average of the cell density; boundary faces of walls take the adjacent cell."""
    out = []
    for d in range(3):
        ax = 2 - d
        lo = np.take(rho, np.arange(-1, rho.shape[ax]), axis=ax, mode="wrap")
        hi = np.take(rho, np.arange(0, rho.shape[ax] + 1), axis=ax, mode="wrap")
        f = 0.5 * (lo + hi)
        if not per[d]:
            first = [slice(None)] * 3
            first[ax] = 0
            last = [slice(None)] * 3
            last[ax] = -1
            f[tuple(first)] = np.take(rho, [0], axis=ax).squeeze(ax)
            f[tuple(last)] = np.take(rho, [rho.shape[ax] - 1], axis=ax).squeeze(ax)
        out.append(np.ascontiguousarray(f))
    return out


def _cfg(name):
    if name not in _CACHE:
        c = synth.taylor_green_noise(64) if name == "cfg1" else synth.variable_density_rt(256)
        _CACHE[name] = c
    return _CACHE[name]


def _nodal_oracle(name):
    key = (name, "nodal")
    if key not in _CACHE:
        c = _cfg(name)
        g = O.Grid(c["n"], c["lo"], c["hi"], c["bclo"], c["bchi"])
        vel = synth.with_ghosts(c["vel"])
        sigma = 1.0 / c["rho"]
        vel_or, phi_or, grad_or, st = O.nodal_project(g, sigma, vel, rtol=1e-13)
        assert st["status"] == 0
        _CACHE[key] = (g, vel, sigma, vel_or, phi_or, grad_or)
    return _CACHE[key]


def _nodal_gpu(name, precision, rtol, atol=0.0):
    g, vel, sigma, *_ = _nodal_oracle(name)
    c = _cfg(name)
    vt = cuda(vel)
    proj = NodalProjector(vt, cuda(sigma), Geometry(c["n"], c["lo"], c["hi"]),
                          options=make_options(0, precision=precision))
    proj.setDomainBC(c["bclo"], c["bchi"])
    st = proj.project(rtol=rtol, atol=atol)
    phi = unique_nodes(g, proj.getPhi().cpu().numpy())
    out = vt.cpu().numpy()
    del proj, vt
    torch.cuda.empty_cache()
    return st, phi, out


def _check_nodal(name, precision, rtol, atol):
    g, vel, sigma, vel_or, phi_or, grad_or = _nodal_oracle(name)
    st, phi, out = _nodal_gpu(name, precision, rtol, atol)
    assert st["status"] == 0 and st["final_rel_resid"] <= rtol
    err = rel_l2(phi, phi_or)
    print(f"\n{name} nodal {precision}: phi rel-L2 vs oracle {err:.3e}, {st['vcycles']} V-cycles")
    assert err <= 1e-9, (err, st)
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))
    np.testing.assert_allclose(out[inner], vel_or[inner], rtol=0, atol=1e-9 * np.abs(vel_or[inner]).max())
    div_gpu = np.abs(O.nodal_rhs(g, out)).max()
    div_or = np.abs(O.nodal_rhs(g, vel_or)).max()
    assert div_gpu <= div_or * (1 + 1e-6) + 1e-12


def _mac_case(name):
    key = (name, "mac")
    if key not in _CACHE:
        c = _cfg(name)
        per = [b == O.PERIODIC for b in c["bclo"]]
        g = O.Grid(c["n"], c["lo"], c["hi"], c["bclo"], c["bchi"])
        umac = cell_to_faces(c["vel"], per)
        beta = [1.0 / r for r in rho_to_faces(c["rho"], per)]
        un_or, phi_or, st = O.mac_project(g, beta, umac, rtol=1e-13)
        assert st["status"] == 0
        _CACHE[key] = (g, umac, beta, un_or, phi_or)
    return _CACHE[key]


def _check_mac(name, precision, rtol, atol):
    g, umac, beta, un_or, phi_or = _mac_case(name)
    c = _cfg(name)
    ut = [cuda(u) for u in umac]
    mp = MacProjector(Geometry(c["n"], c["lo"], c["hi"]), options=make_options(1, precision=precision))
    mp.initProjector(beta=[cuda(b) for b in beta])
    mp.setDomainBC(c["bclo"], c["bchi"])
    mp.setUMAC(ut)
    phi = cuda(np.zeros(g.cell_shape))
    st = mp.project(rtol=rtol, atol=atol, phi=phi, phi_guess=False)
    assert st["status"] == 0 and st["final_rel_resid"] <= rtol
    err = rel_l2(phi.cpu().numpy(), phi_or)
    print(f"\n{name} MAC {precision}: phi rel-L2 vs oracle {err:.3e}, {st['vcycles']} V-cycles")
    assert err <= 1e-9, (err, st)
    got = [u.cpu().numpy() for u in ut]
    for d in range(3):
        np.testing.assert_allclose(got[d], un_or[d], rtol=0, atol=1e-9 * np.abs(un_or[d]).max())
    # the MAC projection removes the discrete divergence to the solver tolerance
    div0 = np.abs(O.mac_rhs(g, *umac)).max()
    assert np.abs(O.mac_rhs(g, *got)).max() <= max(10 * rtol * div0, np.abs(O.mac_rhs(g, *un_or)).max() * 10)
    del mp, ut
    torch.cuda.empty_cache()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cfg1_taylor_green_nodal(gpu_lib, precision):
    _check_nodal("cfg1", precision, 1e-11, 1e-14)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cfg1_taylor_green_mac(gpu_lib, precision):
    _check_mac("cfg1", precision, 1e-11, 1e-14)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cfg2_variable_density_nodal_256(gpu_lib, precision):
    _check_nodal("cfg2", precision, 1e-12, 0.0)


def test_cfg2_mixed_error_at_benchmark_tolerance(gpu_lib):
    """The chosen form at the benchmark's stopping rule (1e-10 relative residual): the phi error it
    leaves against the FP64 oracle."""
    g, vel, sigma, vel_or, phi_or, grad_or = _nodal_oracle("cfg2")
    st, phi, out = _nodal_gpu("cfg2", "mixed", 1e-10)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-10
    err = rel_l2(phi, phi_or)
    print(f"\ncfg2 nodal mixed at rtol 1e-10: phi rel-L2 vs oracle {err:.3e}")
    assert err <= 1e-7


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cfg2_variable_density_mac_256(gpu_lib, precision):
    _check_mac("cfg2", precision, 1e-12, 0.0)


# ------------------------------------------------------------------------------------------ cfg4
# Channel [0, 4] x [0, 1]^2 with a z-aligned cylinder of radius 0.125 at (1, 0.5): inflow u = 1 at
# x = 0, outflow (p = 0) at x = 4, walls in y, periodic in z, rho = 1, u = 1 + U(-1e-3, 1e-3) noise.
# The direct cut-cell oracles finish in seconds at a quarter of the resolution (64 x 16 x 16, the same
# geometry); at the configuration's own 256 x 64 x 64 the GPU result is checked in the oracles' own
# operators: the nodal residual of the GPU phi and the velocity correction from it, and the cut-cell
# divergence of the MAC-projected face velocities.
def _cfg4_inputs(n, seed=4):
    from incflo_gb300 import eb

    ext = (4.0, 1.0, 1.0)
    rng = np.random.Generator(np.random.PCG64(seed))
    vel = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vel[:, 1:-1, 1:-1, 1:-1] = 1e-3 * rng.uniform(-1.0, 1.0, (3, n[2], n[1], n[0]))
    vel[0, 1:-1, 1:-1, 1:-1] += 1.0
    vel[0, :, :, 0] = 1.0  # inflow ghost cells
    M = eb.cylinder_moments(n, (0, 0, 0), ext, (1.0, 0.5, 0.0), 0.125, small_volfrac=1e-4)
    geo = eb.cylinder(n, (0, 0, 0), ext, (1.0, 0.5, 0.0), 0.125, small_volfrac=1e-4)
    shapes = [(n[2], n[1], n[0] + 1), (n[2], n[1] + 1, n[0]), (n[2] + 1, n[1], n[0])]
    umac = [1e-3 * rng.uniform(-1.0, 1.0, sh) for sh in shapes]
    umac[0] += 1.0
    umac[0][:, :, 0] = 1.0
    umac[1][:, 0, :] = 0.0
    umac[1][:, -1, :] = 0.0
    umac[2][-1] = umac[2][0]
    return ext, vel, M, geo, umac


def _cfg4_nodal_gpu(n, ext, vel, M, precision, rtol):
    from incflo_gb300 import apply_nodal_projection, eb

    vt = cuda(vel)
    rho = torch.ones((n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    gp = torch.zeros((3, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    pnd = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device="cuda")
    st = apply_nodal_projection(Geometry(n, (0, 0, 0), ext), (O.INFLOW, O.NEUMANN, O.PERIODIC),
                                (O.DIRICHLET, O.NEUMANN, O.PERIODIC), vt, rho, gp, pnd, set_inflow_bc=True,
                                options=make_options(0, precision=precision, mg_rtol=rtol, mg_atol=0.0),
                                eb_moments=cuda(eb.moments_components(M)))
    return st, vt.cpu().numpy(), pnd.cpu().numpy()


def _cfg4_mac_gpu(n, ext, geo, umac, precision, rtol):
    ut = [cuda(u) for u in umac]
    mp = MacProjector(Geometry(n, (0, 0, 0), ext), options=make_options(1, precision=precision))
    mp.initProjector(beta=1.0)
    mp.setDomainBC((O.INFLOW, O.NEUMANN, O.PERIODIC), (O.DIRICHLET, O.NEUMANN, O.PERIODIC))
    mp.setEB(cuda(geo["vfrac"]), [cuda(geo[k]) for k in ("apx", "apy", "apz")],
             [cuda(np.moveaxis(geo[k], -1, 0)) for k in ("fcx", "fcy", "fcz")])
    mp.setUMAC(ut)
    phi = cuda(np.zeros((n[2], n[1], n[0])))
    st = mp.project(rtol=rtol, atol=0.0, phi=phi, phi_guess=False)
    return st, [u.cpu().numpy() for u in ut], phi.cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cfg4_cylinder_channel_nodal_quarter(gpu_lib, precision):
    from oracle.eb_nodal import EBNodal

    n = (64, 16, 16)
    ext, vel, M, geo, umac = _cfg4_inputs(n)
    h = [ext[d] / n[d] for d in range(3)]
    o = EBNodal(n, h, (O.INFLOW, O.NEUMANN, O.PERIODIC), (O.DIRICHLET, O.NEUMANN, O.PERIODIC), M)
    u = np.ascontiguousarray(vel[:, 1:-1, 1:-1, 1:-1])
    ref = o.project(np.ones((n[2], n[1], n[0])), u, vel)
    st, vout, pnd = _cfg4_nodal_gpu(n, ext, vel, M, precision, 1e-12)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    fl = o.active.copy()
    got = o.to_unknowns(pnd)[fl]
    want = o.to_unknowns(ref["phi"])[fl]
    err = rel_l2(got, want)
    print(f"\ncfg4/4 nodal {precision}: phi rel-L2 vs oracle {err:.3e}, {st['vcycles']} V-cycles")
    assert err <= 1e-9
    fluid = M[..., 0, 0, 0] > 0
    for d in range(3):
        np.testing.assert_allclose(vout[d, 1:-1, 1:-1, 1:-1][fluid], ref["u"][d][fluid], rtol=0,
                                   atol=1e-9 * np.abs(ref["u"]).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cfg4_cylinder_channel_mac_quarter(gpu_lib, precision):
    from oracle.eb_mac import EBMac

    n = (64, 16, 16)
    ext, vel, M, geo, umac = _cfg4_inputs(n)
    h = [ext[d] / n[d] for d in range(3)]
    ap = [geo["apx"], geo["apy"], geo["apz"]]
    fc = [geo["fcx"], geo["fcy"], geo["fcz"]]
    m = EBMac(n, h, (O.INFLOW, O.NEUMANN, O.PERIODIC), (O.DIRICHLET, O.NEUMANN, O.PERIODIC), geo["vfrac"], ap, fc,
              [np.ones(a.shape) for a in ap])
    un_or, phi_or, _ = m.project(umac)
    st, got, phi = _cfg4_mac_gpu(n, ext, geo, umac, precision, 1e-12)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    err = rel_l2(phi, phi_or)
    print(f"\ncfg4/4 MAC {precision}: phi rel-L2 vs oracle {err:.3e}, {st['vcycles']} V-cycles")
    assert err <= 1e-9
    for d in range(3):
        open_ = m.ap[d] > 0
        np.testing.assert_allclose(got[d][open_], un_or[d][open_], rtol=0, atol=1e-9 * np.abs(un_or[d]).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cfg4_cylinder_channel_full_size(gpu_lib, precision):
    """256 x 64 x 64: the GPU's nodal phi solves the oracle's cut-cell system (its residual in the
    oracle's operator and norm), its corrected velocity is u - grad phi at the fluid centroids from the
    oracle's element gradients, and the MAC-projected face velocities are divergence free in the
    oracle's cut-cell divergence."""
    from oracle.eb_mac import EBMac
    from oracle.eb_nodal import EBNodal

    n = (256, 64, 64)
    ext, vel, M, geo, umac = _cfg4_inputs(n)
    h = [ext[d] / n[d] for d in range(3)]
    bclo, bchi = (O.INFLOW, O.NEUMANN, O.PERIODIC), (O.DIRICHLET, O.NEUMANN, O.PERIODIC)
    st, vout, pnd = _cfg4_nodal_gpu(n, ext, vel, M, precision, 1e-12)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    if "cfg4_nodal" not in _CACHE:
        _CACHE["cfg4_nodal"] = EBNodal(n, h, bclo, bchi, M)
    o = _CACHE["cfg4_nodal"]
    sig = np.ones((n[2], n[1], n[0]))
    u = np.ascontiguousarray(vel[:, 1:-1, 1:-1, 1:-1])
    r = o.residual_norm(sig, u, pnd, vel)
    print(f"\ncfg4 nodal {precision}: residual of the GPU phi in the oracle's operator {r:.3e}, "
          f"{st['vcycles']} V-cycles")
    assert r <= 1e-11
    phi_u = o.to_unknowns(pnd)
    g = np.einsum("cad,ca->dc", o.Gcu[o.inv], phi_u[o.ids])
    un = vout[:, 1:-1, 1:-1, 1:-1]
    scale = np.abs(u).max()
    for d in range(3):
        want = u[d, o.cell_k, o.cell_j, o.cell_i] - g[d]
        np.testing.assert_allclose(un[d, o.cell_k, o.cell_j, o.cell_i], want, rtol=0, atol=1e-12 * scale)
    st, got, phi = _cfg4_mac_gpu(n, ext, geo, umac, precision, 1e-12)
    assert st["status"] == 0 and st["final_rel_resid"] <= 1e-12
    if "cfg4_mac" not in _CACHE:
        ap = [geo["apx"], geo["apy"], geo["apz"]]
        fc = [geo["fcx"], geo["fcy"], geo["fcz"]]
        _CACHE["cfg4_mac"] = EBMac(n, h, bclo, bchi, geo["vfrac"], ap, fc, [np.ones(a.shape) for a in ap])
    m = _CACHE["cfg4_mac"]
    d0, d1 = m.divergence(umac), m.divergence(got)
    print(f"cfg4 MAC {precision}: cut-cell divergence {d0:.3e} -> {d1:.3e}, {st['vcycles']} V-cycles")
    assert d1 <= 1e-11 * d0
