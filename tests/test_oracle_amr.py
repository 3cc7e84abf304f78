"""The two-level composite nodal oracle (oracle/amr_nodal.py) pinned on the CPU: with no fine cells it
is the single-level oracle, with the whole domain refined it is the single-level oracle at the fine
resolution, and for a partial fine region its composite operator is symmetric, has the constants as its
null space (walls / periodic) and projects the velocity onto the composite discrete divergence-free
space."""
import numpy as np
import pytest

import oracle as O
from oracle.amr_nodal import CompositeNodal
from tests.helpers import D, N, P, rel_l2, unique_nodes

CASES = [((P, N, D), (P, N, N)), ((P, P, N), (P, P, N))]


def _fields(n, rng):
    nf = [2 * v for v in n]
    sig_c = rng.uniform(0.5, 2.0, (n[2], n[1], n[0]))
    sig_f = rng.uniform(0.5, 2.0, (nf[2], nf[1], nf[0]))
    u_c = rng.standard_normal((3, n[2], n[1], n[0]))
    u_f = rng.standard_normal((3, nf[2], nf[1], nf[0]))
    return sig_c, sig_f, u_c, u_f


@pytest.mark.parametrize("bcs", CASES, ids=["dirichlet", "singular"])
def test_reduces_to_single_level(bcs):
    n, ext = (8, 6, 4), (1.0, 0.75, 0.5)
    h = [ext[d] / n[d] for d in range(3)]
    rng = np.random.default_rng(0)
    sig_c, sig_f, u_c, u_f = _fields(n, rng)
    nf = [2 * v for v in n]
    g = O.Grid(n, hi=ext, bclo=bcs[0], bchi=bcs[1])
    vg = np.zeros((3, n[2] + 2, n[1] + 2, n[0] + 2))
    vg[:, 1:-1, 1:-1, 1:-1] = u_c
    vn, phi, _, _ = O.nodal_project(g, sig_c, vg, rtol=1e-14)
    r = CompositeNodal(n, h, bcs[0], bcs[1], np.zeros((nf[2], nf[1], nf[0]), bool)).project(sig_c, sig_f, u_c, u_f)
    assert rel_l2(unique_nodes(g, r["phi_c"]) - unique_nodes(g, r["phi_c"]).mean() * (g.bclo[2] != D),
                  phi - phi.mean() * (g.bclo[2] != D)) <= 1e-11 or rel_l2(unique_nodes(g, r["phi_c"]), phi) <= 1e-11
    np.testing.assert_allclose(r["u_c"], vn[:, 1:-1, 1:-1, 1:-1], rtol=0, atol=1e-11)
    gf = O.Grid(nf, hi=ext, bclo=bcs[0], bchi=bcs[1])
    vgf = np.zeros((3, nf[2] + 2, nf[1] + 2, nf[0] + 2))
    vgf[:, 1:-1, 1:-1, 1:-1] = u_f
    vnf, phif, _, _ = O.nodal_project(gf, sig_f, vgf, rtol=1e-14)
    r = CompositeNodal(n, h, bcs[0], bcs[1], np.ones((nf[2], nf[1], nf[0]), bool)).project(sig_c, sig_f, u_c, u_f)
    np.testing.assert_allclose(r["u_f"], vnf[:, 1:-1, 1:-1, 1:-1], rtol=0, atol=1e-11)


@pytest.mark.parametrize("bcs", CASES, ids=["dirichlet", "singular"])
def test_partial_region_symmetric(bcs):
    n, ext = (8, 6, 4), (1.0, 0.75, 0.5)
    h = [ext[d] / n[d] for d in range(3)]
    rng = np.random.default_rng(1)
    sig_c, sig_f, u_c, u_f = _fields(n, rng)
    nf = [2 * v for v in n]
    fm = np.zeros((nf[2], nf[1], nf[0]), bool)
    fm[:, 2:8, 4:12] = True
    cn = CompositeNodal(n, h, bcs[0], bcs[1], fm)
    r = cn.project(sig_c, sig_f, u_c, u_f)
    A = r["A"]
    assert abs(A - A.T).max() <= 1e-14 * abs(A).max()
    if cn.singular:
        assert np.abs(A @ np.ones(cn.ndof)).max() <= 1e-12 * abs(A).max()
    assert np.abs(A @ r["x"] - r["b"]).max() <= 1e-10 * np.abs(r["b"]).max()


def test_linear_potential_exact_across_the_interface():
    """sigma = 1 and a uniform velocity in a walled box: the composite solution is the linear potential
    (hanging nodes interpolate it exactly), so phi is linear on both levels and the projected velocity
    vanishes on every leaf cell."""
    n, ext = (8, 8, 4), (1.0, 1.0, 0.5)
    h = [ext[d] / n[d] for d in range(3)]
    nf = [2 * v for v in n]
    fm = np.zeros((nf[2], nf[1], nf[0]), bool)
    fm[2:6, 4:10, 2:12] = True
    fm[2:6, 10:14, 6:10] = True
    u = np.array([1.0, -2.0, 0.5])
    u_c = np.broadcast_to(u[:, None, None, None], (3, n[2], n[1], n[0])).copy()
    u_f = np.broadcast_to(u[:, None, None, None], (3, nf[2], nf[1], nf[0])).copy()
    cn = CompositeNodal(n, h, (N, N, N), (N, N, N), fm)
    r = cn.project(np.ones((n[2], n[1], n[0])), np.ones((nf[2], nf[1], nf[0])), u_c, u_f)
    zc, yc, xc = np.meshgrid(*[np.arange(n[d] + 1) * h[d] for d in (2, 1, 0)], indexing="ij")
    lin = u[0] * xc + u[1] * yc + u[2] * zc
    pc = r["phi_c"]
    np.testing.assert_allclose(pc - pc.mean(), lin - lin.mean(), rtol=0, atol=1e-11)
    np.testing.assert_allclose(r["u_c"], 0.0, atol=1e-11)
    np.testing.assert_allclose(r["u_f"][:, fm], 0.0, atol=1e-11)
    # the fine level's phi is the same linear function on the region's nodes
    hf = [v / 2 for v in h]
    zf, yf, xf = np.meshgrid(*[np.arange(nf[d] + 1) * hf[d] for d in (2, 1, 0)], indexing="ij")
    linf = u[0] * xf + u[1] * yf + u[2] * zf
    ok = ~np.isnan(r["phi_f"])
    shift = (pc - lin).mean()
    np.testing.assert_allclose(r["phi_f"][ok], linf[ok] + shift, rtol=0, atol=1e-11)


def test_tagging_boxes_cover_the_tags_and_follow_the_grid_rules():
    """synth.tag_and_box (incflo's regrid: blocking_factor, max_grid_size): disjoint boxes of whole blocks,
    at most max_grid fine cells per side, covering every tagged coarse cell and no untagged block."""
    import numpy as np

    from incflo_gb300 import synth

    rng = np.random.default_rng(2)
    tag = np.zeros((32, 32, 32), bool)
    tag[12:20] = True
    tag[rng.integers(0, 32, 40), rng.integers(0, 32, 40), rng.integers(0, 32, 40)] = True
    boxes = synth.tag_and_box(tag, blocking=8, max_grid=16)
    fine = np.zeros((64, 64, 64), int)
    for lo, hi in boxes:
        ext = [hi[d] - lo[d] + 1 for d in range(3)]
        assert all(e in (8, 16) for e in ext) and all(v % 8 == 0 for v in lo)
        fine[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] += 1
    assert fine.max() == 1
    covered = fine.reshape(32, 2, 32, 2, 32, 2).all(axis=(1, 3, 5))
    assert np.all(covered[tag])
    blocks_tagged = tag.reshape(8, 4, 8, 4, 8, 4).any(axis=(1, 3, 5))
    blocks_fine = covered.reshape(8, 4, 8, 4, 8, 4).all(axis=(1, 3, 5))
    assert np.array_equal(blocks_tagged, blocks_fine)
