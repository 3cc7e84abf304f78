"""The oracle's inflow/outflow solvability restatement (CPU): zero net flux afterwards, only the
outflow velocities change, and nothing changes without outflow."""
import numpy as np

import oracle as O


def net_flux_cell(g, v, dd_lo, dd_hi):
    tot = 0.0
    for d in range(3):
        area = g.h[(d + 1) % 3] * g.h[(d + 2) % 3]
        for side, on in ((0, dd_lo[d]), (1, dd_hi[d])):
            if on:
                sl = [slice(1, -1)] * 3
                sl[2 - d] = -1 if side else 0
                f = v[(d,) + tuple(sl)].sum() * area
                tot += -f if side else f
    return tot


def test_cell_form_balances_flux_and_scales_outflow_only():
    g = O.Grid((8, 6, 5), hi=(1.0, 0.75, 0.5), bclo=(2, 2, 2))
    rng = np.random.default_rng(0)
    vel = rng.standard_normal((3, 7, 8, 10))
    dd_lo, dd_hi = (1, 0, 1), (1, 1, 0)
    v2, inflow, outflow = O.enforce_inout_solvability(g, vel, dd_lo, dd_hi)
    assert inflow > 0 and outflow > 0
    assert abs(net_flux_cell(g, vel, dd_lo, dd_hi) - (inflow - outflow)) < 1e-12
    assert abs(net_flux_cell(g, v2, dd_lo, dd_hi)) < 1e-12
    changed = v2 != vel
    # the low-x face: only cells with u < 0 (outflow there) may change
    lo_x = (0, slice(1, -1), slice(1, -1), 0)
    assert np.all(vel[lo_x][changed[lo_x]] < 0)
    # interior untouched
    assert np.array_equal(v2[:, 1:-1, 1:-1, 1:-1], vel[:, 1:-1, 1:-1, 1:-1])


def test_no_outflow_leaves_velocity_unchanged():
    g = O.Grid((4, 4, 4), bclo=(2, 2, 2))
    vel = np.zeros((3, 6, 6, 6))
    vel[0, 1:-1, 1:-1, 0] = 1.0  # inflow through low x only
    v2, inflow, outflow = O.enforce_inout_solvability(g, vel, (1, 0, 0), (1, 0, 0))
    assert outflow == 0.0 and inflow > 0
    assert np.array_equal(v2, vel)


def test_face_form_balances_flux():
    g = O.Grid((6, 5, 4), bclo=(2, 2, 2))
    rng = np.random.default_rng(1)
    umac = [rng.standard_normal(g.face_shape(d)) for d in range(3)]
    u2, inflow, outflow = O.mac_enforce_inout_solvability(g, umac, (1, 1, 0), (1, 0, 1))
    net = 0.0
    for d, lo, hi in ((0, 1, 1), (1, 1, 0), (2, 0, 1)):
        area = g.h[(d + 1) % 3] * g.h[(d + 2) % 3]
        for side, on in ((0, lo), (1, hi)):
            if on:
                sl = [slice(None)] * 3
                sl[2 - d] = -1 if side else 0
                f = u2[d][tuple(sl)].sum() * area
                net += -f if side else f
    assert abs(net) < 1e-12
