"""Cut-cell geometry of an embedded boundary from an implicit surface (the role of AMReX's EB2::Build
for incflo's cylinder, src/embedded_boundaries/eb_cylinder.cpp:15-64, which is not available here).

For a cylinder along one axis the fluid is outside the circle (EB2::CylinderIF with fluid outside):
  - a face normal to a direction in the circle's plane is a rectangle crossed by the cylinder along
    a chord; its aperture is the fraction of the face outside [c - s, c + s], s = sqrt(r^2 - d^2);
  - a face normal to the axis, and a cell's volume fraction, are the fraction of a rectangle outside
    the circle. The covered part is integrated exactly: between the break points (the circle's extreme
    points and where it crosses the rectangle's sides) its height is a + b s(u), u = x - cx, and the
    integrals of 1, u, s, u s and s^2 have closed forms.
Arrays follow incflo_gb300.projection: cells (nz, ny, nx), x faces (nz, ny, nx+1), ... (last axis x).
Face centroids follow AMReX's fcx / fcy / fcz: the offset of the open part's centroid from the face
centre in units of the cell size, in [-0.5, 0.5], for the two tangential directions in increasing
order (x faces: (y, z); y faces: (x, z); z faces: (x, y)); last axis of size 2.
"""
from __future__ import annotations

import math

import numpy as np


def _outside_fraction_1d(a, b, c, s):
    """Fraction of the interval [a, b] outside [c - s, c + s] (s <= 0: no overlap)."""
    lo = np.maximum(a, c - np.maximum(s, 0.0))
    hi = np.minimum(b, c + np.maximum(s, 0.0))
    covered = np.clip(hi - lo, 0.0, None)
    covered = np.where(s > 0.0, covered, 0.0)
    return 1.0 - covered / (b - a)


def _outside_moment_1d(a, b, c, s):
    """First moment of the part of [a, b] outside [c - s, c + s] (s <= 0: no overlap)."""
    lo = np.maximum(a, c - np.maximum(s, 0.0))
    hi = np.minimum(b, c + np.maximum(s, 0.0))
    cov = np.where((s > 0.0) & (hi > lo), 0.5 * (hi * hi - lo * lo), 0.0)
    return 0.5 * (b * b - a * a) - cov


def _snap(u, r):
    """u within rounding of +-r is +-r: the closed forms below (asin near +-1) would otherwise turn the
    last bit of a grid line that touches the circle's extreme point into an area error of ~1e-10."""
    return math.copysign(r, u) if abs(abs(u) - r) <= 1e-12 * r else u


def _rect_disk(x0, x1, y0, y1, cx, cy, r):
    """Area and first moments (int x, int y) of the rectangle's part inside the circle, exactly."""
    ua, ub = max(_snap(x0 - cx, r), -r), min(_snap(x1 - cx, r), r)
    if ub <= ua:
        return 0.0, 0.0, 0.0
    r2 = r * r

    def s(u):
        return math.sqrt(max(r2 - u * u, 0.0))

    def i_s(u):  # int s du
        return 0.5 * (u * s(u) + r2 * math.asin(max(-1.0, min(1.0, u / r))))

    def i_s2(u):  # int s^2 du
        return r2 * u - u ** 3 / 3.0

    def i_us(u):  # int u s du
        return -s(u) ** 3 / 3.0

    cuts = [ua, ub]
    for yb in (y0, y1):
        d = yb - cy
        if abs(d) < r:
            w = _snap(math.sqrt(r2 - d * d), r)
            cuts += [w, -w]
    cuts = sorted(c for c in cuts if ua <= c <= ub)
    area = mx = my = 0.0
    for a, b in zip(cuts[:-1], cuts[1:]):
        if b <= a:
            continue
        sm = s(0.5 * (a + b))
        if min(y1, cy + sm) <= max(y0, cy - sm):
            continue
        # upper bound y1 or the circle (cy + s), lower bound y0 or the circle (cy - s)
        h0, h1 = (cy, 1.0) if cy + sm < y1 else (y1, 0.0)
        l0, l1 = (cy, -1.0) if cy - sm > y0 else (y0, 0.0)
        du = b - a
        ds = i_s(b) - i_s(a)
        area_p = (h0 - l0) * du + (h1 - l1) * ds
        area += area_p
        mx += cx * area_p + (h0 - l0) * 0.5 * (b * b - a * a) + (h1 - l1) * (i_us(b) - i_us(a))
        my += 0.5 * ((h0 * h0 - l0 * l0) * du + 2.0 * (h0 * h1 - l0 * l1) * ds
                     + (h1 * h1 - l1 * l1) * (i_s2(b) - i_s2(a)))
    return area, mx, my


def _outside_rect(x0, x1, y0, y1, cx, cy, r):
    """Fraction of the rectangle outside the circle and the centroid (x, y) of that part."""
    full = (x1 - x0) * (y1 - y0)
    ca, cmx, cmy = _rect_disk(x0, x1, y0, y1, cx, cy, r)
    area = full - ca
    if area <= 1e-15 * full:
        return 0.0, 0.5 * (x0 + x1), 0.5 * (y0 + y1)
    mx = 0.5 * (x1 * x1 - x0 * x0) * (y1 - y0) - cmx
    my = 0.5 * (y1 * y1 - y0 * y0) * (x1 - x0) - cmy
    return min(1.0, area / full), mx / area, my / area


def cylinder(n, lo, hi, center, radius, axis=2, small_volfrac=0.0):
    """Volume fractions, face apertures and face centroids of the region outside a cylinder along
    `axis`. Returns dict(vfrac, apx, apy, apz, fcx, fcy, fcz) as float64 arrays. Cells whose volume
    fraction is below `small_volfrac` are made covered, with their faces closed (EB2's small-cell
    removal, the eb2.small_volfrac input; incflo's cylinder benchmarks use 1e-4)."""
    n = tuple(int(v) for v in n)
    h = [(hi[d] - lo[d]) / n[d] for d in range(3)]
    edges = [lo[d] + h[d] * np.arange(n[d] + 1) for d in range(3)]
    p, q = [d for d in range(3) if d != axis]  # the circle's plane, p < q
    cp, cq = center[p], center[q]
    shape_cells = (n[2], n[1], n[0])

    def grid(d, faces):
        """coordinates along d broadcast to the (z, y, x) array of cells or d-faces"""
        e = edges[d]
        v = e if faces else 0.5 * (e[:-1] + e[1:])
        sh = [1, 1, 1]
        sh[2 - d] = v.size
        return v.reshape(sh)

    def lohi(d):
        e = edges[d]
        sh = [1, 1, 1]
        sh[2 - d] = n[d]
        return e[:-1].reshape(sh), e[1:].reshape(sh)

    # cells (and axis-normal faces): rectangles of the (p, q) cross-section, indexed [q, p]
    frac = np.ones((n[q], n[p]))
    offp = np.zeros((n[q], n[p]))
    offq = np.zeros((n[q], n[p]))
    ep, eq = edges[p], edges[q]
    for b in range(n[q]):
        if abs(0.5 * (eq[b] + eq[b + 1]) - cq) > radius + h[q]:
            continue
        for a in range(n[p]):
            if abs(0.5 * (ep[a] + ep[a + 1]) - cp) > radius + h[p]:
                continue
            f, xc, yc = _outside_rect(ep[a], ep[a + 1], eq[b], eq[b + 1], cp, cq, radius)
            frac[b, a] = f
            if 0.0 < f < 1.0:
                offp[b, a] = (xc - 0.5 * (ep[a] + ep[a + 1])) / h[p]
                offq[b, a] = (yc - 0.5 * (eq[b] + eq[b + 1])) / h[q]

    def to_cells(a2, extra_axis=None):
        """[q, p] cross-section -> (z, y, x) array (the axis direction extended by one if asked);
        array axes run z, y, x, so q (the larger direction) comes first as in a2"""
        sh = [1, 1, 1]
        sh[2 - q] = n[q]
        sh[2 - p] = n[p]
        fs = list(shape_cells)
        if extra_axis is not None:
            fs[2 - extra_axis] += 1
        return np.broadcast_to(a2.reshape(sh), tuple(fs)).copy()

    vfrac = to_cells(frac)
    ap = [None, None, None]
    fc = [None, None, None]
    ap[axis] = to_cells(frac, axis)
    off = {p: to_cells(offp, axis), q: to_cells(offq, axis)}
    fc[axis] = np.stack([off[t] for t in range(3) if t != axis], axis=-1)
    # faces normal to p (and q): chord at the face position, fraction of the other extent
    for d, o in ((p, q), (q, p)):
        xd = grid(d, True)
        cd = center[d]
        # a face line within rounding of the circle's extreme point is tangent to it (no chord)
        inside = (xd - cd) ** 2 < radius * radius * (1.0 - 2e-12)
        s = np.where(inside, np.sqrt(np.clip(radius ** 2 - (xd - cd) ** 2, 0, None)), -1.0)
        o0, o1 = lohi(o)
        f = _outside_fraction_1d(o0, o1, center[o], s)
        length = (o1 - o0) * f
        mom = _outside_moment_1d(o0, o1, center[o], s)
        cen = np.where(length > 0.0, mom / np.where(length > 0.0, length, 1.0), 0.5 * (o0 + o1))
        fs = list(shape_cells)
        fs[2 - d] += 1
        ap[d] = np.broadcast_to(f, tuple(fs)).copy()
        cut = (ap[d] > 0.0) & (ap[d] < 1.0)
        offo = np.where(cut, np.broadcast_to((cen - 0.5 * (o0 + o1)) / h[o], tuple(fs)), 0.0)
        comps = [offo if t == o else np.zeros(tuple(fs)) for t in range(3) if t != d]
        fc[d] = np.stack(comps, axis=-1)
    if small_volfrac > 0.0:
        small = (vfrac > 0.0) & (vfrac < small_volfrac)
        if small.any():
            vfrac[small] = 0.0
            for d in range(3):
                ax = 2 - d
                pad = [(0, 0)] * 3
                pad[ax] = (0, 1)
                lo_side = np.pad(small, pad)
                pad[ax] = (1, 0)
                hi_side = np.pad(small, pad)
                shut = lo_side | hi_side
                ap[d][shut] = 0.0
                fc[d][shut] = 0.0
    return dict(vfrac=vfrac, apx=ap[0], apy=ap[1], apz=ap[2], fcx=fc[0], fcy=fc[1], fcz=fc[2])


_GL16_X, _GL16_W = np.polynomial.legendre.leggauss(16)


def _outside_moments_2d(x0, x1, y0, y1, cx, cy, r, pmax=2):
    """Moments int xi^p eta^q (p, q <= pmax) of the part of the rectangle outside the circle, over the
    rectangle's normalised coordinates xi = (x - xm) / (x1 - x0), eta likewise, in [-1/2, 1/2]. The covered
    part is integrated piecewise between the break points in the angle theta (u = x - cx = r sin theta),
    where the integrand is smooth, by 16-point Gauss-Legendre."""
    hx, hy = x1 - x0, y1 - y0
    xm, ym = 0.5 * (x0 + x1), 0.5 * (y0 + y1)
    full = np.zeros((pmax + 1, pmax + 1))
    for p in range(pmax + 1):
        for q in range(pmax + 1):
            ix = (0.5 ** (p + 1) - (-0.5) ** (p + 1)) / (p + 1)
            iy = (0.5 ** (q + 1) - (-0.5) ** (q + 1)) / (q + 1)
            full[p, q] = ix * iy
    ua, ub = max(_snap(x0 - cx, r), -r), min(_snap(x1 - cx, r), r)
    cov = np.zeros_like(full)
    if ub > ua:
        cuts = [ua, ub]
        for yb in (y0, y1):
            d = yb - cy
            if abs(d) < r:
                w = math.sqrt(r * r - d * d)
                cuts += [w, -w]
        cuts = sorted(c for c in cuts if ua <= c <= ub)
        for a, b in zip(cuts[:-1], cuts[1:]):
            if b <= a:
                continue
            ta, tb = math.asin(max(-1.0, min(1.0, a / r))), math.asin(max(-1.0, min(1.0, b / r)))
            tm, th = 0.5 * (ta + tb), 0.5 * (tb - ta)
            for t, w in zip(_GL16_X, _GL16_W):
                theta = tm + th * t
                u = r * math.sin(theta)
                s = r * math.cos(theta)
                jac = r * math.cos(theta) * th * w  # du = r cos(theta) dtheta
                lo, hi = max(y0, cy - s), min(y1, cy + s)
                if hi <= lo:
                    continue
                xi = (cx + u - xm) / hx
                elo, ehi = (lo - ym) / hy, (hi - ym) / hy
                for p in range(pmax + 1):
                    for q in range(pmax + 1):
                        cov[p, q] += jac / hx * xi ** p * (ehi ** (q + 1) - elo ** (q + 1)) / (q + 1)
    return full - cov


def cylinder_moments(n, lo, hi, center, radius, axis=2, small_volfrac=0.0):
    """Second moments of the fluid part of every cell for the cylinder of `cylinder`: an array
    (nz, ny, nx, 3, 3, 3) of int xi^p eta^q zeta^r dV / V over the fluid part, in the cell's
    normalised coordinates (xi, eta, zeta) in [-1/2, 1/2]^3 along (x, y, z), p, q, r <= 2. A regular
    cell has M[0,0,0] = 1, M[2,.,.] etc. = 1/12 products; a covered cell all zeros. The fluid part of a
    cell is a prism along the axis, so the axial factor is exact (1, 0, 1/12). Cells whose volume
    fraction is below `small_volfrac` are made covered (as in `cylinder`)."""
    n = tuple(int(v) for v in n)
    h = [(hi[d] - lo[d]) / n[d] for d in range(3)]
    edges = [lo[d] + h[d] * np.arange(n[d] + 1) for d in range(3)]
    p_, q_ = [d for d in range(3) if d != axis]
    za = np.array([1.0, 0.0, 1.0 / 12.0])
    M = np.zeros((n[2], n[1], n[0], 3, 3, 3))
    m2 = np.zeros((n[q_], n[p_], 3, 3))
    full2 = None
    for b in range(n[q_]):
        for a in range(n[p_]):
            x0, x1 = edges[p_][a], edges[p_][a + 1]
            y0, y1 = edges[q_][b], edges[q_][b + 1]
            if (abs(0.5 * (x0 + x1) - center[p_]) > radius + h[p_] or
                    abs(0.5 * (y0 + y1) - center[q_]) > radius + h[q_]):
                if full2 is None:
                    full2 = _outside_moments_2d(0.0, 1.0, 0.0, 1.0, 10.0, 10.0, 1e-3)
                m2[b, a] = full2
            else:
                mm = _outside_moments_2d(x0, x1, y0, y1, center[p_], center[q_], radius)
                if mm[0, 0] <= 1e-14 or mm[0, 0] < small_volfrac:  # covered (rounding, or a small cell)
                    mm[:] = 0.0
                elif mm[0, 0] >= 1.0 - 1e-14:  # a full cell the circle only touches
                    mm = _outside_moments_2d(0.0, 1.0, 0.0, 1.0, 10.0, 10.0, 1e-3)
                m2[b, a] = mm
    # assemble (p along x, q along y, r along z): direction p_ -> index of m2's first moment axis
    for pz in range(3):
        for qy in range(3):
            for rx in range(3):
                e = {0: rx, 1: qy, 2: pz}
                val = m2[:, :, e[p_], e[q_]] * za[e[axis]]
                sh = [1, 1, 1]
                sh[2 - q_] = n[q_]
                sh[2 - p_] = n[p_]
                M[..., rx, qy, pz] = np.broadcast_to(val.reshape(sh), (n[2], n[1], n[0]))
    return M


def moments_components(M):
    """(nz, ny, nx, 3, 3, 3) moments -> the (27, nz, ny, nx) array of gbp_nodal_set_eb, component
    p + 3q + 9r."""
    M = np.asarray(M, dtype=np.float64)
    return np.ascontiguousarray(M.transpose(5, 4, 3, 0, 1, 2).reshape((27,) + M.shape[:3]))


def _arc_centroid(x0, x1, y0, y1, cx, cy, r):
    """Centroid of the part of the circle (cx, cy, r) inside the rectangle, or None when the circle
    does not pass through it. The circle is cut at the angles where it crosses the rectangle's four
    side lines; each piece between two cuts is wholly inside or outside (tested at its midpoint)."""
    cuts = [0.0, 2.0 * math.pi]
    for xb in (x0, x1):
        c = (xb - cx) / r
        if abs(c) < 1.0:
            a = math.acos(c)
            cuts += [a, 2.0 * math.pi - a]
    for yb in (y0, y1):
        s = (yb - cy) / r
        if abs(s) < 1.0:
            a = math.asin(s)
            cuts += [a % (2.0 * math.pi), (math.pi - a) % (2.0 * math.pi)]
    cuts = sorted(cuts)
    length = sx = sy = 0.0
    for a, b in zip(cuts[:-1], cuts[1:]):
        if b - a <= 1e-15:
            continue
        m = 0.5 * (a + b)
        px, py = cx + r * math.cos(m), cy + r * math.sin(m)
        if x0 <= px <= x1 and y0 <= py <= y1:
            length += b - a
            sx += math.sin(b) - math.sin(a)
            sy += math.cos(a) - math.cos(b)
    if length <= 0.0:
        return None
    return cx + r * sx / length, cy + r * sy / length


def cylinder_boundary(n, lo, hi, center, radius, axis=2, small_volfrac=0.0):
    """The embedded-boundary face of every cell for the cylinder of `cylinder` (the EB factory's
    boundary area, normal and centroid, getBndryArea / getBndryNormal / getBndryCent in AMReX).
    Returns dict(dap, bnorm, bcent), each (3, nz, ny, nx):
      dap[d]   = ap_d(low face) - ap_d(high face): the boundary's area vector int_EB n dA divided by
                 the cell's d-face area (n the unit normal out of the fluid, into the body), which the
                 divergence theorem gives exactly from the area fractions (so it includes any face that
                 small-cell removal closed);
      bnorm    = the unit normal out of the fluid (dap scaled by the face areas, normalised), 0 on
                 cells without a boundary face;
      bcent    = the boundary centroid's offset from the cell centre in cell widths ([-1/2, 1/2]):
                 the exact centroid of the circle's arc inside the cell in the circle's plane, 0 along
                 the axis (and 0 on cells without an arc of their own)."""
    n = tuple(int(v) for v in n)
    geo = cylinder(n, lo, hi, center, radius, axis=axis, small_volfrac=small_volfrac)
    h = [(hi[d] - lo[d]) / n[d] for d in range(3)]
    ap = (geo["apx"], geo["apy"], geo["apz"])
    dap = np.zeros((3, n[2], n[1], n[0]))
    for d in range(3):
        sl_lo = [slice(None)] * 3
        sl_hi = [slice(None)] * 3
        sl_lo[2 - d] = slice(0, n[d])
        sl_hi[2 - d] = slice(1, n[d] + 1)
        dap[d] = ap[d][tuple(sl_lo)] - ap[d][tuple(sl_hi)]
    dap[:, geo["vfrac"] <= 0.0] = 0.0
    dap[np.abs(dap) < 1e-14] = 0.0
    V = h[0] * h[1] * h[2]
    vec = np.stack([dap[d] * V / h[d] for d in range(3)])
    mag = np.sqrt((vec * vec).sum(axis=0))
    bnorm = np.where(mag > 0.0, vec / np.where(mag > 0.0, mag, 1.0), 0.0)
    bcent = np.zeros((3, n[2], n[1], n[0]))
    p, q = [d for d in range(3) if d != axis]
    edges = [lo[d] + h[d] * np.arange(n[d] + 1) for d in range(3)]
    has = mag > 0.0
    for b in range(n[q]):
        for a in range(n[p]):
            x0, x1 = edges[p][a], edges[p][a + 1]
            y0, y1 = edges[q][b], edges[q][b + 1]
            if abs(0.5 * (x0 + x1) - center[p]) > radius + h[p] or abs(0.5 * (y0 + y1) - center[q]) > radius + h[q]:
                continue
            c = _arc_centroid(x0, x1, y0, y1, center[p], center[q], radius)
            if c is None:
                continue
            idx = [slice(None)] * 3
            idx[2 - p] = a
            idx[2 - q] = b
            idx = tuple(idx)
            bcent[(p,) + idx] = np.where(has[idx], (c[0] - 0.5 * (x0 + x1)) / h[p], 0.0)
            bcent[(q,) + idx] = np.where(has[idx], (c[1] - 0.5 * (y0 + y1)) / h[q], 0.0)
    return dict(dap=dap, bnorm=bnorm, bcent=bcent)


def eb_inflow_velocity(bnorm, vel_mag=None, velocity=None, normal=None, normal_tol_deg=0.0):
    """The velocity on the embedded boundary of every cell (incflo::set_eb_velocity,
    src/boundary_conditions/incflo_set_bcs.cpp:195-280, from the eb_flow.* inputs): with `vel_mag`
    the boundary blows into the fluid along its normal (u = -vel_mag n, n out of the fluid); with
    `velocity` the given vector. With `normal` only the cells whose boundary normal lies within
    `normal_tol_deg` of -normal take it (the mask of incflo's rule, with its float-epsilon pad).
    Cells without a boundary face get 0. Returns (3, nz, ny, nx)."""
    bnorm = np.asarray(bnorm, dtype=np.float64)
    cut = (bnorm * bnorm).sum(axis=0) > 0.0
    mask = cut.astype(np.float64)
    if normal is not None:
        tol = normal_tol_deg * math.pi / 180.0 + float(np.finfo(np.float32).eps)
        dot = sum(bnorm[d] * normal[d] for d in range(3))
        mask = mask * ((dot >= -1.0 - tol) & (dot <= -1.0 + tol))
    if vel_mag is not None:
        return -mask[None] * bnorm * vel_mag
    v = np.asarray(velocity, dtype=np.float64).reshape(3, 1, 1, 1)
    return mask[None] * v
