"""Seeded synthetic inputs of the projection workloads (numpy PCG64; no datasets are read).

incflo itself cannot run here, so these generators stand in for the states incflo would hand to
its projections. Every array uses the C-order layout of incflo_gb300.projection (last axis x).

  taylor_green_noise     [0,2pi]^3 triply periodic, u = sin x cos y cos z, v = -cos x sin y cos z,
                         w = 0, plus U(-a, a) noise per component (seed 1, a = 1e-2)
  variable_density_rt    unit cube, periodic x/y, walls in z: rho = 1 below / 3 above a tanh
                         interface of width 2 cells at z = 0.5 + h(x, y), h a seeded sum of
                         cosine modes 1..8 with max amplitude 0.01 (seed 2); velocity a Gaussian
                         random field with E(k) ~ k^-2, zero mean, unit RMS (seed 3)
  double_shear_layer     u = tanh(30 (y - 1/4)) for y <= 1/2, tanh(30 (3/4 - y)) above,
                         v = 0.05 sin(2 pi x), w = 0 (the reference's form,
                         src/prob/prob_init_fluid.cpp:879-898)
"""
from __future__ import annotations

import numpy as np

PERIODIC, DIRICHLET, NEUMANN, INFLOW = 0, 1, 2, 3


def _cell_centres(n, lo, hi):
    h = [(hi[d] - lo[d]) / n[d] for d in range(3)]
    xs = [lo[d] + (np.arange(n[d]) + 0.5) * h[d] for d in range(3)]
    Z, Y, X = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    return X, Y, Z


def taylor_green_noise(n=64, seed=1, amp=1e-2):
    lo, hi = (0.0,) * 3, (2 * np.pi,) * 3
    X, Y, Z = _cell_centres((n, n, n), lo, hi)
    rng = np.random.Generator(np.random.PCG64(seed))
    vel = np.empty((3, n, n, n))
    vel[0] = np.sin(X) * np.cos(Y) * np.cos(Z)
    vel[1] = -np.cos(X) * np.sin(Y) * np.cos(Z)
    vel[2] = 0.0
    vel += rng.uniform(-amp, amp, size=vel.shape)
    rho = np.ones((n, n, n))
    return dict(n=(n, n, n), lo=lo, hi=hi, bclo=(PERIODIC,) * 3, bchi=(PERIODIC,) * 3, vel=vel, rho=rho)


def gaussian_random_field(n, seed, slope=-2.0, ncomp=3):
    """Periodic Gaussian random vector field with energy spectrum E(k) ~ k^slope, zero mean, unit RMS."""
    rng = np.random.Generator(np.random.PCG64(seed))
    k = [np.fft.fftfreq(n[d]) * n[d] for d in range(3)]
    kz, ky, kx = np.meshgrid(k[2], k[1], np.fft.rfftfreq(n[0]) * n[0], indexing="ij")
    kk = np.sqrt(kx * kx + ky * ky + kz * kz)
    # |u_hat|^2 ~ E(k) / k^2 in three dimensions
    amp = np.zeros_like(kk)
    nz = kk > 0
    amp[nz] = kk[nz] ** ((slope - 2.0) / 2.0)
    out = np.empty((ncomp, n[2], n[1], n[0]))
    for c in range(ncomp):
        white = rng.standard_normal((n[2], n[1], n[0]))
        f = np.fft.rfftn(white) * amp
        out[c] = np.fft.irfftn(f, s=(n[2], n[1], n[0]), axes=(0, 1, 2))
    out -= out.mean(axis=(1, 2, 3), keepdims=True)
    out /= np.sqrt(np.mean(np.sum(out * out, axis=0)))
    return out


def interface_height(n, seed=2, modes=8, amplitude=0.01, t=0.0, growth=0.0):
    """Interface height 0.5 + h(x, y): a seeded sum of cosine modes (wavenumbers 1..modes) scaled to the
    amplitude. t > 0 displaces it slowly (the interface of a time sequence): mode m travels by phase
    0.05 m t and its amplitude grows by the factor 1 + growth t."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x = (np.arange(n[0]) + 0.5) / n[0]
    y = (np.arange(n[1]) + 0.5) / n[1]
    Y, X = np.meshgrid(y, x, indexing="ij")
    a = rng.uniform(-1.0, 1.0, size=(2, modes))
    th = rng.uniform(0.0, 2 * np.pi, size=(2, modes))
    h = np.zeros_like(X)
    for m in range(1, modes + 1):
        h += a[0, m - 1] * np.cos(2 * np.pi * m * X + th[0, m - 1] + 0.05 * m * t)
        h += a[1, m - 1] * np.cos(2 * np.pi * m * Y + th[1, m - 1] - 0.05 * m * t)
    h0 = np.zeros_like(X)
    for m in range(1, modes + 1):
        h0 += a[0, m - 1] * np.cos(2 * np.pi * m * X + th[0, m - 1])
        h0 += a[1, m - 1] * np.cos(2 * np.pi * m * Y + th[1, m - 1])
    h *= amplitude * (1.0 + growth * t) / np.abs(h0).max()
    return 0.5 + h


def variable_density_rt(n=256, seed_h=2, seed_u=3, rho_lo=1.0, rho_hi=3.0):
    nn = (n, n, n) if np.isscalar(n) else tuple(n)
    lo, hi = (0.0,) * 3, (1.0,) * 3
    dz = 1.0 / nn[2]
    z = (np.arange(nn[2]) + 0.5) * dz
    hxy = interface_height(nn, seed_h)
    rho = rho_lo + (rho_hi - rho_lo) * 0.5 * (1.0 + np.tanh((z[:, None, None] - hxy[None, :, :]) / (2.0 * dz)))
    vel = gaussian_random_field(nn, seed_u)
    return dict(n=nn, lo=lo, hi=hi, bclo=(PERIODIC, PERIODIC, NEUMANN), bchi=(PERIODIC, PERIODIC, NEUMANN),
                vel=vel, rho=rho)


def double_shear_layer(n=128, seed=None, amp_noise=0.0):
    nn = (n, n, n) if np.isscalar(n) else tuple(n)
    lo, hi = (0.0,) * 3, (1.0,) * 3
    X, Y, Z = _cell_centres(nn, lo, hi)
    vel = np.zeros((3,) + X.shape)
    vel[0] = np.where(Y <= 0.5, np.tanh(30.0 * (Y - 0.25)), np.tanh(30.0 * (0.75 - Y)))
    vel[1] = 0.05 * np.sin(2 * np.pi * X)
    if seed is not None and amp_noise > 0:
        rng = np.random.Generator(np.random.PCG64(seed))
        vel += rng.uniform(-amp_noise, amp_noise, size=vel.shape)
    rho = np.ones(X.shape)
    return dict(n=nn, lo=lo, hi=hi, bclo=(PERIODIC,) * 3, bchi=(PERIODIC,) * 3, vel=vel, rho=rho)


def rt_sequence(n=256, seed=2, steps=8, dt=1.0, rho_lo=1.0, rho_hi=3.0):
    """Successive projections of a slowly displaced variable-density interface (the setting of a
    time-stepping run, where each projection can start from the previous one's phi): step t has the
    interface of interface_height(t, growth 0.02) and the velocity cos(w t) u_a + sin(w t) u_b of two
    seeded k^-2 fields, w = 0.05, so consecutive right-hand sides differ by a few percent. Yields the
    cases of variable_density_rt's layout."""
    nn = (n, n, n) if np.isscalar(n) else tuple(n)
    ua = gaussian_random_field(nn, seed + 101)
    ub = gaussian_random_field(nn, seed + 202)
    dz = 1.0 / nn[2]
    z = (np.arange(nn[2]) + 0.5) * dz
    for q in range(steps):
        t = q * dt
        hxy = interface_height(nn, seed, t=t, growth=0.02)
        rho = rho_lo + (rho_hi - rho_lo) * 0.5 * (1.0 + np.tanh((z[:, None, None] - hxy[None, :, :]) / (2.0 * dz)))
        vel = np.cos(0.05 * t) * ua + np.sin(0.05 * t) * ub
        yield dict(n=nn, lo=(0.0,) * 3, hi=(1.0,) * 3, bclo=(PERIODIC, PERIODIC, NEUMANN),
                   bchi=(PERIODIC, PERIODIC, NEUMANN), vel=vel, rho=rho)


def double_shear_sequence(n=128, seed=5, steps=8, dt=1.0, amp_noise=0.05):
    """Successive projections of a double shear layer (u = tanh(30 (y - 1/4)) for y <= 1/2, tanh(30 (3/4 - y))
    above, v = 0.05 sin(2 pi (x - 0.01 t)), w = 0) plus a seeded k^-2 perturbation of RMS amp_noise that
    turns slowly (as rt_sequence's velocity); constant density. Same boundary layout as rt_sequence
    (periodic x / y, walls in z)."""
    nn = (n, n, n) if np.isscalar(n) else tuple(n)
    X, Y, _ = _cell_centres(nn, (0.0,) * 3, (1.0,) * 3)
    ua = gaussian_random_field(nn, seed + 303)
    ub = gaussian_random_field(nn, seed + 404)
    for q in range(steps):
        t = q * dt
        vel = amp_noise * (np.cos(0.05 * t) * ua + np.sin(0.05 * t) * ub)
        vel[0] += np.where(Y <= 0.5, np.tanh(30.0 * (Y - 0.25)), np.tanh(30.0 * (0.75 - Y)))
        vel[1] += 0.05 * np.sin(2 * np.pi * (X - 0.01 * t))
        yield dict(n=nn, lo=(0.0,) * 3, hi=(1.0,) * 3, bclo=(PERIODIC, PERIODIC, NEUMANN),
                   bchi=(PERIODIC, PERIODIC, NEUMANN), vel=vel, rho=np.ones((nn[2], nn[1], nn[0])))


def with_ghosts(vel, ng=1):
    """Pad a (3, nz, ny, nx) cell field with ng zero ghost layers (the state after setBndry(0))."""
    return np.pad(vel, ((0, 0),) + ((ng, ng),) * 3)


def variable_density_rt_amr(n=256, band=(0.375, 0.625), box=64, seed_h=2, seed_u=3, rho_lo=1.0, rho_hi=3.0):
    """Two-level form of variable_density_rt: the base level as above plus a refined (ratio 2) band of
    whole-domain x/y extent around the interface, z in `band`, split into box^3 fine boxes (the fine
    BoxArray, max_grid_size = box). Fine density from the same interface at the fine resolution; fine
    velocity injected from the base level (a freshly regridded level). Returns the base fields, the
    fine boxes [(lo, hi)] and the fine band arrays (band origin at fine z index zlo)."""
    base = variable_density_rt(n, seed_h, seed_u, rho_lo, rho_hi)
    nn = base["n"]
    nf = tuple(2 * v for v in nn)
    zlo = int(round(band[0] * nf[2])) // box * box
    zhi = int(round(band[1] * nf[2])) // box * box
    dz = 1.0 / nf[2]
    z = (np.arange(zlo, zhi) + 0.5) * dz
    hxy = interface_height(nf, seed_h)
    rho_f = rho_lo + (rho_hi - rho_lo) * 0.5 * (1.0 + np.tanh((z[:, None, None] - hxy[None, :, :]) / (2.0 * dz)))
    vc = base["vel"][:, zlo // 2:zhi // 2]
    vel_f = np.repeat(np.repeat(np.repeat(vc, 2, axis=1), 2, axis=2), 2, axis=3)
    boxes = []
    for k in range(zlo, zhi, box):
        for j in range(0, nf[1], box):
            for i in range(0, nf[0], box):
                boxes.append(((i, j, k), (i + box - 1, j + box - 1, k + box - 1)))
    return dict(base=base, boxes=boxes, zlo=zlo, rho_f=rho_f, vel_f=np.ascontiguousarray(vel_f))


def tag_and_box(tag, blocking=32, max_grid=64):
    """incflo's regrid of a tagged coarse level into a ratio-2 fine BoxArray (amr.blocking_factor /
    amr.max_grid_size, in fine cells): a coarse block of blocking/2 cells per side is refined when any of
    its cells is tagged; refined blocks are gathered into boxes of at most max_grid fine cells per side
    (a super-block of (max_grid/2)^3 coarse cells becomes one box when all its blocks are refined, else
    each refined block is a box of its own). tag: (nz, ny, nx) bool over the coarse cells. Returns the
    fine boxes [((lo), (hi))] in fine cell indices, disjoint, lo even and hi odd."""
    nz, ny, nx = tag.shape
    bc = blocking // 2
    if any(v % bc for v in (nx, ny, nz)):
        raise ValueError("the coarse level must be a multiple of the blocking factor / 2")
    blk = tag.reshape(nz // bc, bc, ny // bc, bc, nx // bc, bc).any(axis=(1, 3, 5))
    g = max(1, max_grid // blocking)  # blocks per box side
    boxes = []
    for K in range(0, blk.shape[0], g):
        for J in range(0, blk.shape[1], g):
            for I in range(0, blk.shape[2], g):
                sub = blk[K:K + g, J:J + g, I:I + g]
                if sub.size == g ** 3 and sub.all():
                    lo = (2 * bc * I, 2 * bc * J, 2 * bc * K)
                    boxes.append((lo, tuple(v + 2 * bc * g - 1 for v in lo)))
                    continue
                for k, j, i in zip(*np.nonzero(sub)):
                    lo = (2 * bc * (I + i), 2 * bc * (J + j), 2 * bc * (K + k))
                    boxes.append((lo, tuple(v + 2 * bc - 1 for v in lo)))
    return boxes


def rt_amr_tagged(n=256, seed_h=2, seed_u=3, band=0.1, pct=90.0, blocking=32, max_grid=64, rho_lo=1.0,
                  rho_hi=3.0):
    """Two-level variable-density interface with the fine level from tagging (incflo_tagging.cpp's rules
    as the benchmark's two-level case states them): coarse cells within +-band of the interface, or whose
    vorticity magnitude exceeds its pct-th percentile, refined by 2 with amr.blocking_factor = blocking and
    amr.max_grid_size = max_grid (fine cells). The velocity is the k^-2 field concentrated at the interface
    (weight exp(-((z - h) / band)^2)), where a Rayleigh-Taylor run moves the fluid. Fine density from the
    interface at the fine resolution, fine velocity injected from the base level. Returns the base fields,
    the fine boxes and per-box fine velocity / density arrays."""
    base = variable_density_rt(n, seed_h, seed_u, rho_lo, rho_hi)
    nn = base["n"]
    dz = 1.0 / nn[2]
    z = (np.arange(nn[2]) + 0.5) * dz
    hxy = interface_height(nn, seed_h)
    dist = z[:, None, None] - hxy[None, :, :]
    vel = base["vel"] * np.exp(-(dist / band) ** 2)[None]
    base["vel"] = vel
    h = [1.0 / v for v in nn]
    # vorticity by centred differences (periodic x / y, one-sided at the z walls)
    def ddx(f, axis, hh, periodic):
        if periodic:
            return (np.roll(f, -1, axis) - np.roll(f, 1, axis)) / (2 * hh)
        return np.gradient(f, hh, axis=axis)
    u, v, w = vel
    wx = ddx(w, 1, h[1], True) - ddx(v, 0, h[2], False)
    wy = ddx(u, 0, h[2], False) - ddx(w, 2, h[0], True)
    wz = ddx(v, 2, h[0], True) - ddx(u, 1, h[1], True)
    om = np.sqrt(wx * wx + wy * wy + wz * wz)
    tag = (np.abs(dist) <= band) | (om > np.percentile(om, pct))
    boxes = tag_and_box(tag, blocking, max_grid)
    nf = tuple(2 * v for v in nn)
    dzf = 1.0 / nf[2]
    hf = interface_height(nf, seed_h)
    rho_f, vel_f = [], []
    for lo, hi in boxes:
        zf = (np.arange(lo[2], hi[2] + 1) + 0.5) * dzf
        hb = hf[lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]
        rho_f.append(np.ascontiguousarray(
            rho_lo + (rho_hi - rho_lo) * 0.5 * (1.0 + np.tanh((zf[:, None, None] - hb[None]) / (2.0 * dzf)))))
        vc = vel[:, lo[2] // 2:(hi[2] + 1) // 2, lo[1] // 2:(hi[1] + 1) // 2, lo[0] // 2:(hi[0] + 1) // 2]
        vel_f.append(np.ascontiguousarray(np.repeat(np.repeat(np.repeat(vc, 2, axis=1), 2, axis=2), 2, axis=3)))
    return dict(base=base, boxes=boxes, rho_f=rho_f, vel_f=vel_f, tagged_fraction=float(tag.mean()))
