"""gbp_nodal_divergence_noalloc against gbp_nodal_divergence, through the C ABI.

The no-allocation entry point serves callers that cannot allocate device memory (device memory owned
by another framework's allocator, or a plugin that may not create a plan). Its scratch is a static device array
that every call reuses, so it is called twice in a row here: the second result must match as well,
which shows that state left by the first call does not leak into the second. This file is named so
that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from incflo_gb300 import Geometry, _abi
from incflo_gb300.projection import array4, nodal_divergence
from tests.helpers import D, I, N, P, cuda, nodal_case

pytestmark = pytest.mark.gpu

CASES = [
    ((16, 16, 16), (1.0, 1.0, 1.0), (P, P, P), (P, P, P)),
    ((24, 16, 20), (1.0, 0.75, 1.25), (P, P, N), (P, P, N)),
    ((12, 16, 8), (1.5, 2.0, 1.0), (N, D, P), (I, N, P)),
    ((64, 32, 48), (2.0, 1.0, 1.5), (D, N, I), (D, I, N)),
]


def _noalloc(geom, bclo, bchi, vel, out):
    lib = _abi.load()
    m = ctypes.c_double(-1.0)
    lo = (ctypes.c_int * 3)(*bclo)
    hi = (ctypes.c_int * 3)(*bchi)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.gbp_nodal_divergence_noalloc(ctypes.byref(geom.c()), lo, hi, ctypes.byref(array4(vel, 1)), 1,
                                          ctypes.byref(array4(out)), ctypes.byref(m), stream)
    _abi.check(rc, "gbp_nodal_divergence_noalloc")
    return m.value


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[2]}-{c[3]}" for c in CASES])
def test_noalloc_divergence_matches_plan_entry_point(gpu_lib, case):
    n, ext, bclo, bchi = case
    geom = Geometry(n, (0, 0, 0), ext)
    results = []
    for seed in (7, 8):  # two calls in a row, different inputs
        _, _, vel = nodal_case(n, ext, bclo, bchi, seed=seed)
        vt = cuda(vel)
        m_ref, ref = nodal_divergence(geom, bclo, bchi, vt)
        out = torch.full((n[2] + 1, n[1] + 1, n[0] + 1), np.nan, dtype=torch.float64, device="cuda")
        m = _noalloc(geom, bclo, bchi, vt, out)
        r = ref.cpu().numpy()
        o = out.cpu().numpy()
        scale = max(np.abs(r).max(), 1e-300)
        np.testing.assert_allclose(o, r, rtol=0, atol=1e-12 * scale)
        assert abs(m - m_ref) <= 1e-12 * scale
        results.append(o)
    assert not np.array_equal(results[0], results[1])


def test_noalloc_rejects_oversized_grid(gpu_lib):
    lib = _abi.load()
    geom = Geometry((1024, 1024, 1024))
    lo = (ctypes.c_int * 3)(0, 0, 0)
    v = torch.zeros((3, 3, 3, 3), dtype=torch.float64, device="cuda")
    o = torch.zeros((2, 2, 2), dtype=torch.float64, device="cuda")
    m = ctypes.c_double()
    a = array4(v, 1)
    a.lo[0] = a.lo[1] = a.lo[2] = -1
    a.hi[0] = a.hi[1] = a.hi[2] = 1024
    b = array4(o)
    b.hi[0] = b.hi[1] = b.hi[2] = 1024
    rc = lib.gbp_nodal_divergence_noalloc(ctypes.byref(geom.c()), lo, lo, ctypes.byref(a), 0, ctypes.byref(b),
                                          ctypes.byref(m), None)
    assert rc == _abi.GBP_BAD_ARG
    assert b"65536" in lib.gbp_last_error()


def test_noalloc_reads_only_the_ghost_layer_it_is_given(gpu_lib):
    """A velocity view that ends exactly at the ghost layer of the high-z inflow face (no ghosts
    anywhere else), inside a buffer whose remainder holds NaN: the result must match the plan entry
    point, which it cannot if the kernel read past the view."""
    n, ext = (40, 24, 20), (1.0, 1.0, 1.0)
    bclo, bchi = (P, N, D), (P, N, I)
    geom = Geometry(n, (0, 0, 0), ext)
    _, _, vel = nodal_case(n, ext, bclo, bchi, seed=11)
    vt = cuda(vel)
    m_ref, ref = nodal_divergence(geom, bclo, bchi, vt)
    tight = vel[:, 1:, 1:-1, 1:-1]  # z cells 0..n (the top ghost plane), y / x valid cells only
    count = tight.size
    buf = torch.full((count + 4096,), float("nan"), dtype=torch.float64, device="cuda")
    view = buf[:count].view(tight.shape)
    view.copy_(cuda(tight))
    for _ in range(2):
        out = torch.full((n[2] + 1, n[1] + 1, n[0] + 1), np.nan, dtype=torch.float64, device="cuda")
        lib = _abi.load()
        m = ctypes.c_double(-1.0)
        lo = (ctypes.c_int * 3)(*bclo)
        hi = (ctypes.c_int * 3)(*bchi)
        a = array4(view, lo=(0, 0, 0))
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        rc = lib.gbp_nodal_divergence_noalloc(ctypes.byref(geom.c()), lo, hi, ctypes.byref(a), 1,
                                              ctypes.byref(array4(out)), ctypes.byref(m), stream)
        _abi.check(rc, "gbp_nodal_divergence_noalloc")
        r = ref.cpu().numpy()
        o = out.cpu().numpy()
        scale = max(np.abs(r).max(), 1e-300)
        assert np.isfinite(o).all()
        np.testing.assert_allclose(o, r, rtol=0, atol=1e-12 * scale)
        assert abs(m.value - m_ref) <= 1e-12 * scale


def test_noalloc_rejects_missing_inflow_ghost(gpu_lib):
    """The ghost layer is required only on inflow sides, and there it is required."""
    n = (16, 16, 16)
    bclo, bchi = (P, P, N), (P, P, I)
    geom = Geometry(n)
    _, _, vel = nodal_case(n, (1.0, 1.0, 1.0), bclo, bchi, seed=3)
    short = cuda(vel[:, 1:-1, 1:-1, 1:-1])  # no top ghost plane
    out = torch.zeros((n[2] + 1, n[1] + 1, n[0] + 1), dtype=torch.float64, device="cuda")
    lib = _abi.load()
    m = ctypes.c_double()
    lo = (ctypes.c_int * 3)(*bclo)
    hi = (ctypes.c_int * 3)(*bchi)
    rc = lib.gbp_nodal_divergence_noalloc(ctypes.byref(geom.c()), lo, hi, ctypes.byref(array4(short, lo=(0, 0, 0))),
                                          1, ctypes.byref(array4(out)), ctypes.byref(m), None)
    assert rc == _abi.GBP_BAD_ARG
