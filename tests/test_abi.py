"""CPU checks of the C ABI: the library builds, loads, exports every declared symbol, and its
host-side logic (options / inputs surface, status strings, argument checks) works without a GPU."""
import ctypes
import os
import re

import pytest
import torch

from incflo_gb300 import _abi as A
from incflo_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build()
    return A.load()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "incflo_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbp_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(A.EXPORTS) == names


def test_version_and_status_strings(lib):
    assert lib.gbp_abi_version() == 3
    assert lib.gbp_status_string(A.GBP_NOT_CONVERGED) == b"not converged"
    assert lib.gbp_status_string(99) == b"unknown status"


def test_options_defaults_match_incflo(lib):
    o = A.default_options(A.GBP_NODAL)
    # src/incflo.H:425-455 (double precision build), InputsMultigrid.rst
    assert o.rtol == 1e-11 and o.atol == 1e-14 and o.max_coarsening_level == 100 and o.maxiter == 100
    assert A.default_options(A.GBP_MAC).maxiter == 200
    assert o.precision == A.PREC_FP64


def test_options_inputs_surface(lib):
    text = """
    # incflo deck fragment
    nodal_proj.mg_rtol = 1.0e-10
    nodal_proj.mg_atol = 1.0e-13   # trailing comment
    nodal_proj.mg_max_coarsening_level = 5
    nodal_proj.bottom_solver = bicgstab
    nodal_proj.precision = mixed
    nodal_proj.verbose = 1
    mac_proj.mg_rtol = 1.0e-6
    """
    o = A.default_options(A.GBP_NODAL)
    assert lib.gbp_options_parse(ctypes.byref(o), b"nodal_proj", text.encode()) == A.GBP_OK
    assert o.rtol == 1e-10 and o.atol == 1e-13 and o.max_coarsening_level == 5
    assert o.precision == A.PREC_MIXED and o.verbose == 1
    m = A.default_options(A.GBP_MAC)
    assert lib.gbp_options_parse(ctypes.byref(m), b"mac_proj", text.encode()) == A.GBP_OK
    assert m.rtol == 1e-6 and m.atol == 1e-14


def test_options_reject_bad_values(lib):
    o = A.default_options(A.GBP_NODAL)
    assert lib.gbp_options_set(ctypes.byref(o), b"mg_rtol", b"abc") == A.GBP_BAD_ARG
    assert b"mg_rtol" in lib.gbp_last_error()
    assert lib.gbp_options_set(ctypes.byref(o), b"no_such_key", b"1") == A.GBP_BAD_ARG
    assert lib.gbp_options_set(ctypes.byref(o), b"precision", b"fp16") == A.GBP_BAD_ARG
    assert lib.gbp_options_set(ctypes.byref(o), b"maxiter", b"2.5") == A.GBP_BAD_ARG


def test_plan_create_without_device_fails_cleanly(lib):
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    g = A.Geometry()
    for d in range(3):
        g.n_cell[d] = 8
        g.prob_hi[d] = 1.0
    bc = (ctypes.c_int * 3)(0, 0, 0)
    p = ctypes.c_void_p()
    rc = lib.gbp_plan_create(ctypes.byref(g), A.GBP_NODAL, bc, bc, None, None, ctypes.byref(p))
    assert rc == A.GBP_NO_DEVICE and not p.value


def _build_shim(tmp_path):
    import shutil
    import subprocess

    from incflo_gb300.build import LIB

    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "shim_check"
    cuda_inc = "/usr/local/cuda/include"
    cuda_lib = "/usr/local/cuda/lib64"
    cmd = [cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "shim_check.cpp"), LIB, "-L", cuda_lib, "-lcudart",
           f"-Wl,-rpath,{os.path.dirname(LIB)}", f"-Wl,-rpath,{cuda_lib}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_shim_compiles_and_reports_status(lib, tmp_path):
    """include/gb_projectors.H compiles as incflo would include it; without a GPU the call
    surfaces GBP_NO_DEVICE through gb::Error instead of aborting."""
    import subprocess

    exe = _build_shim(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stdout + r.stderr
    else:
        assert r.returncode == 3, r.stdout + r.stderr


def test_null_arguments_rejected(lib):
    assert lib.gbp_plan_create(None, 0, None, None, None, None, None) == A.GBP_BAD_ARG
    assert lib.gbp_nodal_project(None, None, None, None, 0, None) == A.GBP_BAD_ARG
    assert lib.gbp_mac_project(None, None, None, None, None, 0, None) == A.GBP_BAD_ARG
    assert lib.gbp_plan_destroy(None) == A.GBP_OK
