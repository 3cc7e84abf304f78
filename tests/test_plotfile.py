"""AMReX checkpoint / plotfile I/O (incflo_gb300.plotfile): bit-exact round trips of the projection's
fields, the documented text layout of headers and FAB records, multi-box assembly, and the pressure
that the checkpoint holds (the projection's own, not incflo's swapped p_nd / p_cc)."""
import os

import numpy as np

from incflo_gb300 import plotfile as pf


def test_checkpoint_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    n = (8, 6, 4)
    vel = rng.standard_normal((3, n[2], n[1], n[0]))
    rho = rng.uniform(1, 3, (n[2], n[1], n[0]))
    gp = rng.standard_normal((3, n[2], n[1], n[0]))
    p_nd = rng.standard_normal((n[2] + 1, n[1] + 1, n[0] + 1))
    path = str(tmp_path / "chk00010")
    pf.write_checkpoint(path, n, (0, 0, 0), (1.0, 0.75, 0.5), vel, rho, gp, p_nd, nstep=10, time=0.25, dt=0.01,
                        prev_dt=0.011, prev_prev_dt=0.012)
    r = pf.read_checkpoint(path)
    assert r["nstep"] == 10 and r["time"] == 0.25 and r["dt"] == 0.01 and r["prev_prev_dt"] == 0.012
    assert r["prob_hi"] == [1.0, 0.75, 0.5] and r["boxes"] == [((0, 0, 0), (7, 5, 3), (0, 0, 0))]
    assert np.array_equal(r["velocity"], vel) and np.array_equal(r["density"], rho)
    assert np.array_equal(r["gradp"], gp) and np.array_equal(r["p_nd"], p_nd)
    assert "p_cc" not in r
    # the nodal MultiFab is written with nodal box type and node bounds
    with open(os.path.join(path, "Level_0", "p_nd_H")) as f:
        assert "((0,0,0) (8,6,4) (1,1,1))" in f.read()
    # with the cell-centred projection the checkpoint holds p_cc
    path2 = str(tmp_path / "chk_cc")
    pcc = rng.standard_normal((n[2], n[1], n[0]))
    pf.write_checkpoint(path2, n, (0, 0, 0), (1, 1, 1), vel, rho, gp, pcc, use_cc_proj=True)
    r2 = pf.read_checkpoint(path2)
    assert "p_nd" not in r2 and np.array_equal(r2["p_cc"], pcc)


def test_fab_record_layout(tmp_path):
    a = np.arange(2 * 3 * 4 * 5, dtype=np.float64).reshape(2, 3, 4, 5)  # (ncomp, nz, ny, nx)
    pf.write_multifab(str(tmp_path / "f"), a)
    raw = open(tmp_path / "f_D_00000", "rb").read()
    head, body = raw.split(b"\n", 1)
    assert head.decode() == "FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))((0,0,0) (4,3,2) (0,0,0)) 2"
    vals = np.frombuffer(body, dtype="<f8")
    assert vals[1] == 1.0 and vals[5] == 5.0 and vals[60] == 60.0  # x fastest, then y, z, component
    hdr = open(tmp_path / "f_H").read().splitlines()
    assert hdr[:4] == ["1", "0", "2", "0"] and hdr[4] == "(1 0" and hdr[7] == "1"
    assert hdr[8] == "FabOnDisk: f_D_00000 0"


def test_multibox_assembly(tmp_path):
    """A two-box MultiFab (as a multi-rank AMReX run writes it) is assembled on its bounding box."""
    rng = np.random.default_rng(1)
    full = rng.standard_normal((1, 4, 4, 8))
    boxes = [((0, 0, 0), (3, 3, 3)), ((4, 0, 0), (7, 3, 3))]
    prefix = str(tmp_path / "m")
    with open(prefix + "_D_00000", "wb") as f:
        offs = []
        for lo, hi in boxes:
            offs.append(f.tell())
            f.write(("FAB " + pf._REAL_DESC + pf._box_str(lo, hi, False) + " 1\n").encode())
            f.write(np.ascontiguousarray(full[:, :, :, lo[0]:hi[0] + 1]).astype("<f8").tobytes())
    with open(prefix + "_H", "w") as f:
        f.write("1\n0\n1\n0\n" + pf.boxarray_text(boxes) + "2\n")
        f.write("".join("FabOnDisk: m_D_00000 %d\n" % o for o in offs))
    a, lo, nodal = pf.read_multifab(prefix)
    assert lo == (0, 0, 0) and not nodal and np.array_equal(a, full)


def test_plotfile_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    n = (8, 4, 4)
    p_nd = rng.standard_normal((5, 5, 9))
    v = {"velx": rng.standard_normal((4, 4, 8)), "vely": rng.standard_normal((4, 4, 8)),
         "p_nd": pf.node_to_cell(p_nd)}
    path = str(tmp_path / "plt00005")
    pf.write_plotfile(path, n, (0, 0, 0), (2.0, 1.0, 1.0), v, time=0.5, nstep=5)
    r = pf.read_plotfile(path)
    assert r["time"] == 0.5 and r["nstep"] == 5 and r["n_cell"] == [8, 4, 4] and r["prob_hi"] == [2.0, 1.0, 1.0]
    assert list(r["variables"]) == ["velx", "vely", "p_nd"]
    for k in v:
        assert np.array_equal(r["variables"][k], v[k])
    assert open(os.path.join(path, "Header")).readline().strip() == "HyperCLaw-V1.1"
