"""AMReX checkpoint and plotfile reader / writer for the projection's fields (host-side I/O).

incflo writes its state with WriteCheckPointFile / ReadCheckpointFile and WritePlotFile
(src/utilities/io.cpp:16-66, 69-250, 337-...): a directory with a text ``Header`` and, per level, one
VisMF MultiFab per field (``Level_<l>/<name>_H`` header + ``<name>_D_00000`` data) or, for plotfiles,
one ``Level_<l>/Cell`` MultiFab holding every plotted variable. This module reads and writes those
formats so fields can be exchanged with reference runs and stored as warm-start datasets:

  * VisMF (version 1, one data file): header = version, how, ncomp, nghost, the BoxArray, the box
    count, one ``FabOnDisk: <file> <offset>`` line per box, then per-component min and max per box;
    data = per box a ``FAB (<real descriptor>)(<box>) <ncomp>`` line followed by the box's values in
    Fortran order (x fastest, components slowest), IEEE double little-endian;
  * BoxArray text: ``(<n> 0`` then one ``((lo) (hi) (type))`` per box and ``)``; a nodal MultiFab
    (p_nd) has type (1,1,1) and node index bounds;
  * checkpoint Header: ``Checkpoint version: 1``, finest level, step, time, dt, prev_dt,
    prev_prev_dt, prob_lo, prob_hi, one BoxArray per level; plotfile Header: ``HyperCLaw-V1.1`` and
    the AMReX plotfile header fields.

One deliberate difference: incflo writes and reads ``p_nd`` when the cell-centred projection is on
and ``p_cc`` otherwise (io.cpp:99-105, 234-240), i.e. the pressure that the run does not use; here the
checkpoint holds the pressure of the projection in use (p_cc with the cell-centred projection, p_nd
otherwise).

Arrays follow incflo_gb300.projection: one box per level here, cell fields (ncomp, nz, ny, nx) or
(nz, ny, nx), nodal fields (nz+1, ny+1, nx+1).
"""
from __future__ import annotations

import os
import re

import numpy as np

_REAL_DESC = "((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))"  # IEEE double, little-endian


def _box_str(lo, hi, nodal):
    t = (1, 1, 1) if nodal else (0, 0, 0)
    return "((%d,%d,%d) (%d,%d,%d) (%d,%d,%d))" % (*lo, *hi, *t)


_BOX_RE = re.compile(r"\(\((-?\d+),(-?\d+),(-?\d+)\) \((-?\d+),(-?\d+),(-?\d+)\) \((\d+),(\d+),(\d+)\)\)")


def _parse_box(s):
    m = _BOX_RE.search(s)
    if not m:
        raise ValueError(f"not an AMReX box: {s!r}")
    v = [int(x) for x in m.groups()]
    return tuple(v[0:3]), tuple(v[3:6]), tuple(v[6:9])


def boxarray_text(boxes, nodal=False):
    out = ["(%d 0" % len(boxes)]
    out += [_box_str(lo, hi, nodal) for lo, hi in boxes]
    out.append(")")
    return "\n".join(out) + "\n"


def _read_boxarray(lines, i):
    head = lines[i].strip().lstrip("(").split()
    n = int(head[0])
    boxes = [_parse_box(lines[i + 1 + b]) for b in range(n)]
    return boxes, i + n + 2


def _as4(a):
    a = np.asarray(a, dtype=np.float64)
    return a[None] if a.ndim == 3 else a


def write_multifab(prefix, data, nodal=False, lo=(0, 0, 0)):
    """VisMF write of one single-box MultiFab: ``prefix``_H and ``prefix``_D_00000."""
    d = _as4(data)
    ncomp = d.shape[0]
    hi = tuple(lo[q] + d.shape[3 - q] - 1 for q in range(3))
    dname = os.path.basename(prefix) + "_D_00000"
    head = "FAB " + _REAL_DESC + _box_str(lo, hi, nodal) + " %d\n" % ncomp
    with open(prefix + "_D_00000", "wb") as f:
        f.write(head.encode())
        f.write(np.ascontiguousarray(d, dtype="<f8").tobytes())
    mins = ",".join("%.17g" % v for v in d.reshape(ncomp, -1).min(axis=1)) + ","
    maxs = ",".join("%.17g" % v for v in d.reshape(ncomp, -1).max(axis=1)) + ","
    with open(prefix + "_H", "w") as f:
        f.write("1\n0\n%d\n0\n" % ncomp)
        f.write(boxarray_text([(lo, hi)], nodal))
        f.write("1\nFabOnDisk: %s 0\n\n" % dname)
        f.write("1,%d\n%s\n\n1,%d\n%s\n" % (ncomp, mins, ncomp, maxs))


def read_multifab(prefix):
    """VisMF read: returns (array (ncomp, nz, ny, nx) of the first box, box lo, nodal flag). Multi-box
    MultiFabs are assembled onto their bounding box."""
    with open(prefix + "_H") as f:
        lines = f.read().splitlines()
    ncomp = int(lines[2])
    boxes, i = _read_boxarray(lines, 4)
    nbox = int(lines[i].strip())
    fabs = []
    for b in range(nbox):
        parts = lines[i + 1 + b].split()
        fabs.append((parts[1], int(parts[2])))
    los = np.array([bx[0] for bx in boxes])
    his = np.array([bx[1] for bx in boxes])
    nodal = boxes[0][2] == (1, 1, 1)
    glo, ghi = los.min(axis=0), his.max(axis=0)
    out = np.zeros((ncomp,) + tuple(int(ghi[q] - glo[q] + 1) for q in (2, 1, 0)))
    base = os.path.dirname(prefix)
    for (lo, hi, _), (fname, off) in zip(boxes, fabs):
        with open(os.path.join(base, fname), "rb") as f:
            f.seek(off)
            head = f.readline().decode()
            if "(8 7 6 5 4 3 2 1)" not in head:
                raise ValueError("only little-endian IEEE double FABs are supported")
            shape = tuple(hi[q] - lo[q] + 1 for q in (2, 1, 0))
            nc = int(head.rsplit(")", 1)[1])
            vals = np.frombuffer(f.read(8 * nc * int(np.prod(shape))), dtype="<f8").reshape((nc,) + shape)
        sl = tuple(slice(lo[q] - glo[q], hi[q] - glo[q] + 1) for q in (2, 1, 0))
        out[(slice(None),) + sl] = vals
    return out, tuple(int(v) for v in glo), nodal


def write_checkpoint(path, n_cell, prob_lo, prob_hi, velocity, density, gradp, pressure, *, use_cc_proj=False,
                     tracer=None, nstep=0, time=0.0, dt=0.0, prev_dt=0.0, prev_prev_dt=0.0):
    """incflo::WriteCheckPointFile for one single-box level: velocity (3, nz, ny, nx), density, gradp,
    and the projection's pressure (p_nd nodal, or p_cc with use_cc_proj)."""
    lev = os.path.join(path, "Level_0")
    os.makedirs(lev, exist_ok=True)
    hi = tuple(v - 1 for v in n_cell)
    with open(os.path.join(path, "Header"), "w") as f:
        f.write("Checkpoint version: 1\n0\n%d\n%.17g\n%.17g\n%.17g\n%.17g\n" % (nstep, time, dt, prev_dt, prev_prev_dt))
        f.write(" ".join("%.17g" % v for v in prob_lo) + " \n")
        f.write(" ".join("%.17g" % v for v in prob_hi) + " \n")
        f.write(boxarray_text([((0, 0, 0), hi)]))
    write_multifab(os.path.join(lev, "velocity"), velocity)
    write_multifab(os.path.join(lev, "density"), density)
    if tracer is not None:
        write_multifab(os.path.join(lev, "tracer"), tracer)
    write_multifab(os.path.join(lev, "gradp"), gradp)
    if use_cc_proj:
        write_multifab(os.path.join(lev, "p_cc"), pressure)
    else:
        write_multifab(os.path.join(lev, "p_nd"), pressure, nodal=True)


def read_checkpoint(path):
    """incflo::ReadCheckpointFile: header values and the level-0 fields present (velocity, density,
    tracer, gradp, p_nd, p_cc), each (ncomp, ...) or (...) for one component."""
    with open(os.path.join(path, "Header")) as f:
        lines = f.read().splitlines()
    if not lines[0].startswith("Checkpoint version"):
        raise ValueError("not an incflo checkpoint header")
    out = {"finest_level": int(lines[1]), "nstep": int(lines[2]), "time": float(lines[3]), "dt": float(lines[4]),
           "prev_dt": float(lines[5]), "prev_prev_dt": float(lines[6]),
           "prob_lo": [float(v) for v in lines[7].split()], "prob_hi": [float(v) for v in lines[8].split()]}
    boxes, _ = _read_boxarray(lines, 9)
    out["boxes"] = boxes
    lev = os.path.join(path, "Level_0")
    for name in ("velocity", "density", "tracer", "gradp", "p_nd", "p_cc"):
        if os.path.exists(os.path.join(lev, name + "_H")):
            a, _, _ = read_multifab(os.path.join(lev, name))
            out[name] = a[0] if a.shape[0] == 1 else a
    return out


def write_plotfile(path, n_cell, prob_lo, prob_hi, variables, *, time=0.0, nstep=0):
    """AMReX single-level plotfile (HyperCLaw-V1.1): variables = {name: cell array (nz, ny, nx)} in
    order (incflo's names: velx, vely, velz, gpx, gpy, gpz, density, p_nd (node average), ...)."""
    names = list(variables)
    data = np.stack([np.asarray(variables[k], dtype=np.float64) for k in names])
    lev = os.path.join(path, "Level_0")
    os.makedirs(lev, exist_ok=True)
    hi = tuple(v - 1 for v in n_cell)
    dx = [(prob_hi[d] - prob_lo[d]) / n_cell[d] for d in range(3)]
    with open(os.path.join(path, "Header"), "w") as f:
        f.write("HyperCLaw-V1.1\n%d\n" % len(names))
        f.write("".join(k + "\n" for k in names))
        f.write("3\n%.17g\n0\n" % time)
        f.write(" ".join("%.17g" % v for v in prob_lo) + " \n")
        f.write(" ".join("%.17g" % v for v in prob_hi) + " \n")
        f.write("\n")
        f.write(_box_str((0, 0, 0), hi, False) + " \n")
        f.write("%d \n" % nstep)
        f.write(" ".join("%.17g" % v for v in dx) + " \n")
        f.write("0\n0\n")
        f.write("0 1 %.17g\n%d\n" % (time, nstep))
        for d in range(3):
            f.write("%.17g %.17g\n" % (prob_lo[d], prob_hi[d]))
        f.write("Level_0/Cell\n")
    write_multifab(os.path.join(lev, "Cell"), data)


def read_plotfile(path):
    """Single-level AMReX plotfile: dict(time, nstep, prob_lo, prob_hi, n_cell, variables={name: array})."""
    with open(os.path.join(path, "Header")) as f:
        lines = f.read().splitlines()
    if not lines[0].startswith("HyperCLaw"):
        raise ValueError("not an AMReX plotfile header")
    nv = int(lines[1])
    names = [lines[2 + q].strip() for q in range(nv)]
    i = 2 + nv
    time = float(lines[i + 1])
    finest = int(lines[i + 2])
    prob_lo = [float(v) for v in lines[i + 3].split()]
    prob_hi = [float(v) for v in lines[i + 4].split()]
    lo, hi, _ = _parse_box(lines[i + 6])
    nstep = int(lines[i + 7].split()[0])
    data, _, _ = read_multifab(os.path.join(path, "Level_0", "Cell"))
    return {"time": time, "finest_level": finest, "nstep": nstep, "prob_lo": prob_lo, "prob_hi": prob_hi,
            "n_cell": [hi[q] - lo[q] + 1 for q in range(3)],
            "variables": {k: data[q] for q, k in enumerate(names)}}


def node_to_cell(p_nd):
    """amrex::average_node_to_cellcenter of a nodal field (incflo plots p_nd this way)."""
    p = np.asarray(p_nd)
    return 0.125 * (p[:-1, :-1, :-1] + p[:-1, :-1, 1:] + p[:-1, 1:, :-1] + p[:-1, 1:, 1:]
                    + p[1:, :-1, :-1] + p[1:, :-1, 1:] + p[1:, 1:, :-1] + p[1:, 1:, 1:])
