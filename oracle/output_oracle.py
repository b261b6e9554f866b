"""CPU restatement of PLUTO's .dbl / .flt / .vtk writers -- test infrastructure.

Only the tests use this module, as the checker of the device writer
(pg_write_output); the library never calls it.  It restates, for a serial
run on a uniform Cartesian grid:

  WriteData           Src/write_data.c:29-330 (file names, variable order,
                      single_file / multiple_files), the ".out" record
                      Src/write_data.c:360-385;
  FileWriteData       Src/bin_io.c:216-259 (interior [k][j][i]; a staggered
                      component from face BEG-1 to END along its own axis);
  Convert_dbl2flt     Src/bin_io.c:51-83 ((float)(v*unit), byte swap for VTK);
  WriteVTK_Header     Src/write_vtk.c (legacy binary VTK, RECTILINEAR_GRID,
                      big-endian float node coordinates, z = 0 in 2D);
  WriteVTK_Vector     Src/write_vtk.c ((float)v*unit over the first
                      DIMENSIONS components, zero beyond, big endian);
  WriteVTK_Scalar     Src/write_vtk.c;
  SetOutput           Src/set_output.c:84-215 (default variable list: the
                      primitives in PLUTO's NVAR order, then Bx1s.. under CT;
                      staggered fields only in .dbl; VTK_VECTOR_DUMP).

State arrays use the 8-slot order of the C ABI: vc[8, nz, ny, nx] = RHO, VX1,
VX2, VX3, BX1, BX2, BX3, PRS; faces[d] one longer along d.
"""
from __future__ import annotations

import os

import numpy as np

VTK_VECTOR = 5  # Src/pluto.h:97
# SetDefaultVarNames (Src/var_names.c): the field components are "Bx1".."Bx3",
# so WriteVTK_Vector's test for "bx1" never matches them: with VTK_VECTOR_DUMP
# a single VTK file gets no magnetic vector (and Bx2, Bx3 are not dumped), and
# multiple_files mode stops with "unknown vector type".
SLOT_NAMES = ["rho", "vx1", "vx2", "vx3", "Bx1", "Bx2", "Bx3", "prs"]


def default_vars(fmt: str, dims: int, components: int, ct: bool, vtk_vector: bool = False):
    """[(var id, name, dump)] as SetOutput leaves them: var id 0..7 a cell slot,
    8 + d the staggered component d."""
    slots = [0, 1, 2] + ([3] if components == 3 else []) + [4, 5] + ([6] if components == 3 else []) + [7]
    out = [[q, SLOT_NAMES[q], 1] for q in slots]
    if ct:
        out += [[8 + d, f"Bx{d + 1}s", 1 if fmt == "dbl" else 0] for d in range(dims)]
    if fmt == "vtk" and vtk_vector:
        for first in (1, 4):  # D_EXPAND(dump[VX1] = VTK_VECTOR, dump[VX2] = NO, dump[VX3] = NO)
            for e in out:
                if first <= e[0] < first + dims:
                    e[2] = VTK_VECTOR if e[0] == first else 0
    return [tuple(e) for e in out]


def nodes(lo: float, hi: float, n: int) -> np.ndarray:
    """Left node coordinates of a uniform patch, xl_glob[BEG .. END+1]
    (Src/set_grid.c:395-403 and :60-64): xL + i*dx, the last one the right
    edge of the last zone."""
    dx = (hi - lo) / float(n)
    x = np.array([lo + float(i) * dx for i in range(n)] + [0.0])
    x[n] = x[n - 1] + dx
    return x


def _cells(vc, faces, vid):
    return faces[vid - 8] if vid >= 8 else vc[vid]


def _vtk_header(dims, nx, xnode) -> bytes:
    nx1 = nx[0]
    nx2 = nx[1] if dims >= 2 else 1
    nx3 = nx[2] if dims == 3 else 1
    n = [nx1 + 1, nx2 + (dims >= 2), nx3 + (dims == 3)]
    h = b"# vtk DataFile Version 2.0\nPLUTO 4.3 VTK Data\nBINARY\nDATASET RECTILINEAR_GRID\n"
    h += b"DIMENSIONS %d %d %d\n" % tuple(n)
    for d, ax in enumerate("XYZ"):
        h += (b"\n" if d else b"") + b"%s_COORDINATES %d float\n" % (ax.encode(), n[d])
        c = np.zeros(n[d]) if (d == 2 and dims == 2) else np.asarray(xnode[d][: n[d]], dtype=np.float64)
        h += c.astype(">f4").tobytes()
    h += b"\nCELL_DATA %d\n" % (nx1 * nx2 * nx3)
    return h


def _flt(a, unit, big):
    f = (np.asarray(a, dtype=np.float64) * unit).astype(np.float32)
    return f.astype(">f4" if big else "<f4").tobytes()


def _vector(vc, first, dims, unit):
    comps = []
    for m in range(3):
        v = vc[first + m] if m < dims else np.zeros_like(vc[first])
        comps.append((v.astype(np.float32).astype(np.float64) * unit).astype(np.float32))
    return np.stack(comps, axis=-1).astype(">f4").tobytes()


def write(directory, fmt, nfile, vc, faces, dims, components, ct, *, single_file=True, vars=None,
          vtk_vector=False, xnode=None, units=None, time=0.0, dt=0.0, step=0, write_record=True):
    """Write the files WriteData writes for format fmt ("dbl", "flt", "vtk")."""
    vars = vars if vars is not None else default_vars(fmt, dims, components, ct, vtk_vector)
    units = units or {}
    nx = [vc.shape[3], vc.shape[2], vc.shape[1]]
    files = {}
    header = _vtk_header(dims, nx, xnode) if fmt == "vtk" else b""
    single = bytearray(header)
    if fmt == "vtk":
        order = [v for v in vars if v[2] == VTK_VECTOR] + [v for v in vars if v[2] == 1]
    else:
        order = [v for v in vars if v[2]]
    for vid, name, dump in order:
        unit = 1.0 if fmt == "dbl" else units.get(name, 1.0)
        if fmt == "dbl":
            body = np.ascontiguousarray(_cells(vc, faces, vid), dtype="<f8").tobytes()
            fname = f"{name}.{nfile:04d}.dbl"
        elif fmt == "flt":
            body = _flt(_cells(vc, faces, vid), unit, False)
            fname = f"{name}.{nfile:04d}.flt"
        elif dump == VTK_VECTOR:
            if name not in ("vx1", "bx1"):
                if not single_file:
                    raise ValueError("unknown vector type in VTK output")
                continue
            kind = "Velocity" if name == "vx1" else "Magnetic"
            body = b"\nVECTORS %dD_%s_Field float\n" % (dims, kind.encode()) + _vector(vc, vid, dims, unit)
            fname = f"{'vfield' if name == 'vx1' else 'bfield'}.{nfile:04d}.vtk"
        else:
            body = b"\nSCALARS %s float\nLOOKUP_TABLE default\n" % name.encode() + _flt(vc[vid], unit, True)
            fname = f"{name}.{nfile:04d}.vtk"
        if single_file:
            single += body
        else:
            files[fname] = header + body
    if single_file:
        files[f"data.{nfile:04d}.{fmt}"] = bytes(single)
    os.makedirs(directory, exist_ok=True)
    for fname, data in files.items():
        with open(os.path.join(directory, fname), "wb") as f:
            f.write(data)
    if write_record:
        rec = "%d %12.6e %12.6e %ld " % (nfile, time, dt, step)
        rec += "single_file " if single_file else "multiple_files "
        rec += "little "
        rec += "".join(f"{name} " for _, name, dump in vars if dump) + "\n"
        path = os.path.join(directory, f"{fmt}.out")
        if nfile == 0 or not os.path.exists(path):
            mode = "w"
            lines = []
        else:
            with open(path) as f:
                lines = f.readlines()[:nfile]
            mode = "w"
        # WriteData overwrites from record nfile on without truncating the rest
        old = open(path).read() if os.path.exists(path) and nfile > 0 else ""
        head = "".join(lines)
        tail = old[len(head) + len(rec):] if len(old) > len(head) + len(rec) else ""
        with open(path, mode) as f:
            f.write(head + rec + tail)
    return sorted(files)
