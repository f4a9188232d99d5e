"""Oracle of the output path (test infrastructure only): the bytes the
reference's `output` subroutine writes (source/HydroCore.f90:253-395) for a
UPrim array in the reference layout (5, nx+4, ny+4, nz+4), Fortran order.

* BIN (HydroCore.f90:276-280): `write(unitout) UPrim(:,:,:,:)`, stream
  access, little-endian: the raw array, ghosts included.
* DAT (:290-310): one formatted record per interior cell, format
  '(14(e16.7e3))' with float(i)*dx, float(j)*dy, float(k)*dz, UPrim(:,i,j,k);
  the loops run k over the x range, j over y, i over the z range (the
  reference's own bounds).
* VTK (:312-387): big-endian stream; header lines, DIMENSIONS '(3i6,1x)',
  ORIGIN/SPACING '3e15.7' (trimmed), POINT_DATA '(a,i10)', then density,
  pressure and the velocity triplets of the interior, x fastest.
File names (:269-271): points<rank i3.3>N<nout i3.3>.bin/.dat, EPV...vtk.
"""
from __future__ import annotations

import math

import numpy as np


def fortran_e(v: float, w: int, d: int, e: int = 0) -> str:
    """Fortran Ew.d (e = 0) or Ew.dEe edit descriptor as gfortran writes it:
    0.ddd form with the optional leading zero, exponent letter dropped when a
    2-digit exponent field overflows, asterisks when the field overflows."""
    if math.isnan(v):
        s = "NaN"
    elif math.isinf(v):
        s = "-Infinity" if v < 0 else "Infinity"
    else:
        m = f"{v:.{d - 1}e}"  # d significant digits, correctly rounded
        neg = m.startswith("-")
        m = m.lstrip("-")
        mant, ex = m.split("e")
        digits = mant.replace(".", "")
        ex = int(ex) + (1 if v != 0.0 else 0)
        sign = "-" if ex < 0 else "+"
        if e > 0:
            es = f"E{sign}{abs(ex):0{e}d}"
        elif abs(ex) <= 99:
            es = f"E{sign}{abs(ex):02d}"
        else:
            es = f"{sign}{abs(ex):03d}"
        s = ("-" if neg else "") + "0." + digits + es
    return "*" * w if len(s) > w else s.rjust(w)


def file_name(fmt: int, outputpath: str, nout: int, rank: int = 0) -> str:
    tag = f"{rank:03d}N{nout:03d}"
    return outputpath + {3: f"points{tag}.bin", 1: f"points{tag}.dat", 2: f"EPV{tag}.vtk"}[fmt]


def bin_bytes(W: np.ndarray) -> bytes:
    return np.asfortranarray(W, dtype="<f8").tobytes(order="F")


def dat_bytes(W: np.ndarray, nx: int, ny: int, nz: int, dx: float, dy: float, dz: float) -> bytes:
    out = []
    for k in range(1, nx + 1):
        for j in range(1, ny + 1):
            for i in range(1, nz + 1):
                vals = [i * dx, j * dy, k * dz] + [float(W[e, i + 1, j + 1, k + 1]) for e in range(5)]
                out.append("".join(fortran_e(v, 16, 7, 3) for v in vals) + "\n")
    return "".join(out).encode()


def vtk_bytes(W: np.ndarray, nx: int, ny: int, nz: int, xl: float, yl: float, zl: float, dx: float, dy: float,
              dz: float) -> bytes:
    lf = b"\n"
    hdr = [b"# vtk DataFile Version 2.0", b"output from Diable", b"BINARY", b"DATASET STRUCTURED_POINTS",
           f"DIMENSIONS {nx:6d}{ny:6d}{nz:6d}".encode(),
           ("ORIGIN " + "".join(fortran_e(v, 15, 7) for v in (xl, yl, zl))).rstrip().encode(),
           ("SPACING" + "".join(fortran_e(v, 15, 7) for v in (dx, dy, dz))).rstrip().encode(),
           f"POINT_DATA {nx * ny * nz:10d}".encode()]
    inner = W[:, 2:nx + 2, 2:ny + 2, 2:nz + 2]
    be = lambda a: np.asarray(a, dtype=">f8").tobytes(order="F")
    body = b"".join(h + lf for h in hdr)
    body += b"SCALARS Density double 1" + lf + b"LOOKUP_TABLE default" + lf + be(inner[0]) + lf
    body += b"SCALARS Pressure double 1" + lf + b"LOOKUP_TABLE default" + lf + be(inner[4]) + lf
    vel = np.stack([inner[1], inner[2], inner[3]], axis=0)  # (3, nx, ny, nz): triplets, x fastest
    body += b"VECTORS Velocity double" + lf + be(vel) + lf
    return body
