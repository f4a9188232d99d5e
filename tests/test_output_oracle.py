"""The output oracle's Fortran edit descriptors against known gfortran
output (Fortran 2008 10.7.2.3.3: Ew.d writes 0.d1d2...dd x 10^exp, the
exponent letter omitted when |exp| > 99 with a 2-digit field), and the
byte layout of its BIN / VTK writers on a tiny array."""
import numpy as np

from oracle import output as out


def test_fortran_e_known_answers():
    assert out.fortran_e(1.0, 15, 7) == "  0.1000000E+01"
    assert out.fortran_e(-2.5e-3, 15, 7) == " -0.2500000E-02"
    assert out.fortran_e(0.0, 15, 7) == "  0.0000000E+00"
    assert out.fortran_e(1.234e123, 15, 7) == "  0.1234000+124"
    assert out.fortran_e(3.0857e18, 16, 7, 3) == "  0.3085700E+019"
    assert out.fortran_e(-1.2345678e-20, 16, 7, 3) == " -0.1234568E-019"
    assert out.fortran_e(9.99999996, 15, 7) == "  0.1000000E+02"  # rounds up into the next decade
    assert out.fortran_e(1e300, 8, 7) == "********"


def test_file_names_and_layouts():
    assert out.file_name(3, "./DATA/", 7) == "./DATA/points000N007.bin"
    assert out.file_name(2, "", 12, 1) == "EPV001N012.vtk"
    W = np.arange(5 * 5 * 6 * 7, dtype=float).reshape((5, 5, 6, 7), order="F")  # nx, ny, nz = 1, 2, 3
    b = out.bin_bytes(W)
    assert len(b) == W.size * 8 and np.frombuffer(b, "<f8")[1] == W[1, 0, 0, 0]
    v = out.vtk_bytes(W, 1, 2, 3, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
    assert v.startswith(b"# vtk DataFile Version 2.0\noutput from Diable\nBINARY\nDATASET STRUCTURED_POINTS\n"
                        b"DIMENSIONS      1     2     3\n")
    assert b"POINT_DATA          6\nSCALARS Density double 1\nLOOKUP_TABLE default\n" in v
