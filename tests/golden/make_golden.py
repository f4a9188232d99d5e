"""Regenerate tests/golden/reference_solutions.npz from the reference tree.

Reads the golden data that tlaloque ships (its tests' exact solutions and the
cooling table) and stores them as arrays, so that the test suite needs no
copy of the reference at run time:

* solutions/sod_e1rpex.out      -> sod_e1rpex (1000 x 5: x, rho, u, p, e), the
  exact diagonal Sod solution at t = 0.12 used by tests_analisis.jl:77-85;
* solutions/sedov_solution_53.txt -> sedov53 (n x 7: xi, rho/rho1, V, P,
  u/u1, P/P1, T/T1) and its header's xi0;
* Z1.0.dat                       -> z1_T, z1_b (T and -log10 Lambda columns,
  cooling.f90:32-39 reads them).

Usage:  python tests/golden/make_golden.py /path/to/tlaloque
"""
import os
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_golden.py /path/to/tlaloque  (the reference source tree)")
ref = sys.argv[1]
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_solutions.npz")

sod = np.loadtxt(os.path.join(ref, "solutions", "sod_e1rpex.out"))
sed_path = os.path.join(ref, "solutions", "sedov_solution_53.txt")
sed = np.loadtxt(sed_path, comments="#")
xi0 = None
with open(sed_path) as f:
    for line in f:
        if line.startswith("# xi0"):
            xi0 = float(line.split("=")[1].split()[0])
with open(os.path.join(ref, "Z1.0.dat")) as f:
    n = int(f.readline().split()[0])
    rows = np.array([[float(v) for v in f.readline().split()] for _ in range(n)])
np.savez_compressed(out, sod_e1rpex=sod, sedov53=sed, sedov53_xi0=np.array(xi0), z1_T=rows[:, 0], z1_b=rows[:, 1])
print(out, sod.shape, sed.shape, xi0, rows.shape)
