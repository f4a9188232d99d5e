"""The C ABI from a plain C program (tests/c_driver/sod_driver.c): it
compiles and links against include/tlq.h and libtlq.so with gcc (CPU), and
on the GPU its Sod run matches the oracle's (the same bits as the Python
binding's path: t, it and the conserved sums)."""
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT

SRC = os.path.join(ROOT, "tests", "c_driver", "sod_driver.c")
LIBDIR = os.path.join(ROOT, "tlaloque_gb300", "_lib")


def build_driver(tmp_path):
    from tlaloque_gb300 import build as b
    b.build()
    exe = str(tmp_path / "sod_driver")
    subprocess.run(["gcc", "-std=c11", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, "-L", LIBDIR,
                    "-ltlq", "-Wl,-rpath," + LIBDIR, "-lm"], check=True)
    return exe


def test_c_driver_compiles_and_links(tmp_path):
    exe = build_driver(tmp_path)
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_c_driver_sod_matches_oracle(gpu_lib, tmp_path):
    exe = build_driver(tmp_path)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=300).stdout.split()
    t, it = float(out[1]), int(out[3])
    sums = np.array([float(v) for v in out[5:10]])
    from oracle.oracle import Run
    from tests.helpers import oracle_params
    from tlaloque_gb300 import problems
    cfg, U0 = problems.sod_tube()
    run = Run(oracle_params(cfg), U0)
    run.run(1 << 20, tfin=problems.SOD_TFIN)
    assert (t, it) == (run.t, run.it)
    ref = run.U[:, 2:-2, 2:-2, 2:-2].sum(axis=(1, 2, 3))
    np.testing.assert_allclose(sums, ref, rtol=1e-14, atol=1e-14)
