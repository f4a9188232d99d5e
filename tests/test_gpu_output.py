"""Output path (tlq_output): the files the library writes, byte for byte
against the output oracle (the reference's `output`,
source/HydroCore.f90:253-395) applied to the UPrim tlq_download returns; the
write overlaps the steps queued after it."""
import numpy as np
import pytest

from oracle import output as oo
from tlaloque_gb300 import problems, tlq

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [tlq.PREC_FP64, tlq.PREC_MIXED])
def test_output_files_match_the_reference_writer(gpu_lib, tmp_path, precision):
    cfg, U0 = problems.wind_bubble(10)  # cooling: the plain form's UPrim(5) is the carried pressure
    cfg = tlq.Config(**{**cfg.__dict__, "nz": 11, "zr": cfg.zl + 11 * cfg.dz, "precision": precision})
    U0 = cfg.zeros()
    U0[0], U0[4] = 1.3 * problems.AMU, problems.KB * 2e4
    U1 = U0.copy(order="F")
    path = str(tmp_path) + "/"
    with tlq.Context(cfg) as ctx:
        ctx.borders(U1, 1)
        ctx.upload(U1)
        ctx.advance(3)
        for fmt, nout in ((tlq.OUT_BIN, 1), (tlq.OUT_DAT, 2), (tlq.OUT_VTK, 3)):
            ctx.output(fmt, path, nout)
            ctx.output_wait()
        _, W = ctx.state()
        # queued behind later steps: the snapshot is the state after them
        ctx.advance(2)
        ctx.output(tlq.OUT_BIN, path, 4)
        ctx.advance(3)  # runs while the copy and the write proceed
        ctx.output_wait()
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    got = lambda fmt, n: open(oo.file_name(fmt, path, n), "rb").read()
    assert got(tlq.OUT_BIN, 1) == oo.bin_bytes(W)
    assert got(tlq.OUT_DAT, 2) == oo.dat_bytes(W, nx, ny, nz, cfg.dx, cfg.dy, cfg.dz)
    assert got(tlq.OUT_VTK, 3) == oo.vtk_bytes(W, nx, ny, nz, cfg.xl, cfg.yl, cfg.zl, cfg.dx, cfg.dy, cfg.dz)
    # the 4th snapshot equals the state after 5 steps
    U2 = U0.copy(order="F")
    with tlq.Context(cfg) as ctx:
        ctx.borders(U2, 1)
        ctx.upload(U2)
        ctx.advance(5)
        _, W5 = ctx.state()
    assert got(tlq.OUT_BIN, 4) == oo.bin_bytes(W5)


def test_dat_output_rejects_the_out_of_array_bounds(gpu_lib, tmp_path):
    cfg = tlq.Config(nx=8, ny=8, nz=16, bc=(tlq.BC_PERIODIC,) * 6)
    with tlq.Context(cfg) as ctx:
        ctx.upload(cfg.zeros() + 1.0)
        with pytest.raises(tlq.TlqError):
            ctx.output(tlq.OUT_DAT, str(tmp_path) + "/", 0)
