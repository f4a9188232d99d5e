"""The oracle's self-gravity (MultiGrid, source/sources.f90:99-787) against
physics it must reproduce: the potential of a uniform sphere with the
multipole boundary values, convergence of the V-cycles, and the zero-boundary
build's ghosts.  CPU only."""
import numpy as np
import pytest

from oracle.oracle import GBC_MULTIPOLE, GBC_ZERO, Oracle, Params, Run, count_flops
from tests.helpers import oracle_params
from tlaloque_gb300 import problems

pytestmark = pytest.mark.timeout(600)

PC = 3.085677588e18
G = 6.67430e-8


def sphere(n, bc, rho0=1e-21, bg=0.0, R=1.6 * PC, L=4 * PC):
    p = Params(nx=n, ny=n, nz=n, xl=-L, xr=L, yl=-L, yr=L, zl=-L, zr=L, self_gravity=1, grav_bc=bc)
    U = p.zeros()
    dx = 2 * L / n
    c = -L + dx * (np.arange(-1, n + 3) - 0.5)
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    r = np.sqrt(X * X + Y * Y + Z * Z)
    U[0] = np.where(r < R, rho0, bg)
    M = np.sum(np.where(r[2:-2, 2:-2, 2:-2] < R, rho0 - bg, 0.0)) * dx ** 3
    rc = r[1:-1, 1:-1, 1:-1]
    exact = np.where(rc < R, -G * M * (3 * R * R - rc * rc) / (2 * R ** 3), -G * M / rc)
    return p, U, rc, exact, R


def test_uniform_sphere_potential_converges():
    """Multipole faces: the solution approaches the analytic potential as the
    mesh refines, the faces carry -GM/r, and a second call from the converged
    potential changes it by round-off only."""
    errs = []
    for n in (16, 32, 64):
        p, U, r, exact, R = sphere(n, GBC_MULTIPOLE)
        o = Oracle(p)
        phi = np.zeros(p.phi_shape, order="F")
        cycles = o.multigrid(U, phi, 0)
        assert 2 <= cycles < 31
        inner = r < 0.5 * R
        errs.append(np.abs(phi - exact)[inner].max() / np.abs(exact).max())
        face = phi[0, 1:-1, 1:-1]
        assert np.abs(face - exact[0, 1:-1, 1:-1]).max() / np.abs(exact[0, 1:-1, 1:-1]).max() < 2e-3
        phi2 = phi.copy()
        o.multigrid(U, phi2, 1)  # it % 10 != 0: the faces stay
        assert np.abs(phi2 - phi).max() <= 1e-10 * np.abs(phi).max()
    assert errs[0] > errs[1] > errs[2] and errs[2] < 0.02


def test_zero_build_keeps_face_ghosts():
    """The serial build imposes nothing: the level-0 face ghosts keep their
    values (zero) and the potential is the Dirichlet-zero solution, shallower
    than the isolated one."""
    p, U, r, exact, R = sphere(32, GBC_ZERO)
    phi = np.zeros(p.phi_shape, order="F")
    Oracle(p).multigrid(U, phi, 0)
    assert np.all(phi[0] == 0.0) and np.all(phi[-1] == 0.0) and np.all(phi[:, 0] == 0.0)
    assert np.all(phi[:, :, -1] == 0.0)
    assert phi.min() < 0.0 and phi.min() > exact.min()


def test_self_gravity_run_conserves_mass_and_collapses():
    """A few steps of the gravitating cloud: with reflective walls the mass
    stays put (to 1e-8: the viscosity step takes U's ghost values from UP,
    HydroCore.f90:195-206, so its Laplacian is not exactly flux-free) and the
    cloud starts falling inward."""
    cfg, U0 = problems.gravitating_cloud(32)
    cfg.bc = (2,) * 6
    r = Run(oracle_params(cfg), U0)
    m0 = r.U[0, 2:-2, 2:-2, 2:-2].sum()
    r.run(20)
    U = r.U
    assert abs(U[0, 2:-2, 2:-2, 2:-2].sum() - m0) <= 1e-8 * m0
    n = cfg.nx
    # x momentum left of the centre points right (+), right of it left (-)
    assert U[1, 2 + n // 4, 2 + n // 2, 2 + n // 2] > 0.0 > U[1, 2 + 3 * n // 4, 2 + n // 2, 2 + n // 2]


def test_counting_build_with_self_gravity():
    cfg, U0 = problems.gravitating_cloud(16)
    ref = Run(oracle_params(cfg, nthreads=1), U0)
    ref.run(3)
    counts, got = count_flops(oracle_params(cfg), U0, 3)
    np.testing.assert_array_equal(got.U, ref.U)
    np.testing.assert_array_equal(got.arrays["PHIG"], ref.arrays["PHIG"])
    assert counts["trans"] > 0  # the moments' acos/atan2/cos/sin
