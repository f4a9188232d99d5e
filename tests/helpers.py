"""Shared test helpers: mirror a package Config into oracle Params, compare
arrays on the cells the scheme defines."""
import numpy as np

from oracle.oracle import Params, params_from_config


def oracle_params(cfg, nthreads: int = 0) -> Params:
    return params_from_config(cfg, nthreads)


def interior(a):
    return a[:, 2:-2, 2:-2, 2:-2]


def face_ghost_mask(cfg):
    """Cells the step defines: the interior and the first ghost layer of each
    face (transverse indices interior)."""
    m = np.zeros(cfg.shape[1:], bool)
    m[2:-2, 2:-2, 2:-2] = True
    m[1, 2:-2, 2:-2] = m[-2, 2:-2, 2:-2] = True
    m[2:-2, 1, 2:-2] = m[2:-2, -2, 2:-2] = True
    m[2:-2, 2:-2, 1] = m[2:-2, 2:-2, -2] = True
    return m


def rel_l1(a, b):
    """Relative L1 difference per conserved variable over the given cells."""
    return np.array([np.sum(np.abs(a[e] - b[e])) / max(np.sum(np.abs(b[e])), 1e-300) for e in range(a.shape[0])])
