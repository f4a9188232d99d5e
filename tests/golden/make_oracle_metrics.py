"""Record the oracle's own error metrics at the full test resolutions.

The reference publishes no error numbers; its "own error" on a test is what
its algorithm (here: the oracle restatement) scores on that test.  This
script runs the oracle (OpenMP, all cores) on

* the reference's diagonal Sod test at 150^3 (tests_utilities.jl:214-224),
  scored with utils_analisis.jl's metrics against sod_e1rpex.out;
* the 128^3 Sedov-Taylor blast, scored against the gamma = 5/3 similarity
  profile (sedov_solution_53.txt);
* the 256x4x4 Sod tube (HLL, gamma 1.4) against the exact Riemann solution;

and writes tests/golden/oracle_metrics.json.  The GPU tests reproduce these
numbers (same algorithm, same arithmetic).

Usage:  python tests/golden/make_oracle_metrics.py
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Run  # noqa: E402
from oracle.oracle import params_from_config as oracle_params  # noqa: E402
from tlaloque_gb300 import analysis, problems  # noqa: E402


def sod_metrics(cfg, W, golden):
    ref = golden["sod_e1rpex"]
    xex = ref[:, 0] - 0.25
    r, rho, vel, p, e = analysis.diagonal_profiles(cfg, W)
    out = {}
    for name, col, y in (("rho", 1, rho), ("p", 3, p), ("v", 2, vel), ("e", 4, e)):
        _, mape, rmspe, L1, L2, Linf = analysis.all_error_metrics(xex, ref[:, col], r, y)
        out[name] = {"MAPE": mape, "RMSPE": rmspe, "L1": L1, "L2": L2, "Linf": Linf}
    return out


def sedov_metrics(cfg, W, t, golden):
    Rs = problems.sedov_shock_radius(t, xi0=float(golden["sedov53_xi0"]))
    rc, prof = analysis.radial_profile(cfg, W[0, 2:-2, 2:-2, 2:-2], nbins=cfg.nx // 2, rmax=0.48)
    ok = np.isfinite(prof)
    exact = analysis.sedov_density(rc, t, golden["sedov53"])
    inner = ok & (rc < 1.2 * Rs)
    return {"t": t, "R_shock": Rs, "r_peak": float(rc[ok][np.argmax(prof[ok])]),
            "L1_rho": analysis.norm_L1(exact[inner], prof[inner]), "rho_peak": float(np.nanmax(prof))}


def main():
    golden = np.load(os.path.join(HERE, "reference_solutions.npz"))
    res = {}
    t0 = time.time()
    cfg, U0 = problems.sod_tube()
    run = Run(oracle_params(cfg), U0)
    run.run(10 ** 7, problems.SOD_TFIN)
    x = cfg.xl + cfg.dx * (np.arange(cfg.nx) + 0.5)
    rho_ex, u_ex, p_ex = analysis.sod_exact(x, run.t)
    res["sod_tube_256"] = {"t": run.t, "it": run.it, "L1_rho": analysis.norm_L1(rho_ex, run.UPrim[0, 2:-2, 4, 4]),
                           "L1_p": analysis.norm_L1(p_ex, run.UPrim[4, 2:-2, 4, 4])}
    print("sod tube", res["sod_tube_256"], time.time() - t0, flush=True)

    cfg, U0 = problems.diagonal_sod(150)
    run = Run(oracle_params(cfg), U0)
    run.run(10 ** 7, problems.DIAG_SOD_TFIN)
    res["diagonal_sod_150"] = {"t": run.t, "it": run.it, "metrics": sod_metrics(cfg, run.UPrim, golden)}
    print("diagonal sod", res["diagonal_sod_150"], time.time() - t0, flush=True)

    cfg, U0 = problems.sedov(128)
    run = Run(oracle_params(cfg), U0)
    run.run(10 ** 7, problems.SEDOV_TFIN)
    res["sedov_128"] = dict(it=run.it, **sedov_metrics(cfg, run.UPrim, run.t, golden))
    print("sedov", res["sedov_128"], time.time() - t0, flush=True)

    with open(os.path.join(HERE, "oracle_metrics.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
