"""FP64 operations per zone-update of the reference algorithm, counted by the
oracle's counting build (measurement infrastructure, like the oracle).

    python -m oracle.flops_report [--wind-n 128] [--sedov-n 128]

Prints one JSON object: per configuration the counts per zone-update by
category (add, mul, div, sqrt, cmp, trans) and their sum without cmp (the
arithmetic flops).  The first step of each run is skipped (set-up effects:
the wind bubble's first step cools many more cells than later ones).
"""
from __future__ import annotations

import argparse
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from oracle.oracle import count_flops  # noqa: E402
from oracle.oracle import params_from_config as oracle_params  # noqa: E402
from tlaloque_gb300 import problems  # noqa: E402


def per_zone(cfg, U0, steps: int) -> dict:
    counts, run = count_flops(oracle_params(cfg), U0, steps, skip=1)
    zu = cfg.nx * cfg.ny * cfg.nz * counts.pop("steps")
    out = {k: round(v / zu, 2) for k, v in counts.items()}
    out["flops"] = round(sum(v for k, v in out.items() if k != "cmp"), 1)
    out["mesh"] = [cfg.nx, cfg.ny, cfg.nz]
    out["steps_counted"] = steps
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--wind-n", type=int, default=128)
    ap.add_argument("--sedov-n", type=int, default=128)
    ap.add_argument("--steps", type=int, default=1)
    a = ap.parse_args()
    rep = {}
    cfg, U0 = problems.sod_tube(256)
    rep["sod_256x4x4_hll"] = per_zone(cfg, U0, 4)
    cfg, U0 = problems.sedov(a.sedov_n)
    rep[f"sedov_{a.sedov_n}_hllc"] = per_zone(cfg, U0, a.steps)
    cfg, U0 = problems.wind_bubble(a.wind_n)
    rep[f"wind_bubble_{a.wind_n}_hllc_cooling_gravity"] = per_zone(cfg, U0, a.steps)
    print(json.dumps(rep, indent=1))


if __name__ == "__main__":
    main()
