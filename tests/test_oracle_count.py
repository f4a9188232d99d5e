"""The FP64 operation count of the reference algorithm: the oracle's source
compiled with a counting double (oracle/tlq_oracle_count.cpp).  The counting
build must compute exactly the oracle's numbers; then its counts per
zone-update are the algorithmic flops of the step.  CPU only."""
import numpy as np
import pytest

from oracle.oracle import Run, count_flops
from tests.helpers import oracle_params
from tlaloque_gb300 import problems

pytestmark = pytest.mark.timeout(600)


@pytest.mark.parametrize("name", ["sod", "sedov", "wind"])
def test_counting_build_is_the_oracle(name):
    """Same state after a few steps, bit for bit, and counts that grow with
    the work (positive in every category the problem uses)."""
    if name == "sod":
        cfg, U0 = problems.sod_tube(64)
    elif name == "sedov":
        cfg, U0 = problems.sedov(16)
    else:
        cfg, U0 = problems.wind_bubble(16)
    steps = 4
    ref = Run(oracle_params(cfg, nthreads=1), U0)
    ref.run(steps)
    counts, got = count_flops(oracle_params(cfg), U0, steps)
    assert counts["steps"] == steps == ref.it
    np.testing.assert_array_equal(got.U, ref.U)
    assert got.t == ref.t and got.dt == ref.dt
    zu = cfg.nx * cfg.ny * cfg.nz * steps
    for k in ("add", "mul", "div", "sqrt", "cmp"):
        assert counts[k] > zu, k
    if name == "wind":
        assert counts["trans"] > 0  # cooling's exp/log10/pow
    # per zone-update: hundreds of adds and multiplies, tens of divisions
    assert 100 < counts["add"] / zu < 5000 and 100 < counts["mul"] / zu < 5000
    assert 5 < counts["div"] / zu < 500
