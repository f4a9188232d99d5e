"""The cooling surrogate's CPU oracle (oracle/mlp_oracle.py) pinned on its
own: BF16 rounding against known bit patterns, and the FP64 network's
backward pass against central finite differences of its forward pass."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-30], dtype=np.float32)
    r = mo.bf16(x)
    # 1 + 2^-8 is a tie: rounds to even (1.0); 1 + 3*2^-8 ties up to 1 + 2^-6
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == 1.0 + 2 ** -6
    assert r[4] == -2.5
    assert abs(r[5] - 3.0e-30) <= 3.0e-30 * 2 ** -8


def test_fp64_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    P = mo.init_params(1).astype(np.float64)
    P[mo.OFF_B1:mo.OFF_W2] = 0.1 * rng.standard_normal(mo.HID)
    X = rng.uniform(-1, 1, (37, 3))
    Y = rng.uniform(0, 2, 37)
    loss, g = mo.loss_grad(P, X, Y, bf16_round=False)
    idx = np.concatenate([rng.choice(np.arange(a, b), 6, replace=False) for a, b in
                          [(mo.OFF_W1, mo.OFF_B1), (mo.OFF_B1, mo.OFF_W2), (mo.OFF_W2, mo.OFF_B2),
                           (mo.OFF_B2, mo.OFF_W3), (mo.OFF_W3, mo.OFF_B3), (mo.OFF_B3, mo.OFF_W4),
                           (mo.OFF_W4, mo.OFF_B4)]] + [[mo.OFF_B4]])
    h = 1e-6
    for q in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[q] += h
        Pm[q] -= h
        fd = (mo.loss_grad(Pp, X, Y, False)[0] - mo.loss_grad(Pm, X, Y, False)[0]) / (2 * h)
        assert abs(fd - g[q]) <= 1e-6 * max(1.0, abs(g[q])), (q, fd, g[q])
    assert loss > 0


def test_bf16_network_close_to_fp64():
    rng = np.random.default_rng(4)
    P = mo.init_params(2)
    X = rng.uniform(-1, 1, (200, 3))
    y64, _ = mo.forward(P, X, bf16_round=False)
    y16, _ = mo.forward(P, X, bf16_round=True)
    assert np.max(np.abs(y16 - y64)) < 0.05 * np.max(np.abs(y64))
