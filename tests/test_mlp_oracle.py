"""CPU checks of the learned warm start's oracle (oracle/mlp_ref.py).

The backward pass is pinned against central finite differences of the exact
(unrounded) network; the BF16 rounding helper against known bit patterns.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mlp_ref  # noqa: E402


def random_params(seed=0, scale=0.5):
    rng = np.random.default_rng(seed)
    return rng.uniform(-scale, scale, mlp_ref.N_PARAMS)


def test_param_layout_matches_header():
    text = open(os.path.join(ROOT, "include", "alens_gpu.h")).read()
    assert f"#define ALENS_MLP_NUM_PARAMS {mlp_ref.N_PARAMS}" in text
    assert f"#define ALENS_MLP_NUM_FEATURES {mlp_ref.N_IN}" in text


def test_bf16_rounding_known_values():
    one = 1.0
    ulp = 2.0 ** -7  # BF16 spacing at 1
    assert mlp_ref.bf16(one) == one
    assert mlp_ref.bf16(one + ulp / 2) == one              # tie -> even (1.0)
    assert mlp_ref.bf16(one + 3 * ulp / 2) == one + 2 * ulp  # tie -> even
    assert mlp_ref.bf16(one + 0.51 * ulp) == one + ulp
    assert mlp_ref.bf16(-3.0) == -3.0
    assert mlp_ref.bf16(0.0) == 0.0
    x = np.random.default_rng(1).standard_normal(1000)
    r = mlp_ref.bf16(x)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8 + 1e-30)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = random_params(3)
    X = rng.standard_normal((37, mlp_ref.N_IN))
    t = rng.standard_normal(37)
    loss, g = mlp_ref.loss_and_grad(p, X, t, rounding=False)
    idx = np.concatenate([rng.choice(mlp_ref.N_PARAMS, 60, replace=False),
                          [mlp_ref.OFF_B1, mlp_ref.OFF_B2, mlp_ref.OFF_W3, mlp_ref.OFF_B3]])
    h = 1e-6
    for i in idx:
        pp = p.copy()
        pm = p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp_ref.loss_and_grad(pp, X, t, rounding=False)[0] -
              mlp_ref.loss_and_grad(pm, X, t, rounding=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_rounded_network_close_to_exact():
    rng = np.random.default_rng(5)
    p = random_params(5)
    X = rng.standard_normal((200, mlp_ref.N_IN))
    y0, _ = mlp_ref.forward(p, X, rounding=False)
    y1, _ = mlp_ref.forward(p, X, rounding=True)
    assert np.max(np.abs(y1 - y0)) <= 0.05 * np.max(np.abs(y0))
