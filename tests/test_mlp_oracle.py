"""The MLP oracle on the CPU: its analytic backward against central finite
differences in double (tests/gradient_check.h pattern), its BF16 rounding
against torch's, and Adam's update rule."""
from __future__ import annotations

import numpy as np
import torch

from oracle import mlp_oracle as M


def random_case(n=64, seed=0):
    rng = np.random.default_rng(seed)
    params = np.zeros(M.PARAMS)
    params[M.W1:M.B1] = rng.normal(0, np.sqrt(2 / 32), M.HIDDEN * M.IN)
    params[M.B1:M.W2] = rng.normal(0, 0.1, M.HIDDEN)
    params[M.W2:M.B2] = rng.normal(0, np.sqrt(2 / 128), M.HIDDEN * M.HIDDEN)
    params[M.B2:M.W3] = rng.normal(0, 0.1, M.HIDDEN)
    params[M.W3:M.B3] = rng.normal(0, np.sqrt(2 / 128), M.OUT * M.HIDDEN)
    params[M.B3:] = rng.normal(0, 0.1, M.OUT)
    features = rng.normal(0.5, 2.0, (n, M.IN)).astype(np.float32)
    targets = rng.normal(0, 3.0, (n, M.OUT)).astype(np.float32)
    mean = np.full(M.IN, 0.5, np.float32)
    std = np.full(M.IN, 2.0, np.float32)
    scale = np.array([2.0, 3.0, 4.0], np.float32)
    return params, features, targets, mean, std, scale


def test_backward_matches_finite_differences():
    params, f, t, mean, std, scale = random_case()
    rng = np.random.default_rng(1)
    indices = list(rng.integers(0, M.PARAMS, 60))
    # Every tensor is probed (tests/gradient_check.h sweeps each tensor).
    indices += [M.W1, M.B1, M.W2 + 777, M.B2 + 5, M.W3 + 100, M.B3 + 2]
    assert M.finite_difference_check(params, f, t, mean, std, scale, indices) < 1e-6


def test_bf16_rounding_matches_torch():
    x = np.random.default_rng(2).normal(0, 10, 10000).astype(np.float32)
    x[:4] = [0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9]
    ours = M.bf16(x)
    theirs = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(ours.view(np.uint32), theirs.view(np.uint32))


def test_adam_rule():
    p = np.ones(4, np.float32)
    first = np.zeros(4, np.float32)
    second = np.zeros(4, np.float32)
    g = np.array([1.0, -2.0, 0.5, 0.0], np.float32)
    M.adam_step(p, g, first, second, step=1, lr=1e-3)
    # Step 1 with bias correction moves every nonzero-gradient entry by ~lr.
    np.testing.assert_allclose(p[:3], 1.0 - 1e-3 * np.sign(g[:3]), rtol=0, atol=1e-6)
    assert p[3] == 1.0
