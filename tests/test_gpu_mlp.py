"""The tensor-core MLP through the C ABI against the CPU oracle."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch

    assert torch.cuda.is_available()
    return torch


def case(n, seed=0):
    rng = np.random.default_rng(seed)
    features = rng.normal(0.3, 1.5, (n, M.IN)).astype(np.float32)
    targets = rng.normal(0.0, 2.0, (n, M.OUT)).astype(np.float32)
    mean = rng.normal(0.3, 0.1, M.IN).astype(np.float32)
    std = rng.uniform(1.0, 2.0, M.IN).astype(np.float32)
    scale = np.array([1.5, 2.0, 2.5], np.float32)
    return features, targets, mean, std, scale


@pytest.mark.parametrize("n", [1, 127, 128, 129, 1000, 70000])
def test_forward_matches_oracle(native, torch_cuda, n):
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    torch = torch_cuda
    f, _, mean, std, scale = case(n, seed=n)
    with MlpGpu(seed=3) as mlp:
        params = mlp.params()
        params[M.B1:M.W2] = np.linspace(-0.2, 0.2, M.HIDDEN)  # nonzero biases are exercised too
        params[M.B3:] = [0.1, -0.2, 0.3]
        mlp.set_params(params)
        mlp.set_normalisation(mean, std, scale)
        d_f = torch.from_numpy(f).cuda()
        d_out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()  # torch's copies and fill finish before the library's stream reads them
        mlp.forward(d_f.data_ptr(), n, d_out.data_ptr())
        got = d_out.cpu().numpy()
    y, _ = M.forward(params, f, mean, std, scale)
    want = y * scale
    assert np.all(got[:, 3] == 0.0)
    # BF16 activations: a one-ulp difference before rounding can move a BF16
    # value by 2^-8 relative, so compare against the output's own scale.
    err = np.abs(got[:, :3] - want)
    assert err.max() <= 2e-2 * max(1.0, np.abs(want).max()), err.max()
    assert np.median(err) <= 2e-3 * max(1.0, np.abs(want).max())


def test_gradients_match_oracle(native, torch_cuda):
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    torch = torch_cuda
    n = 4096
    f, t, mean, std, scale = case(n, seed=11)
    # Targets well away from the untrained output keep the batch sums of the
    # weight gradients coherent (random targets make them cancel, and the
    # small remainder amplifies BF16 rounding differences).
    t = (scale * (4.0 + 0.5 * np.tanh(f[:, :3]))).astype(np.float32)
    with MlpGpu(seed=5) as mlp:
        mlp.set_normalisation(mean, std, scale)
        params = mlp.params()
        d_f = torch.from_numpy(f).cuda()  # kept alive while the library reads them
        d_t = torch.from_numpy(t).cuda()
        torch.cuda.synchronize()
        loss, g = mlp.gradients(d_f.data_ptr(), d_t.data_ptr(), n)
    ref_loss, ref_g = M.loss_and_grad(params, f, t, mean, std, scale)
    assert loss == pytest.approx(ref_loss, rel=5e-3)
    # The oracle rounds to BF16 where the GPU does; the remaining difference
    # is FP32 accumulation against double.
    typical = np.abs(ref_g).max()
    worst = max(M.relative_error(a, b, typical) for a, b in zip(g, ref_g))
    assert worst < 1e-2, worst
    report = []
    for lo, hi in ((M.W1, M.B1), (M.B1, M.W2), (M.W2, M.B2), (M.B2, M.W3), (M.W3, M.B3), (M.B3, M.PARAMS)):
        a, b = g[lo:hi].astype(np.float64), ref_g[lo:hi]
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))
        report.append((lo, round(rel, 5), round(cos, 6)))
    print("per-tensor gradient agreement (offset, rel L2, cosine):", report)
    for lo, rel, cos in report:
        assert rel < 1e-3 and cos > 0.99999, report


def test_train_step_is_adam_on_the_gradient(native, torch_cuda):
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    torch = torch_cuda
    n = 2048
    f, t, mean, std, scale = case(n, seed=21)
    with MlpGpu(seed=7) as mlp:
        mlp.set_normalisation(mean, std, scale)
        p0 = mlp.params()
        d_f = torch.from_numpy(f).cuda()
        d_t = torch.from_numpy(t).cuda()
        torch.cuda.synchronize()
        _, g = mlp.gradients(d_f.data_ptr(), d_t.data_ptr(), n)
        mlp.train_step(d_f.data_ptr(), d_t.data_ptr(), n, lr=1e-3)
        p1 = mlp.params()
    want = M.adam_step(p0.copy(), g, np.zeros(M.PARAMS, np.float32), np.zeros(M.PARAMS, np.float32), 1, 1e-3)
    np.testing.assert_allclose(p1, want, rtol=0, atol=1e-6)


def test_training_fits_a_smooth_target(native, torch_cuda):
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    torch = torch_cuda
    rng = np.random.default_rng(9)
    n = 65536
    f = rng.normal(0, 1, (n, M.IN)).astype(np.float32)
    t = np.stack([np.tanh(f[:, 0] + 0.5 * f[:, 1]), f[:, 2] * f[:, 3] * 0.5, np.sin(f[:, 4])], 1).astype(np.float32)
    with MlpGpu(seed=1) as mlp:
        mlp.set_normalisation(np.zeros(M.IN), np.ones(M.IN), np.ones(M.OUT))
        d_f = torch.from_numpy(f).cuda()
        d_t = torch.from_numpy(t).cuda()
        torch.cuda.synchronize()
        first = mlp.train_step(d_f.data_ptr(), d_t.data_ptr(), n, lr=1e-3)
        for _ in range(300):
            last = mlp.train_step(d_f.data_ptr(), d_t.data_ptr(), n, lr=1e-3)
    assert last < 0.1 * first, (first, last)


def test_forward_erf_is_within_its_published_bound(native):
    """The forward pass evaluates GELU's erf by Abramowitz & Stegun 7.1.28
    (absolute error 3e-7) with one approximate reciprocal; in FP32 the 16th
    power scales the polynomial's rounding, and a float32 evaluation of the
    same steps stays under 1.8e-6 against the exact erf. Against erff the
    GPU must stay below 2.5e-6, three orders under the BF16 rounding the
    activation gets next."""
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    with MlpGpu() as mlp:
        assert mlp.selftest_erf() < 2.5e-6
