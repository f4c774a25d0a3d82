"""The learned coarse step through the C ABI: with no correction it is the
plain substep bit for bit; features are finite; the committed network
beats the plain coarse step on held-out tanks; the training and fallback
pipeline runs end to end on a small set."""
from __future__ import annotations

import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import training as T
from computer_graphics_lab_00_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def same(a, b) -> bool:
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


@pytest.fixture(scope="module")
def small():
    return T.learned_tanks(tanks=4, particles=4096, seed=2)


@pytest.mark.parametrize("schedule", [0, 1])
def test_zero_correction_is_the_plain_step(native, oracle, small, schedule):
    a = T.load_tanks(small)
    b = T.load_tanks(small)
    a.set_tuning(schedule=schedule)
    a.run_learned(T.COARSE_DT, 3, None)
    b.run(T.COARSE_DT, 3)
    for t in range(small.counts.__len__()):
        pa, va = a.download(t)
        pb, vb = b.download(t)
        assert same(pa, pb) and same(va, vb), t
        op, ov = oracle.run_substeps(small.params[t], *small.initial_state(t), T.COARSE_DT, 3)
        assert same(pa, op) and same(va, ov), t
    a.close()
    b.close()


@pytest.mark.parametrize("tanks,particles,schedule", [(4, 4096, 1), (3, 5000, 0), (1, 65536 + 300, 2)])
def test_learned_step_correction_is_the_forward_pass(native, tanks, particles, schedule):
    """The learned step's own path (features written as BF16 input tiles,
    the warp-specialised forward pass with two tiles in flight per CTA) gives the correction
    the forward pass over the FP32 features gives, bit for bit, on counts
    with a partial last tile and an odd number of tiles."""
    import torch

    from computer_graphics_lab_00_gb300.learned import MlpGpu

    ts = T.learned_tanks(tanks=tanks, particles=particles, seed=5)
    s = T.load_tanks(ts)
    s.set_tuning(schedule=schedule)
    s.run(T.FINE_DT, 20)
    n = s.total_particles
    with MlpGpu() as mlp:
        T.load_model(mlp, T.WEIGHTS)
        f = torch.empty((n, 32), dtype=torch.float32, device="cuda")
        want = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        got = torch.full((n, 4), float("nan"), dtype=torch.float32, device="cuda")
        s.learned_features(T.COARSE_DT, f.data_ptr())
        s.synchronize()
        mlp.forward(f.data_ptr(), n, want.data_ptr())
        torch.cuda.synchronize()
        s.learned_correction(T.COARSE_DT, mlp, got.data_ptr())
        s.synchronize()
    w = want.cpu().numpy()[:, :3]
    g = got.cpu().numpy()[:, :3]
    assert np.isfinite(g).all() and np.abs(g).max() > 0
    assert same(g, w), int((g.view(np.uint32) != w.view(np.uint32)).sum())
    s.close()


def test_features_are_finite_and_plausible(native, small):
    import torch

    s = T.load_tanks(small)
    s.run(T.FINE_DT, 50)
    n = s.total_particles
    f = torch.empty((n, 32), dtype=torch.float32, device="cuda")
    before = [s.download(t) for t in range(len(small.counts))]
    s.learned_features(T.COARSE_DT, f.data_ptr())
    s.synchronize()
    for t in range(len(small.counts)):
        p, v = s.download(t)
        assert same(p, before[t][0]) and same(v, before[t][1])
    f = f.cpu().numpy()
    assert np.isfinite(f).all()
    pairs = f[:, 8] * 32
    assert 5 < np.median(pairs) < 60
    assert (f[:, 26:] >= 0).all() and (f[:, 26:] <= 4).all()
    s.close()


def test_features_do_not_depend_on_the_processing_order(native, small):
    """Sorted, Morton and Hilbert processing orders give the same feature bits."""
    import torch

    got = []
    for schedule in (0, 1, 2):
        s = T.load_tanks(small)
        s.set_tuning(schedule=schedule)
        s.run(T.FINE_DT, 20)
        f = torch.empty((s.total_particles, 32), dtype=torch.float32, device="cuda")
        s.learned_features(T.COARSE_DT, f.data_ptr())
        s.synchronize()
        got.append(f.cpu().numpy())
        s.close()
    assert same(got[0], got[1]) and same(got[0], got[2])


def test_pipeline_end_to_end(native, small, tmp_path):
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    feats, targs = T.generate(small, snapshots=4, duration=0.1)
    assert feats.shape == (4 * sum(small.counts), 32) and targs.shape == (4 * sum(small.counts), 3)
    with MlpGpu(seed=4) as mlp:
        rep = T.train(mlp, feats, targs, steps=60, batch=8192, lr=1e-3, log_every=20)
        assert rep["losses"][-1][1] < rep["losses"][0][1]
        T.save_model(mlp, tmp_path / "m.npz")
        with MlpGpu(seed=9) as other:
            T.load_model(other, tmp_path / "m.npz")
            assert np.array_equal(other.params(), mlp.params())
        cmp = T.compare_with_fine(small, mlp, duration=0.1, every=0.05)
        assert set(cmp) == {"learned", "plain"}
        fb = T.run_with_fallback(small, mlp, coarse_steps=12, check_every=4)
        assert fb["coarse_steps"] == 12 and fb["checks"] >= 1
        assert 0.0 <= fb["fallback_fraction"] <= 1.0


@pytest.mark.parametrize("particles", [32768, 8192])
def test_trained_correction_beats_the_plain_coarse_step(native, particles):
    """What the trained network gains over the method without it. On 16
    held-out tanks (dam breaks and drops of 32,768 particles, config 4's
    size, or of 8,192, the batched learned form's), from seeds used neither
    in training nor in choosing the output gain, over 2 s of simulated time:
    the learned coarse step (D = 1/240 s) has a smaller mean density error
    AND a smaller centre-of-mass drift against the plain fine run (1/1200 s)
    than the plain coarse step at the same D (each ratio below 1; the
    measured ratios are in the design notes)."""
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    held = T.learned_tanks(16, particles, seed=T.HELD_OUT_SEED)
    with MlpGpu() as mlp:
        T.load_model(mlp, T.WEIGHTS)
        cmp = T.compare_with_fine(held, mlp, duration=2.0, every=0.1)
    learned, plain = cmp["learned"], cmp["plain"]
    assert np.isfinite(learned["mean_density_error"]) and np.isfinite(learned["mean_com_drift_m"])
    assert learned["mean_density_error"] < plain["mean_density_error"], cmp
    assert learned["mean_com_drift_m"] < plain["mean_com_drift_m"], cmp


@pytest.mark.parametrize("axes", [7, 5, 0])
def test_net_force_free_axes_take_each_tank_mean_off_exactly(native, small, axes):
    """A model whose output is the constant (0.5, -0.25, 0.125) in every row
    (all weights zero; the last bias is the output, exactly representable in
    the 2^-24 fixed point of the tank sums). With all three axes net-force
    free each correction minus its tank's mean is +0, so the learned step is
    the plain substep bit for bit; with an axis kept, it is not."""
    from computer_graphics_lab_00_gb300.learned import PARAMS, MlpGpu

    with MlpGpu(seed=1) as mlp:
        params = np.zeros(PARAMS, np.float32)
        params[-3:] = [0.5, -0.25, 0.125]
        mlp.set_params(params)
        mlp.set_normalisation(np.zeros(32, np.float32), np.ones(32, np.float32), np.ones(3, np.float32))
        mlp.set_net_force_free(axes)
        a = T.load_tanks(small)
        b = T.load_tanks(small)
        a.run_learned(T.COARSE_DT, 2, mlp)
        b.run_learned(T.COARSE_DT, 2, None)
        equal = all(same(x, y) for t in range(len(small.counts)) for x, y in zip(a.download(t), b.download(t)))
        a.close()
        b.close()
    assert equal == (axes == 7)
