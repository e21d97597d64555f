"""The FP64 oracle of the closure network, pinned without a GPU: its
gradient against central differences, its BF16 rounding against torch's."""
import numpy as np
import torch

from oracle import mlp as M


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    v = np.concatenate([rng.normal(0, 1, 5000), rng.normal(0, 1e-3, 2000),
                        rng.normal(0, 1e4, 2000), [0.0, -0.0, 1.0, 1.00390625, 1.01171875]])
    want = torch.tensor(v, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(M.bf16(v), want)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = M.init_params(3)
    # biases off zero so their gradients are exercised
    p[M.OFF_B1:M.OFF_W2] = rng.normal(0, 0.1, M.NH)
    p[M.OFF_B2:M.OFF_W3] = rng.normal(0, 0.1, M.NH)
    x = rng.normal(0, 1, (7, M.NIN))
    t = rng.normal(0, 1, (7, M.NOUT))
    _, g = M.backward(p, x, t, emulate=False)
    idx = np.concatenate([rng.integers(M.OFF_W1, M.OFF_B1, 6), rng.integers(M.OFF_B1, M.OFF_W2, 3),
                          rng.integers(M.OFF_W2, M.OFF_B2, 6), rng.integers(M.OFF_B2, M.OFF_W3, 3),
                          rng.integers(M.OFF_W3, M.OFF_B3, 4), [M.OFF_B3, M.OFF_B3 + 1]])
    fd = M.finite_difference(p, x, t, idx)
    np.testing.assert_allclose(g[idx], fd, rtol=1e-5, atol=1e-9)


def test_emulated_gradient_is_close_to_exact():
    rng = np.random.default_rng(2)
    p = M.init_params(4)
    x = rng.normal(0, 1, (64, M.NIN))
    t = rng.normal(0, 1, (64, M.NOUT))
    _, g0 = M.backward(p, x, t, emulate=False)
    _, g1 = M.backward(p, x, t, emulate=True)
    assert np.linalg.norm(g1 - g0) / np.linalg.norm(g0) < 2e-2


def test_adam_first_step_moves_by_lr():
    p = np.zeros(5)
    g = np.array([1.0, -2.0, 0.5, 1e-3, -1e-3])
    p1, m, v = M.adam(p, g, np.zeros(5), np.zeros(5), 1, lr=0.01)
    np.testing.assert_allclose(p1, -0.01 * np.sign(g), rtol=1e-4)
