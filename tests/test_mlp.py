"""The learned prefetcher's network: the CPU restatement (oracle) checked by
finite differences, and the GPU forward / backward / SGD kernels checked
against it."""
import numpy as np
import pytest

import oracle


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, oracle.MLP_IN)).astype(np.float32)
    y = rng.uniform(0, 1, n).astype(np.float32)
    p = (rng.standard_normal(oracle.MLP_PARAMS) * 0.3).astype(np.float32)
    return x, y, p


def test_oracle_gradient_finite_differences():
    x, y, p = _data(37, 1)
    _, g, _ = oracle.mlp_forward_backward(x, y, p)
    p64 = p.astype(np.float64)
    rng = np.random.default_rng(2)
    for k in rng.choice(len(p), 40, replace=False):
        e = np.zeros_like(p64)
        e[k] = 1e-6
        lp = oracle.mlp_forward_backward(x, y, p64 + e)[2]
        lm = oracle.mlp_forward_backward(x, y, p64 - e)[2]
        assert abs((lp - lm) / 2e-6 - g[k]) < 1e-6 + 1e-4 * abs(g[k])


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 31, 1112, 5000])
def test_gpu_forward_backward_matches_oracle(lt, require_gpu, n):
    x, y, p = _data(n, n)
    pred, grad, loss, _ = lt.mlp_check(x, y, p)
    wp, wg, wl = oracle.mlp_forward_backward(x, y, p)
    # FP32 kernels vs float64 reference
    np.testing.assert_allclose(pred, wp, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(grad, wg, rtol=2e-3, atol=1e-6 + 1e-4 * np.abs(wg).max())
    assert abs(loss - wl) <= 1e-4 * max(1.0, wl)


@pytest.mark.gpu
def test_gpu_sgd_step(lt, require_gpu):
    x, y, p = _data(500, 9)
    _, grad, _, newp = lt.mlp_check(x, y, p, lr=0.05, momentum=0.9)
    # fresh momentum: v = g, w -= lr * v
    np.testing.assert_allclose(newp, p - 0.05 * grad, rtol=1e-5, atol=1e-6)
    # repeated steps lower the loss
    q = p
    losses = []
    for _ in range(30):
        _, _, l, q = lt.mlp_check(x, y, q, lr=0.05, momentum=0.0)
        losses.append(l)
    assert losses[-1] < losses[0]
