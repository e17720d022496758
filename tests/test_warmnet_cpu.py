"""The warm-start network's CPU oracle checks itself: float64 analytic
gradients against central finite differences (CPU only)."""
import numpy as np

from oracle import warmnet_ref as W


def test_oracle_gradients_match_finite_differences():
    L, hidden = 16, 32
    rng = np.random.default_rng(3)
    params = W.init_params(L, hidden, seed=1).astype(np.float64)
    x = rng.uniform(0, 1, (2, 5, 4, L))
    t = rng.uniform(0, 1, (2, 5, 4, L))
    loss, g = W.gradients(params, x, t, L, hidden, bf16=False)
    idx = rng.choice(len(params), 40, replace=False)
    eps = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        y1, _ = W.forward(p1, x, L, hidden, bf16=False)
        y2, _ = W.forward(p2, x, L, hidden, bf16=False)
        l1 = np.mean((y1 - t) ** 2)
        l2 = np.mean((y2 - t) ** 2)
        num = (l1 - l2) / (2 * eps)
        assert abs(num - g[i]) <= 1e-6 * max(1.0, abs(num)) + 1e-9, (i, num, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    vals = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -2.5, 3.0e-3], np.float32)
    r = W.to_bf16(vals)
    assert r[0] == 1.0
    assert r[1] == 1.0            # exactly half an ulp above 1.0: ties to even
    assert r[2] == 1.0078125      # above the half: rounds up
    assert r[4] == -2.5
