"""The network oracle (oracle/mlp.py) against finite differences and the
BF16 rounding rule (CPU only)."""
import numpy as np

from oracle import mlp


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-5, 65504.0], np.float32)
    r = mlp.bf16(x)
    # representable values stay, halfway cases go to the even mantissa
    assert r[0] == 1.0 and r[3] == -2.5
    assert r[1] == 1.0           # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: even -> 1
    assert r[2] == 1.0078125     # above halfway rounds up
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = mlp.init_params(2, out_scale=1.0).astype(np.float64)
    X = rng.normal(size=(3, 768))
    T = rng.normal(size=(3, 768)) * 0.1
    _, _, g = mlp.forward_backward(p, X, T, exact=True)
    offs = np.cumsum([0] + [o * i + o for i, o in zip(mlp.LAYER_IN, mlp.LAYER_OUT)])
    idx = [offs[l] + k for l in range(4) for k in (0, 17, offs[l + 1] - offs[l] - 1)]
    for i in idx:
        h = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp.forward_backward(pp, X, T, exact=True)[1] -
              mlp.forward_backward(pm, X, T, exact=True)[1]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_rounded_and_exact_agree_to_bf16_level():
    rng = np.random.default_rng(3)
    p = mlp.init_params(4)
    X = rng.normal(size=(8, 768)).astype(np.float32)
    T = rng.normal(size=(8, 768)).astype(np.float32)
    y1, l1, g1 = mlp.forward_backward(p, X, T)
    y2, l2, g2 = mlp.forward_backward(p, X, T, exact=True)
    assert np.linalg.norm(y1 - y2) / np.linalg.norm(y2) < 2e-2
    assert abs(l1 - l2) / l2 < 2e-2
    assert np.dot(g1, g2) / (np.linalg.norm(g1) * np.linalg.norm(g2)) > 0.995
