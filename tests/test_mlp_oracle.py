"""The warm-start model's CPU oracle (oracle/mlp.py) pinned on its own:
the analytic backward pass in exact float64 against central finite
differences, the BF16 rounding against known values, and the BF16-mode
gradient against the exact one."""
import numpy as np

from fclg import workloads
from oracle import mlp


def _batch(n, n_classes, seed):
    b = workloads.mixed(n, seed=seed)
    p = b.pairs.copy()
    p["pair_class"] = np.arange(n) % n_classes
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    return p, u


def test_bf16_rounding():
    x = np.array([1.0, 1 + 2 ** -9, 1 + 3 * 2 ** -9, 1 + 2 ** -8, 1 + 3 * 2 ** -8, -2.5, 3.0e-3], np.float32)
    r = mlp.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                              # below half an ulp (2^-7 at 1.0)
    assert r[2] == np.float32(1 + 2 ** -7)          # above half an ulp
    assert r[3] == 1.0                              # tie, to the even mantissa below
    assert r[4] == np.float32(1 + 2 ** -6)          # tie, to the even mantissa above
    assert r[5] == -2.5
    assert abs(r[6] - 3.0e-3) / 3.0e-3 < 2 ** -8
    assert (r.view(np.uint32) & 0xFFFF).max() == 0


def test_gradient_matches_finite_differences():
    nc = 3
    pairs, u = _batch(8, nc, 11)
    params = mlp.init_params(nc, seed=3)
    loss, g = mlp.gradient(params, pairs, u, nc, on=False)
    assert np.isclose(loss, mlp.loss_only(params, pairs, u, nc))
    o = mlp.offsets(nc)
    rng = np.random.default_rng(0)
    idx = []
    for name in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4", "E"):
        start, size = o[name]
        cand = np.arange(start, start + size)
        if name == "W1":
            cand = cand[(cand - start) % mlp.IN < 28]     # the zero-padding columns have zero gradient
        if name in ("W4", "b4"):
            cand = cand[(cand - start) // (mlp.H if name == "W4" else 1) < 3]
        idx += list(rng.choice(cand, min(6, len(cand)), replace=False))
    eps = 1e-6
    for i in idx:
        pp, pm = params.copy(), params.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (mlp.loss_only(pp, pairs, u, nc) - mlp.loss_only(pm, pairs, u, nc)) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (i, fd, g[i])


def test_bf16_gradient_close_to_exact():
    nc = 4
    pairs, u = _batch(256, nc, 12)
    params = mlp.init_params(nc, seed=4)
    _, g64 = mlp.gradient(params, pairs, u, nc, on=False)
    _, g16 = mlp.gradient(params, pairs, u, nc, on=True)
    cos = g64 @ g16 / (np.linalg.norm(g64) * np.linalg.norm(g16))
    assert cos > 0.99
