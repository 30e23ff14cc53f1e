"""CPU restatement of the warm-start direction model (test infrastructure:
the checker for the CUDA forward / backward kernels, never a product path).

The model is not part of the reference (mind-fcl's GJKSolver takes a single
fixed or cached guess, include/fcl/narrowphase/detail/gjk_solver-inl.h:1129);
its definition is the one in include/fclg.h.  Two modes:

* ``bf16=True`` follows the CUDA kernels' rounding points: features, weight
  copies, hidden activations and the back-propagated pre-activation
  gradients are rounded to BF16 (round to nearest even), products accumulate
  in FP32 or wider, pre-activations and the output stay FP32.
* ``bf16=False`` with float64 arrays is the exact model, used to pin the
  analytic backward pass against central finite differences.

Pinned by tests/test_mlp_oracle.py (finite differences); GPU parity in
tests/test_gpu_warmstart.py.
"""
import numpy as np

IN, H, OUT, EMB, POSE = 32, 256, 8, 16, 12


def offsets(n_classes):
    o = {}
    k = 0
    for name, size in (("W1", H * IN), ("b1", H), ("W2", H * H), ("b2", H), ("W3", H * H), ("b3", H),
                       ("W4", OUT * H), ("b4", OUT), ("E", EMB * n_classes)):
        o[name] = (k, size)
        k += size
    o["total"] = k
    return o


def unpack(params, n_classes):
    o = offsets(n_classes)
    assert len(params) == o["total"]
    shapes = {"W1": (H, IN), "b1": (H,), "W2": (H, H), "b2": (H,), "W3": (H, H), "b3": (H,), "W4": (OUT, H),
              "b4": (OUT,), "E": (n_classes, EMB)}
    return {k: params[o[k][0]:o[k][0] + o[k][1]].reshape(shapes[k]) for k in shapes}


def pack(d, n_classes):
    o = offsets(n_classes)
    out = np.zeros(o["total"], d["W1"].dtype)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4", "E"):
        out[o[k][0]:o[k][0] + o[k][1]] = d[k].ravel()
    return out


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


GELU_C = np.sqrt(2.0 / np.pi)
GELU_A = 0.044715


def gelu(x):
    """GELU, tanh form (Hendrycks & Gimpel, 2016)."""
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + GELU_A * x ** 3)))


def gelu_grad(x):
    t = np.tanh(GELU_C * (x + GELU_A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * x * x)


def _rnd(x, on, dt):
    return bf16(x) if on else np.asarray(x, dt)


def features(pairs, E, n_classes, on=True, dt=np.float32):
    cls = pairs["pair_class"].astype(np.int64)
    cls = np.where(cls < n_classes, cls, 0)
    X = np.zeros((len(pairs), IN), dt)
    X[:, :9] = pairs["rot"].reshape(-1, 9)
    X[:, 9:12] = pairs["trans"]
    X[:, 12:28] = _rnd(E, on, dt)[cls]
    return _rnd(X, on, dt), cls


def forward(params, pairs, n_classes, on=True):
    """Returns (y [n][3], cache)."""
    dt = np.float32 if on else np.float64
    p = {k: np.asarray(v, dt) for k, v in unpack(params, n_classes).items()}
    Wb = {k: _rnd(p[k], on, dt) for k in ("W1", "W2", "W3", "W4")}
    X0, cls = features(pairs, p["E"], n_classes, on, dt)
    acc = np.float64
    Z1 = (X0.astype(acc) @ Wb["W1"].T.astype(acc)).astype(dt) + p["b1"]
    A1 = _rnd(gelu(Z1.astype(acc)), on, dt)
    Z2 = (A1.astype(acc) @ Wb["W2"].T.astype(acc)).astype(dt) + p["b2"]
    A2 = _rnd(gelu(Z2.astype(acc)), on, dt)
    Z3 = (A2.astype(acc) @ Wb["W3"].T.astype(acc)).astype(dt) + p["b3"]
    A3 = _rnd(gelu(Z3.astype(acc)), on, dt)
    Y = (A3.astype(acc) @ Wb["W4"].T.astype(acc)).astype(dt) + p["b4"]
    cache = dict(p=p, Wb=Wb, X0=X0, cls=cls, Z1=Z1, A1=A1, Z2=Z2, A2=A2, Z3=Z3, A3=A3, Y=Y, dt=dt)
    return Y[:, :3], cache


def loss_only(params, pairs, labels, n_classes, on=False):
    y, _ = forward(params, pairs, n_classes, on)
    y = y.astype(np.float64)
    h = y / (np.linalg.norm(y, axis=1, keepdims=True) + 1e-12)
    return float(np.mean(1.0 - np.sum(h * labels, axis=1)))


def gradient(params, pairs, labels, n_classes, on=True):
    """Mean cosine loss 1 - <y/|y|, u> and its gradient (flat, the parameter layout)."""
    y, c = forward(params, pairs, n_classes, on)
    dt = c["dt"]
    acc = np.float64
    n = len(pairs)
    y = y.astype(acc)
    u = np.asarray(labels, acc)
    nr = np.linalg.norm(y, axis=1, keepdims=True) + 1e-12
    h = y / nr
    cs = np.sum(h * u, axis=1, keepdims=True)
    loss = float(np.mean(1.0 - cs))
    dY = np.zeros((n, OUT), acc)
    dY[:, :3] = -(u - cs * h) / nr / n
    dY = _rnd(dY.astype(dt), on, dt).astype(acc)
    g = {}
    g["W4"] = dY.T @ c["A3"].astype(acc)
    g["b4"] = dY.sum(0)
    dZ3 = _rnd(((dY @ c["Wb"]["W4"].astype(acc)) * gelu_grad(c["Z3"].astype(acc))).astype(dt), on, dt).astype(acc)
    g["W3"] = dZ3.T @ c["A2"].astype(acc)
    g["b3"] = dZ3.sum(0)
    dZ2 = _rnd(((dZ3 @ c["Wb"]["W3"].astype(acc)) * gelu_grad(c["Z2"].astype(acc))).astype(dt), on, dt).astype(acc)
    g["W2"] = dZ2.T @ c["A1"].astype(acc)
    g["b2"] = dZ2.sum(0)
    dZ1 = _rnd(((dZ2 @ c["Wb"]["W2"].astype(acc)) * gelu_grad(c["Z1"].astype(acc))).astype(dt), on, dt).astype(acc)
    g["W1"] = dZ1.T @ c["X0"].astype(acc)
    g["b1"] = dZ1.sum(0)
    dX0 = dZ1 @ c["Wb"]["W1"].astype(acc)
    dE = np.zeros((n_classes, EMB), acc)
    np.add.at(dE, c["cls"], dX0[:, 12:28])
    g["E"] = dE
    return loss, pack({k: np.asarray(v, np.float64) for k, v in g.items()}, n_classes)


def init_params(n_classes, seed=0):
    """A random parameter vector of the documented shape (zero padding kept)."""
    rng = np.random.default_rng(seed)
    d = {}
    s1, sh = 1 / np.sqrt(28), 1 / np.sqrt(H)
    d["W1"] = rng.uniform(-s1, s1, (H, IN))
    d["W1"][:, 28:] = 0
    d["b1"] = rng.uniform(-s1, s1, H)
    d["W2"] = rng.uniform(-sh, sh, (H, H))
    d["b2"] = rng.uniform(-sh, sh, H)
    d["W3"] = rng.uniform(-sh, sh, (H, H))
    d["b3"] = rng.uniform(-sh, sh, H)
    d["W4"] = np.zeros((OUT, H))
    d["W4"][:3] = rng.uniform(-sh, sh, (3, H))
    d["b4"] = np.zeros(OUT)
    d["b4"][:3] = rng.uniform(-sh, sh, 3)
    d["E"] = rng.uniform(-1, 1, (n_classes, EMB))
    return pack(d, n_classes)
