"""CUDA-graph capture of a query (fclg_graph_*) and the launch-shape autotuner
(fclg_autotune) through the C ABI.

* A replayed graph gives the same bytes as the direct device query on the same
  pairs, also after the pair buffer is refilled between replays (same size).
* A graph goes stale when the context reallocates its scratch for a larger
  batch or its shapes are set again; launching it then fails with an error
  instead of touching freed memory.
* The autotuned launch shape answers like the default one: collision flags
  identical, distances within 1e-5 m for >= 99.9 % of pairs (lane counts change
  the support scan's order, hence FP32 rounding, not the algorithm).
"""
import numpy as np
import pytest

from fclg import workloads
from fclg.layout import RESULT_DTYPE

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def _dev(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).copy()).cuda()


def _direct(torch, ctx, d_pairs, n):
    d_res = torch.zeros(n * RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    ctx.distance_device(d_pairs.data_ptr(), n, d_res.data_ptr())
    torch.cuda.synchronize()
    return d_res.cpu().numpy().tobytes()


def test_graph_replay_matches_direct_query(torch):
    from fclg.api import Context, FclgError
    b = workloads.mixed(20000, seed=workloads.SEED_BASE + 501)
    ctx = Context(0)
    try:
        ctx.set_batch(b)
        n = b.n_pairs
        d_pairs = _dev(torch, b.pairs)
        d_res = torch.zeros(n * RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        g = ctx.graph(d_pairs.data_ptr(), n, d_res.data_ptr())
        for perm_seed in (None, 1, 2):
            pairs = b.pairs if perm_seed is None else b.pairs[np.random.default_rng(perm_seed).permutation(n)]
            d_pairs.copy_(_dev(torch, pairs))
            d_res.zero_()
            g.launch()
            torch.cuda.synchronize()
            got = d_res.cpu().numpy().tobytes()
            assert got == _direct(torch, ctx, _dev(torch, pairs), n)
        # setting the shapes again frees the old shape (and walk) buffers: stale
        ctx.set_batch(b)
        with pytest.raises(FclgError, match="stale"):
            g.launch()
        g.close()
        # a larger batch reallocates the scratch: a graph captured before it must refuse to run
        g = ctx.graph(d_pairs.data_ptr(), n, d_res.data_ptr())
        big = b.subset(np.concatenate([np.arange(n)] * 3))
        _direct(torch, ctx, _dev(torch, big.pairs), big.n_pairs)
        with pytest.raises(FclgError, match="stale"):
            g.launch()
        g.close()
    finally:
        ctx.close()


def test_autotune_keeps_answers(torch):
    from fclg.api import Context
    b = workloads.mixed(100000, seed=workloads.SEED_BASE + 503)
    ctx = Context(0)
    try:
        ctx.set_batch(b)
        n = b.n_pairs
        d_pairs = _dev(torch, b.pairs)
        base = np.frombuffer(_direct(torch, ctx, d_pairs, n), RESULT_DTYPE)
        d_res = torch.zeros(n * RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        best, ms = ctx.autotune(d_pairs.data_ptr(), n, d_res.data_ptr())
        assert ms > 0 and best["gjk_lanes_small"] in (1, 2, 4, 8) and best["gjk_lanes_large"] in (4, 8, 16)
        assert ctx.get_tuning() == best
        tuned = np.frombuffer(_direct(torch, ctx, d_pairs, n), RESULT_DTYPE)
        assert np.array_equal(base["collide"], tuned["collide"])
        err = np.abs(base["distance"].astype(np.float64) - tuned["distance"])
        assert np.mean(err <= 1e-5) >= 0.999
    finally:
        ctx.close()
