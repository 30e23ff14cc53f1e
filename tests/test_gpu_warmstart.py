"""Learned GJK warm start on the GPU (fclg_warmstart_*).

* Forward: the training kernels against the CPU oracle (oracle/mlp.py, BF16
  rounding points): per pair |y - y_oracle| <= 2e-2 (|y_oracle| + 1e-2),
  median relative error <= 2e-3.  The two sides round the same FP32
  pre-activations to BF16 but sum in a different order, so a pre-activation
  within ~1e-6 of a rounding boundary may round the other way; the bound
  covers those.  The two inference kernels (tcgen05 and mma.sync) evaluate
  GELU with the hardware tanh.approx (relative error ~2^-11, a tenth of a
  BF16 step), which moves a few per cent of the activations by one BF16
  step: against the oracle their bound is 5e-2 / median 5e-3, against each
  other median 2e-3.
* Gradient: the GPU backward pass against the oracle's on the same batch:
  per parameter block ||g - g_oracle|| <= 2e-2 ||g_oracle||, loss within 1e-4.
* Training and the gain: a model trained on the GPU on plain-GJK directions
  of held-out arm configurations lowers the mean GJK iteration count of
  unseen configurations by >= 25 % against plain initialisation.
* Answers: a warm-started pair keeps its run only with a certified distance
  (the run's small-improvement stop waits for a duality gap <= 5e-6 m), so
  every warm separation lies within 1e-5 m of the exact distance (the FP64
  oracle run to a 1e-12 tolerance), over all pairs.  Against plain
  initialisation: validity and collision flags identical outside the 1e-6 m
  band, overlapping pairs bit-identical (they rerun from the plain
  direction); separations differ from the plain ones by at most the plain
  answer's own distance from the exact one (the reference's loop stops when
  one iteration improves the bound by less than the tolerance,
  gjk_distance.hpp:78-90, which on curved features leaves up to ~1e-3 m).
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


def test_forward_matches_oracle(torch):
    from fclg.api import WarmStart
    from oracle import mlp
    b = workloads.arm(8, seed=workloads.SEED_BASE + 301)  # 1792 pairs
    n = b.n_pairs
    ws = WarmStart(workloads.ARM_CLASSES, seed=5)
    params = ws.get_params()
    d_pairs = _dev(torch, b.pairs)
    ref, _ = mlp.forward(params, b.pairs, workloads.ARM_CLASSES, on=True)
    scale = np.linalg.norm(ref, axis=1) + 1e-2
    outs = {}
    for kind in ("tcgen05", "mma.sync", "training"):
        d_y = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
        if kind == "training":
            ws.forward(d_pairs.data_ptr(), n, d_y.data_ptr())
        else:
            ws.predict(d_pairs.data_ptr(), n, d_y.data_ptr(), normalize=False, mma_sync=kind == "mma.sync")
        ws.status()
        y = d_y.cpu().numpy().reshape(n, 3)
        outs[kind] = y
        rel = np.linalg.norm(y - ref, axis=1) / scale
        bound, med = (2e-2, 2e-3) if kind == "training" else (5e-2, 5e-3)
        assert rel.max() <= bound and np.median(rel) <= med, (kind, rel.max(), np.median(rel))
    rel = np.linalg.norm(outs["tcgen05"] - outs["mma.sync"], axis=1) / scale
    assert np.median(rel) <= 2e-3, np.median(rel)
    # a ragged batch (an odd number of 128-pair tiles, the last one partial)
    # gives each pair the same outputs, bit for bit
    m = n - 165
    d_y = torch.zeros(m * 3, dtype=torch.float32, device="cuda")
    ws.predict(d_pairs.data_ptr(), m, d_y.data_ptr(), normalize=False)
    ws.status()
    assert np.array_equal(d_y.cpu().numpy().reshape(m, 3), outs["tcgen05"][:m])
    # a batch of 70 copies (980 tiles of 128 pairs: every CTA runs several,
    # with the next tile's weights loading under the current one's
    # epilogues) gives every copy the same outputs, bit for bit
    big = np.tile(b.pairs, 70)
    d_big = _dev(torch, big)
    d_y = torch.zeros(len(big) * 3, dtype=torch.float32, device="cuda")
    ws.predict(d_big.data_ptr(), len(big), d_y.data_ptr(), normalize=False)
    ws.status()
    yb = d_y.cpu().numpy().reshape(70, n, 3)
    assert all(np.array_equal(yb[i], outs["tcgen05"]) for i in range(70))
    # normalised output is the unit direction of the raw one
    d_u = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    ws.predict(d_pairs.data_ptr(), n, d_u.data_ptr(), normalize=True)
    torch.cuda.synchronize()
    u = d_u.cpu().numpy().reshape(n, 3)
    assert np.allclose(np.linalg.norm(u, axis=1), 1.0, atol=1e-5)
    ws.close()


def test_gradient_matches_oracle(torch):
    from fclg.api import WarmStart
    from oracle import mlp
    b = workloads.arm(3, seed=workloads.SEED_BASE + 302)  # 672 pairs: ten 64-row tiles plus a ragged one
    n = b.n_pairs
    rng = np.random.default_rng(7)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    ws = WarmStart(workloads.ARM_CLASSES, seed=6)
    params = ws.get_params()
    d_pairs = _dev(torch, b.pairs)
    d_lab = torch.from_numpy(u.astype(np.float32)).cuda()
    loss, g = ws.gradient(d_pairs.data_ptr(), d_lab.data_ptr(), n)
    ref_loss, ref_g = mlp.gradient(params, b.pairs, u, workloads.ARM_CLASSES, on=True)
    assert abs(loss - ref_loss) <= 1e-4
    o = mlp.offsets(workloads.ARM_CLASSES)
    for name in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4", "E"):
        s, k = o[name]
        a, r = g[s:s + k].astype(np.float64), ref_g[s:s + k]
        assert np.linalg.norm(a - r) <= 2e-2 * np.linalg.norm(r) + 1e-9, name
    ws.close()


def _query(torch, ctx, d_pairs, n, flags):
    from fclg.api import make_request
    d_res = torch.zeros(n * RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    ctx.distance_device(d_pairs.data_ptr(), n, d_res.data_ptr(), make_request(flags=flags))
    torch.cuda.synchronize()
    return d_res.cpu().numpy().view(RESULT_DTYPE).copy()


def test_trained_model_cuts_iterations_and_keeps_answers(torch):
    from fclg.api import Context, FclgError, WarmStart, direction_labels
    WARM = 4  # FCLG_REQ_WARM_START
    ctx = Context(0)
    try:
        # training set: plain-GJK directions of held-out configurations
        train = workloads.arm(1200, seed=workloads.SEED_BASE + 303)  # 268,800 pairs
        ctx.set_batch(train)
        d_tr = _dev(torch, train.pairs)
        res = _query(torch, ctx, d_tr, train.n_pairs, 0)
        lab, ok = direction_labels(res)
        keep = np.nonzero(ok)[0]
        d_tr = _dev(torch, train.pairs[keep])
        d_lab = torch.from_numpy(lab[keep]).cuda()
        ws = WarmStart(workloads.ARM_CLASSES, seed=1)
        losses = ws.train(d_tr.data_ptr(), d_lab.data_ptr(), len(keep), epochs=6, batch=4096, lr=2e-3)
        assert losses[-1] < 0.5 * losses[0], losses

        # unseen configurations
        test = workloads.arm(400, seed=workloads.SEED_BASE + 304)
        ctx.set_batch(test)
        d_te = _dev(torch, test.pairs)
        with pytest.raises(FclgError):
            _query(torch, ctx, d_te, test.n_pairs, WARM)  # no model set
        ctx.set_warmstart(ws)
        plain = _query(torch, ctx, d_te, test.n_pairs, 0)
        warm = _query(torch, ctx, d_te, test.n_pairs, WARM)

        assert np.array_equal(plain["ok"], warm["ok"])
        dp, dw = plain["distance"].astype(np.float64), warm["distance"].astype(np.float64)
        outside = np.abs(dp) > 1e-6
        assert np.array_equal((dp < 0)[outside], (dw < 0)[outside])
        ov = dp < 0
        # overlapping pairs rerun from the plain direction: same EPA answer
        assert np.array_equal(dp[ov], dw[ov])
        sep = ~ov & (plain["ok"] == 1)
        # every warm separation within 1e-5 m of the exact distance
        import oracle
        sub = np.arange(0, test.n_pairs, 4)
        exact = oracle.signed_distance(test.subset(sub), gjk_max_iter=1000, gjk_tol=1e-12)
        both = (exact["ok"] == 1) & sep[sub]
        assert both.mean() >= 0.9 * sep[sub].mean()
        ex = exact["distance"][both]
        e_warm = np.abs(dw[sub][both] - ex)
        e_plain = np.abs(dp[sub][both] - ex)
        print("warm vs exact: max %.3g, over 1e-5: %d of %d; plain vs exact: max %.3g, over 1e-5: %d"
              % (e_warm.max(), np.sum(e_warm > 1e-5), len(e_warm), e_plain.max(), np.sum(e_plain > 1e-5)))
        assert e_warm.max() <= 1e-5, e_warm.max()
        # warm and plain differ by no more than the plain answer's own error
        assert np.all(np.abs(dw[sub][both] - dp[sub][both]) <= e_plain + 1e-5)
        it_p = plain["iterations"][sep].astype(np.float64).mean()
        it_w = warm["iterations"][sep].astype(np.float64).mean()
        assert it_w <= 0.75 * it_p, (it_p, it_w)
        # the refilling GJK pass and the one-pass kernel (bucketing off) take the
        # same warm starts and answer bit for bit as the split launches
        # (bucketed: boolean, distance and redo launches)
        keep_t = ctx.get_tuning()
        ctx.set_tuning(bucketing=True, gjk_lanes_small=1, gjk_lanes_large=1, gjk_refill=False)
        w_group = _query(torch, ctx, d_te, test.n_pairs, WARM)
        ctx.set_tuning(gjk_refill=True)
        w_refill = _query(torch, ctx, d_te, test.n_pairs, WARM)
        ctx.set_tuning(bucketing=False, gjk_refill=False)
        w_one = _query(torch, ctx, d_te, test.n_pairs, WARM)
        ctx.set_tuning(**keep_t)
        assert np.array_equal(w_group.view(np.uint8), w_refill.view(np.uint8))
        assert np.array_equal(w_group.view(np.uint8), w_one.view(np.uint8))
        ctx.set_warmstart(None)
        ws.close()
    finally:
        ctx.close()


def test_learned_hints_seed_incremental_penetration(torch):
    """Incremental minimum-distance penetration seeded by the learned direction
    (FCLG_REQ_INCREMENTAL | FCLG_REQ_WARM_START): a model trained on the
    escape normals of penetrating arm pairs predicts the hints on the device.
    The answers are the reference algorithm's from those hints (flags exact
    outside the 1e-6 m band; depth within 1e-5 m of the FP64 oracle's for
    >= 99 % of pairs valid on both sides), and the learned hints land at
    EPA's minimum depth more often than random unit hints do."""
    import oracle
    from fclg.api import (FCLG_REQ_INCREMENTAL, FCLG_STATUS_INCREMENTAL, Context, FclgError, WarmStart,
                          make_request)
    WARM = 4  # FCLG_REQ_WARM_START
    ctx = Context(0)
    try:
        train = workloads.arm(3000, seed=workloads.SEED_BASE + 311)  # 672,000 pairs
        ctx.set_batch(train)
        res = _query(torch, ctx, _dev(torch, train.pairs), train.n_pairs, 0)
        nrm = res["normal"].astype(np.float64)
        ln = np.linalg.norm(nrm, axis=1)
        keep = np.nonzero((res["ok"] == 1) & (res["distance"] < 0) & (np.abs(ln - 1) < 1e-3))[0]
        assert len(keep) > 5000
        d_tr = _dev(torch, train.pairs[keep])
        d_lab = torch.from_numpy((nrm[keep] / ln[keep, None]).astype(np.float32)).cuda()
        ws = WarmStart(workloads.ARM_CLASSES, seed=2)
        losses = ws.train(d_tr.data_ptr(), d_lab.data_ptr(), len(keep), epochs=40, batch=1024, lr=2e-3)
        assert losses[-1] < 0.5 * losses[0], losses

        test = workloads.arm(400, seed=workloads.SEED_BASE + 312)
        ctx.set_batch(test)
        inc = make_request(flags=FCLG_REQ_INCREMENTAL | WARM)
        with pytest.raises(FclgError):
            ctx.collide_directed(test.pairs, None, inc)  # no model set
        ctx.set_warmstart(ws)
        with pytest.raises(FclgError):
            ctx.collide_directed(test.pairs, None, make_request(flags=WARM))  # not incremental
        got = ctx.collide_directed(test.pairs, None, inc)
        d_te = _dev(torch, test.pairs)
        d_g = torch.zeros(test.n_pairs * 3, dtype=torch.float32, device="cuda")
        ws.predict(d_te.data_ptr(), test.n_pairs, d_g.data_ptr())
        torch.cuda.synchronize()
        hints = d_g.cpu().numpy().reshape(-1, 3)
        ref = oracle.collide_incremental(test, hints)
        sd = oracle.signed_distance(test)
        assert np.all((got["status"] & FCLG_STATUS_INCREMENTAL) != 0)
        outside = np.abs(sd["distance"]) > 1e-6
        assert np.sum((got["collide"] != ref["ok"]) & outside) == 0
        valid = lambda r: np.isin(r, (0, 4))
        gst = ((got["status"] >> 8) & 0xFF).astype(np.int64) - 1
        hit = (got["collide"] == 1) & (ref["ok"] == 1)
        both = hit & valid(gst) & valid(ref["epa_status"])
        assert both.sum() >= 0.97 * hit.sum() and hit.sum() > 500
        err = np.abs(got["distance"][both].astype(np.float64) - ref["distance"][both])
        assert np.mean(err <= 1e-5) >= 0.99

        # learned against random hints: how often the run ends at EPA's depth
        ov = both & (sd["epa_status"] == 1) & (sd["distance"] < 0)
        at_min = lambda r: np.mean(np.abs(-r["distance"][ov].astype(np.float64) + sd["distance"][ov]) <= 1e-4)
        rng = np.random.default_rng(13)
        u = rng.normal(size=(test.n_pairs, 3))
        u = (u / np.linalg.norm(u, axis=1, keepdims=True)).astype(np.float32)
        rnd = ctx.collide_directed(test.pairs, u, make_request(flags=FCLG_REQ_INCREMENTAL))
        assert at_min(got) > at_min(rnd), (at_min(got), at_min(rnd))
        ctx.set_warmstart(None)
        ws.close()
    finally:
        ctx.close()
