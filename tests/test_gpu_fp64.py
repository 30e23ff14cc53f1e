"""The FP64 separation distance (fclg_distance64: GJKSolver<double>::shapeDistance,
gjk_solver-inl.h:760-798) on the GPU against the reference.

Bar: on every golden case (outputs of the reference itself, tests/golden/),
each pair the reference solved as separated with a valid witness gets
ok = 1 and distance and witness points within 1e-9 m of the reference's;
each pair GJK found overlapping gets collide = 1, ok = 0, distance -1.  The
kernel runs the reference's operations in the reference's order with
round-to-nearest FP64 and no fused multiply-add, so the distances come out
bit-equal to the reference's, which is asserted.
"""
import os

import numpy as np
import pytest

from fclg import workloads
from fclg.api import make_request64
from fclg.layout import GJK_INTERSECT, GJK_SEPARATED, RESULT64_DTYPE, gjk_status

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "convex_ref.npz")
TOL = 1e-9


def _golden(name):
    g = np.load(GOLDEN)
    return workloads.Batch(name, g[name + "/shapes"], g[name + "/vertices"], g[name + "/pairs"]), g


@pytest.mark.parametrize("name", ["plain_small", "mixed", "pareto", "capsule_pair"])
def test_distance64_matches_reference(gpu_ctx, name):
    batch, g = _golden(name)
    ref = g[name + "/signed_distance"]
    gpu_ctx.set_batch(batch)
    # the capsule pair is test_gjk2_distance.cpp:70-154, run there with GJK2(1000, 1e-7)
    req = make_request64(1e-7, 1000) if name == "capsule_pair" else None
    got = gpu_ctx.distance64(batch.pairs, req)
    assert got.dtype == RESULT64_DTYPE
    rs = gjk_status(ref["gjk_status"])
    sep = (rs == GJK_SEPARATED) & (ref["ok"] == 1)
    ov = rs == GJK_INTERSECT
    assert np.all(got["ok"][sep] == 1)
    assert np.all((got["status"][sep] & 0xFF) == GJK_SEPARATED)
    err = np.abs(got["distance"][sep] - ref["distance"][sep])
    assert err.max(initial=0.0) <= TOL, "max |d64 - ref| = %.3g" % err.max()
    for a, b in (("p_a", "p0"), ("p_b", "p1")):
        e = np.abs(got[a][sep] - ref[b][sep]).max(initial=0.0)
        assert e <= TOL, "%s: %.3g" % (a, e)
    # the same operations in the same order: the distances are the reference's, bit for bit
    assert np.array_equal(got["distance"][sep], ref["distance"][sep])
    assert np.all(got["collide"][ov] == 1)
    assert np.all(got["ok"][ov] == 0)
    assert np.all(got["distance"][ov] == -1.0)
    # GJK statuses agree pair for pair
    assert np.array_equal(got["status"] & 0xFF, rs)


def test_distance64_device_and_host_agree(gpu_ctx):
    import torch
    batch = workloads.plain_small()
    gpu_ctx.set_batch(batch)
    host = gpu_ctx.distance64(batch.pairs)
    dp = torch.from_numpy(batch.pairs.view(np.uint8).copy()).cuda()
    dr = torch.zeros(len(batch.pairs) * RESULT64_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    gpu_ctx.distance64_device(dp.data_ptr(), len(batch.pairs), dr.data_ptr())
    torch.cuda.synchronize()
    dev = dr.cpu().numpy().view(RESULT64_DTYPE)
    assert np.array_equal(host.view(np.uint8), dev.view(np.uint8))


def test_distance64_matches_oracle_full_plain(gpu_ctx, oracle_lib):
    """Every pair of the 16k-pair plain workload against the FP64 oracle's
    shapeSignedDistance on its separated pairs (same GJK, same guess)."""
    batch = workloads.plain_small()
    gpu_ctx.set_batch(batch)
    got = gpu_ctx.distance64(batch.pairs)
    ref = oracle_lib.signed_distance(batch)
    rs = gjk_status(ref["gjk_status"])
    sep = (rs == GJK_SEPARATED) & (ref["ok"] == 1)
    assert sep.mean() > 0.3
    assert np.abs(got["distance"][sep] - ref["distance"][sep]).max() <= TOL
    assert np.array_equal(got["status"] & 0xFF, rs)


def test_distance64_invalid_indices_and_empty(gpu_ctx):
    """Out-of-range shape indices give GJK_Failed, ok = 0, distance -1 (no
    fault); an empty batch is a no-op."""
    batch = workloads.plain_small(512)
    bad = batch.pairs.copy()
    bad["shape_a"][::5] = len(batch.shapes) + 3
    gpu_ctx.set_batch(batch)
    got = gpu_ctx.distance64(bad)
    sel = np.arange(len(bad)) % 5 == 0
    assert np.all((got["status"][sel] & 0xFF) == 4) and np.all(got["ok"][sel] == 0)
    assert np.all(got["distance"][sel] == -1.0)
    ref = gpu_ctx.distance64(batch.pairs)
    assert np.array_equal(got[~sel].view(np.uint8), ref[~sel].view(np.uint8))
    assert len(gpu_ctx.distance64(batch.pairs[:0])) == 0
