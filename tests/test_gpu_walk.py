"""The hill-climbing convex support on the GPU (fclg_tuning.support_walk).

Hulls above 32 vertices carry an edge graph built when shapes are set; one-lane
GJK / MPR groups climb it (Convex::findExtremeVertexViaNeighbours,
include/fcl/geometry/shape/convex-inl.h:201-283).  Checked against the
oracle running the same rule over qhull face lists, at the parity bar of
test_gpu_convex.check_parity, with every hull size forced onto one-lane
launches; plus the device-pointer shape path and the scan fallback.
"""
import functools

import numpy as np
import pytest

from fclg import workloads
from fclg.api import FCLG_REQ_BOOLEAN_ONLY, make_request
from test_gpu_convex import BAND, check_parity

pytestmark = pytest.mark.gpu


@pytest.fixture
def one_lane(gpu_ctx):
    keep = gpu_ctx.get_tuning()
    gpu_ctx.set_tuning(gjk_lanes_small=1, gjk_lanes_large=1, support_walk=True)
    yield gpu_ctx
    gpu_ctx.set_tuning(**keep)


@functools.lru_cache(maxsize=1)
def _batches():
    mixed = workloads.mixed(200_000, seed=workloads.SEED_BASE + 31)
    pareto = workloads.pareto(400_000, seed=workloads.SEED_BASE + 32)
    big = lambda b: np.nonzero(np.maximum(b.shapes["vert_count"][b.pairs["shape_a"]],
                                          b.shapes["vert_count"][b.pairs["shape_b"]]) > 32)[0][:20000]
    return [("mixed", mixed.subset(big(mixed))), ("pareto", pareto.subset(big(pareto))),
            ("arm", workloads.arm(150, seed=workloads.SEED_BASE + 33))]


@pytest.mark.parametrize("case", [0, 1, 2], ids=["mixed", "pareto", "arm"])
def test_walk_distance_vs_oracle_walk(one_lane, oracle_lib, case):
    name, b = _batches()[case]
    one_lane.set_batch(b)
    got = one_lane.distance(b.pairs)
    ref = oracle_lib.signed_distance(b, walk=oracle_lib.walk_tables(b))
    st = check_parity(got, ref, b)
    assert st["n"] == b.n_pairs


def test_walk_and_scan_agree(one_lane, oracle_lib):
    """Walk on and off on the GPU against the oracle's walk and scan: both
    sides pass the parity bar, and the two GPU answers are the same query."""
    _, b = _batches()[2]
    one_lane.set_batch(b)
    walk = one_lane.distance(b.pairs)
    one_lane.set_tuning(support_walk=False)
    scan = one_lane.distance(b.pairs)
    one_lane.set_tuning(support_walk=True)
    check_parity(scan, oracle_lib.signed_distance(b), b)
    check_parity(walk, oracle_lib.signed_distance(b, walk=oracle_lib.walk_tables(b)), b)
    both = (walk["ok"] == 1) & (scan["ok"] == 1)
    err = np.abs(walk["distance"][both].astype(np.float64) - scan["distance"][both])
    assert np.percentile(err, 99) <= 1e-5 and err.max() <= 1e-3


def test_walk_boolean_collide_vs_oracle(one_lane, oracle_lib):
    """fcl::collide's boolean request (MPR, then the GJK fallback) with the walk."""
    _, b = _batches()[0]
    one_lane.set_batch(b)
    got = one_lane.collide(b.pairs, make_request(flags=FCLG_REQ_BOOLEAN_ONLY))
    tables = oracle_lib.walk_tables(b)
    ref = oracle_lib.collide(b, walk=tables)
    sd = oracle_lib.signed_distance(b, walk=tables)
    outside = np.abs(sd["distance"]) > BAND
    assert np.sum((got["collide"] != ref["ok"]) & outside) == 0


def test_walk_blocks_from_device_shapes(one_lane):
    """fclg_set_shapes_device builds the same walk blocks as fclg_set_shapes:
    the answers are identical bit for bit."""
    torch = pytest.importorskip("torch")
    _, b = _batches()[1]
    one_lane.set_batch(b)
    host = one_lane.distance(b.pairs)
    ds = torch.from_numpy(np.ascontiguousarray(b.shapes).view(np.uint8)).cuda()
    dv = torch.from_numpy(np.ascontiguousarray(b.vertices, np.float32)).cuda()
    one_lane.set_shapes_device(ds, dv)
    dev = one_lane.distance(b.pairs)
    assert np.array_equal(host.view(np.uint8), dev.view(np.uint8))


def test_autotune_considers_the_walk(gpu_ctx):
    import torch
    from fclg.layout import RESULT_DTYPE
    keep = gpu_ctx.get_tuning()
    _, b = _batches()[2]
    gpu_ctx.set_batch(b)
    n = b.n_pairs
    dp = torch.from_numpy(np.ascontiguousarray(b.pairs).view(np.uint8)).cuda()
    dr = torch.zeros(n * RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    best, ms = gpu_ctx.autotune(dp.data_ptr(), n, dr.data_ptr())
    assert best["support_walk"] in (1, -1) and ms > 0
    gpu_ctx.set_tuning(**keep)


@pytest.mark.parametrize("workload,n", [("mixed", 200_000), ("pareto", 400_000), ("arm", 2000), ("plain_small", 4096)])
def test_refill_pass_equals_group_pass(gpu_ctx, workload, n):
    """gjk_refill (one lane per pair, lanes refilled as their pairs finish)
    restates the same GJK as gjk_pass<1>: distance answers identical bit for
    bit, at both lane layouts that use it, with and without bucketing."""
    keep = gpu_ctx.get_tuning()
    if workload == "arm":
        b = workloads.arm(n, seed=workloads.SEED_BASE + 41)
    else:
        b = getattr(workloads, workload)(n, seed=workloads.SEED_BASE + 42) if workload != "plain_small" else \
            workloads.plain_small(seed=workloads.SEED_BASE + 42)
    gpu_ctx.set_batch(b)
    try:
        for bucketing in (True, False):
            gpu_ctx.set_tuning(bucketing=bucketing, gjk_lanes_small=1, gjk_lanes_large=1, gjk_refill=False)
            group = gpu_ctx.distance(b.pairs)
            gpu_ctx.set_tuning(gjk_refill=True)
            refill = gpu_ctx.distance(b.pairs)
            assert np.array_equal(group.view(np.uint8), refill.view(np.uint8)), (workload, bucketing)
    finally:
        gpu_ctx.set_tuning(**keep)


def test_refill_collide_with_contact_equals_group_pass(gpu_ctx):
    """fcl::collide with penetration and without the closed-form solvers runs
    the refilling pass too (GJK, then EPA from its simplex)."""
    NO_ANALYTIC = 16
    keep = gpu_ctx.get_tuning()
    b = workloads.mixed(100_000, seed=workloads.SEED_BASE + 43)
    gpu_ctx.set_batch(b)
    try:
        gpu_ctx.set_tuning(gjk_lanes_small=1, gjk_lanes_large=1, gjk_refill=False)
        group = gpu_ctx.collide(b.pairs, make_request(flags=NO_ANALYTIC))
        gpu_ctx.set_tuning(gjk_refill=True)
        refill = gpu_ctx.collide(b.pairs, make_request(flags=NO_ANALYTIC))
        assert np.array_equal(group.view(np.uint8), refill.view(np.uint8))
    finally:
        gpu_ctx.set_tuning(**keep)
