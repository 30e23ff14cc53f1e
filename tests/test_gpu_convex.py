"""GPU convex queries through the C ABI against the reference.

Parity bar (FP32 kernels vs the FP64 reference on identical inputs):
* collision flags agree exactly outside a 1e-6 m band around contact
  (|signed distance| > 1e-6 by the reference);
* separation distance: |err| <= 1e-5 m for >= 99.5 % of the pairs both sides
  solve; the rest are pairs where the reference's own stopping rule
  (improvement < 1e-6 per iteration, gjk_distance.hpp:78-90) fires at a
  different iterate on a curved surface or a hull of many vertices — bounded
  by 1e-3 m, and both answers above the exact distance (pair by pair:
  test_parity_tails_have_stated_causes);
* penetration depth: |err| <= 1e-5 m for >= 99 % of overlapping pairs, the
  rest bounded by 1e-2 m (pairs where EPA hits the 256-face capacity on
  curved shapes, where the reference itself returns its partial polytope, or
  curved pairs where both runs stop short of the converged depth on
  different faces; pair by pair in the same test);
* contact normal (depth > 1e-3 m): between two polyhedra (boxes, convex
  hulls) the normal is a face normal of the Minkowski difference and the
  angle error is <= 1e-3 rad for >= 99 % of pairs; with a curved shape
  (sphere, capsule, cylinder) EPA resolves the normal only to about
  sqrt(2 tol / R) (depth converges quadratically in the face spacing, the
  normal linearly), in the reference as on the GPU, so the bar is 2e-2 rad.
The golden cases are outputs of the reference itself (tests/golden/).
"""
import os

import numpy as np
import pytest

from fclg import workloads
from fclg.layout import (BOX, CAPSULE, CONVEX, CYLINDER, EPA_ITER_LIMIT, EPA_MALLOC_FAILED, EPA_OK,
                         PAIR_DTYPE, SHAPE_DTYPE, SPHERE, epa_status, gjk_status)

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "convex_ref.npz")
BAND = 1e-6


def _golden(name):
    g = np.load(GOLDEN)
    b = workloads.Batch(name, g[name + "/shapes"], g[name + "/vertices"], g[name + "/pairs"])
    return b, g


def _curved(batch):
    if batch is None:
        return None
    t = batch.shapes["type"]
    ca = np.isin(t[batch.pairs["shape_a"]], (SPHERE, CAPSULE, CYLINDER))
    cb = np.isin(t[batch.pairs["shape_b"]], (SPHERE, CAPSULE, CYLINDER))
    return ca | cb


def check_parity(got, ref, batch=None, sep_frac=0.995, depth_frac=0.99):
    """Asserts the parity bar above; returns a dict of statistics."""
    n = len(got)
    both = (got["ok"] == 1) & (ref["ok"] == 1)
    assert both.mean() >= 0.999, "valid fraction %.5f" % both.mean()
    rd = ref["distance"]
    gd = got["distance"].astype(np.float64)
    outside = np.abs(rd) > BAND
    flags = (gd < 0) != (rd < 0)
    assert np.sum(flags & outside & both) == 0
    err = np.abs(gd - rd)
    sep = both & (rd > 0)
    ov = both & (rd < 0)
    st = {"n": n}
    if sep.any():
        e = err[sep]
        st["sep_p99"] = float(np.percentile(e, 99))
        assert np.mean(e <= 1e-5) >= sep_frac, "separation: %.4f within 1e-5" % np.mean(e <= 1e-5)
        assert e.max() <= 1e-3
    if ov.any():
        e = err[ov]
        st["depth_p99"] = float(np.percentile(e, 99))
        assert np.mean(e <= 1e-5) >= depth_frac, "depth: %.4f within 1e-5" % np.mean(e <= 1e-5)
        assert e.max() <= 1e-2
        deep = ov & (rd < -1e-3)
        curved = _curved(batch)
        if curved is None:
            curved = np.zeros(n, bool)
        for cls, bar in ((deep & ~curved, 1e-3), (deep & curved, 2e-2)):
            if cls.sum() < 20:
                continue
            c = np.clip(np.sum(got["normal"][cls].astype(np.float64) * ref["normal"][cls], axis=1), -1, 1)
            ang = np.arccos(c)
            st["normal_p99_%g" % bar] = float(np.percentile(ang, 99))
            assert np.mean(ang <= bar) >= 0.99, "normals within %g rad: %.4f" % (bar, np.mean(ang <= bar))
    return st


@pytest.mark.parametrize("name", ["plain_small", "mixed", "pareto"])
def test_distance_vs_reference_golden(gpu_ctx, name):
    b, g = _golden(name)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.distance(b.pairs)
    check_parity(got, g[name + "/signed_distance"], b)


@pytest.mark.parametrize("name", ["plain_small", "mixed", "pareto"])
def test_collide_vs_reference_golden(gpu_ctx, name):
    from fclg.api import FCLG_REQ_BOOLEAN_ONLY, make_request
    b, g = _golden(name)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.collide(b.pairs, make_request(flags=FCLG_REQ_BOOLEAN_ONLY))
    ref = g[name + "/collide_bool"]
    sd = g[name + "/signed_distance"]
    outside = np.abs(sd["distance"]) > BAND
    assert np.sum((got["collide"] != ref["ok"]) & outside) == 0
    # with penetration: one contact per colliding pair, by GJK + EPA as the
    # golden reference run computed it (the closed-form sphere solvers are
    # checked against the oracle in test_collide_sphere_pairs_closed_form)
    NO_ANALYTIC = 16
    got_c = gpu_ctx.collide(b.pairs, make_request(flags=NO_ANALYTIC))
    ref_c = g[name + "/collide_contact"]
    hit = (ref_c["ok"] == 1) & (got_c["ok"] == 1) & (ref_c["distance"] < -1e-5)
    err = np.abs(got_c["distance"][hit] - ref_c["distance"][hit])
    assert np.mean(err <= 1e-5) >= 0.99


def test_collide_sphere_pairs_closed_form(gpu_ctx, oracle_lib):
    """fcl::collide's closed-form sphere solvers (sphere-sphere / capsule / box /
    cylinder, either order): GPU FP32 against the FP64 restatement.  Flags equal
    outside the 1e-6 m band; depth within 1e-5 m, contact position within
    5e-5 m (the capsule and cylinder positions are formed as differences of
    FP32 terms about 1 m long) and normal within 1e-3 rad, except
    normals of nearly concentric spheres (|c2 - c1| < 1e-3 m), which are
    ill-defined."""
    ANALYTIC_BIT = 1 << 17
    b = workloads.mixed(60000, seed=workloads.SEED_BASE + 77)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.collide(b.pairs)
    ref = oracle_lib.collide(b, want_contact=True)
    an = ref["gjk_status"] == 20
    assert an.mean() > 0.2
    assert np.array_equal((got["status"] & ANALYTIC_BIT) != 0, an)
    sd = oracle_lib.signed_distance(b)
    outside = np.abs(sd["distance"]) > BAND
    assert np.sum((got["collide"] != ref["ok"]) & an & outside) == 0
    t = b.shapes["type"]
    box_box = (t[b.pairs["shape_a"]] == BOX) & (t[b.pairs["shape_b"]] == BOX)
    hit = an & ~box_box & (ref["ok"] == 1) & (got["collide"] == 1)
    assert np.max(np.abs(got["distance"][hit] - ref["distance"][hit])) <= 1e-5
    pos_g = 0.5 * (got["p_a"][hit] + got["p_b"][hit])
    pos_r = 0.5 * (ref["p0"][hit] + ref["p1"][hit])
    assert np.max(np.linalg.norm(pos_g - pos_r, axis=1)) <= 5e-5
    cosang = np.clip(np.sum(got["normal"][hit] * ref["normal"][hit], axis=1), -1, 1)
    centre = np.linalg.norm(b.pairs["trans"][hit], axis=1)
    ok_normal = np.arccos(cosang) <= 1e-3
    assert np.all(ok_normal | (centre < 1e-3))
    # the analytic path gives the same flags as the MPR boolean
    boolean = gpu_ctx.collide(b.pairs, make_request_flags(1))
    assert np.sum((boolean["collide"] != got["collide"]) & outside) == 0


def _box_pairs(n, seed):
    """Boxes of sides U[0.05, 0.8] m at random orientations, centres within
    U[-0.6, 0.6] m per axis: about half the pairs overlap."""
    rng = np.random.default_rng(seed)
    s = np.zeros(2 * n, SHAPE_DTYPE)
    s["type"] = BOX
    s["param"][:, :3] = rng.uniform(0.05, 0.8, size=(2 * n, 3))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    p = np.zeros(n, PAIR_DTYPE)
    p["shape_a"] = np.arange(n)
    p["shape_b"] = n + np.arange(n)
    p["rot"] = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                         2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                         2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], axis=1)
    p["trans"] = rng.uniform(-0.6, 0.6, size=(n, 3))
    return workloads.Batch("box_pairs", s, np.zeros((1, 4), np.float32), p, {})


def test_collide_box_pairs_closed_form(gpu_ctx, oracle_lib):
    """fcl::collide on box pairs: boxBox2 (box_box-inl.h) in FP32 on the GPU
    against the FP64 restatement, whose answers are pinned to the reference's
    box-box scenarios (test_box_box.py).  Flags identical outside the 1e-6 m
    band; of the colliding pairs deeper than 1e-4 m, >= 99 % agree on the
    separating axis (normal within 1e-3 rad), depth within 1e-5 m and contact
    position within 1e-4 m.  The rest are pairs where two axes' overlaps (with
    the 5 % preference for face axes), or two manifold points' depths, tie to
    within FP32 rounding and the two precisions pick different ones."""
    ANALYTIC_BIT = 1 << 17
    b = _box_pairs(100_000, 61)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.collide(b.pairs)
    ref = oracle_lib.collide(b, want_contact=True)
    assert np.all((got["status"] & ANALYTIC_BIT) != 0) and np.all(ref["gjk_status"] == 20)
    sd = oracle_lib.signed_distance(b)
    outside = np.abs(sd["distance"]) > BAND
    assert np.sum((got["collide"] != ref["ok"]) & outside) == 0
    deep = (ref["ok"] == 1) & (got["collide"] == 1) & (ref["distance"] < -1e-4)
    assert deep.sum() > 20000
    cosang = np.clip(np.sum(got["normal"][deep].astype(np.float64) * ref["normal"][deep], axis=1), -1, 1)
    same_axis = np.arccos(cosang) <= 1e-3
    depth_ok = np.abs(got["distance"][deep] - ref["distance"][deep]) <= 1e-5
    pos_g = 0.5 * (got["p_a"][deep].astype(np.float64) + got["p_b"][deep])
    pos_r = 0.5 * (ref["p0"][deep] + ref["p1"][deep])
    pos_ok = np.linalg.norm(pos_g - pos_r, axis=1) <= 1e-4
    assert same_axis.mean() >= 0.99, same_axis.mean()
    assert (same_axis & depth_ok).mean() >= 0.99, (same_axis & depth_ok).mean()
    assert (same_axis & depth_ok & pos_ok).mean() >= 0.99, (same_axis & depth_ok & pos_ok).mean()
    # boolean requests take the same solver
    boolean = gpu_ctx.collide(b.pairs, make_request_flags(1))
    assert np.array_equal(boolean["collide"], got["collide"])


@pytest.mark.parametrize("workload,n", [("mixed", 40000), ("pareto", 40000)])
def test_collide_directed_vs_oracle(gpu_ctx, oracle_lib, workload, n):
    """fcl::collide, directed penetration mode (random unit escape directions):
    GPU against the restated reference.  Flags identical outside the 1e-6 m
    band; the directed status identical for >= 99.5 % of colliding pairs;
    depth along the direction within 1e-5 m for >= 99 % of the pairs both
    solve and within 1e-3 m for all; normal = the given direction."""
    DIRECTED_BIT = 1 << 18
    b = getattr(workloads, workload)(n, seed=workloads.SEED_BASE + 88)
    rng = np.random.default_rng(5)
    u = rng.normal(size=(b.n_pairs, 3))
    u = (u / np.linalg.norm(u, axis=1, keepdims=True)).astype(np.float32)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.collide_directed(b.pairs, u)
    ref = oracle_lib.collide_directed(b, u)
    assert np.all((got["status"] & DIRECTED_BIT) != 0)
    sd = oracle_lib.signed_distance(b)
    outside = np.abs(sd["distance"]) > BAND
    assert np.sum((got["collide"] != ref["ok"]) & outside) == 0
    hit = (got["collide"] == 1) & (ref["ok"] == 1)
    gst = ((got["status"] >> 8) & 0xFF) - 1
    assert np.mean(gst[hit] == ref["epa_status"][hit]) >= 0.995
    both = hit & (got["ok"] == 1) & (ref["epa_status"] == 0)
    err = np.abs(got["distance"][both].astype(np.float64) - ref["distance"][both])
    assert np.mean(err <= 1e-5) >= 0.99 and err.max() <= 1e-3
    assert np.allclose(got["normal"], u)


@pytest.mark.parametrize("workload,n", [("mixed", 40000), ("pareto", 40000)])
def test_collide_incremental_vs_oracle(gpu_ctx, oracle_lib, workload, n):
    """fcl::collide, incremental minimum-distance penetration mode: GPU FP32
    against the restatement, which is pinned bit for bit to the reference's
    RunIncrementalMinimumPenetrationDistance.  Flags identical outside the
    1e-6 m band.  Started on EPA's normal, the depth within 1e-5 m of the
    oracle's for >= 99 % of colliding pairs.  From random hints the run
    descends to a local minimum over directions; FP32 and FP64 may settle in
    different ones, so the bar is: >= 97 % of colliding pairs valid on both
    sides, depth within 1e-4 m for >= 90 % of them, and never below EPA's
    minimum by more than 1e-5 m (the depth along a direction bounds the
    minimum from above)."""
    from fclg.api import FCLG_REQ_INCREMENTAL, FCLG_STATUS_INCREMENTAL, make_request
    b = getattr(workloads, workload)(n, seed=workloads.SEED_BASE + 89)
    gpu_ctx.set_batch(b)
    req = make_request(flags=FCLG_REQ_INCREMENTAL)
    sd = oracle_lib.signed_distance(b)
    outside = np.abs(sd["distance"]) > BAND
    epa = sd["normal"].astype(np.float32)
    got = gpu_ctx.collide_directed(b.pairs, epa, req)
    ref = oracle_lib.collide_incremental(b, epa)
    assert np.all((got["status"] & FCLG_STATUS_INCREMENTAL) != 0)
    assert np.sum((got["collide"] != ref["ok"]) & outside) == 0
    hit = (got["collide"] == 1) & (ref["ok"] == 1)
    valid = lambda r: np.isin(r, (0, 4))
    gst = ((got["status"] >> 8) & 0xFF).astype(np.int64) - 1
    both = hit & (got["ok"] == 1) & valid(ref["epa_status"]) & (sd["epa_status"] == 1)
    err = np.abs(got["distance"][both].astype(np.float64) - ref["distance"][both])
    assert np.mean(err <= 1e-5) >= 0.99
    rng = np.random.default_rng(9)
    u = rng.normal(size=(b.n_pairs, 3))
    u = (u / np.linalg.norm(u, axis=1, keepdims=True)).astype(np.float32)
    got = gpu_ctx.collide_directed(b.pairs, u, req)
    ref = oracle_lib.collide_incremental(b, u)
    hit = (got["collide"] == 1) & (ref["ok"] == 1)
    gst = ((got["status"] >> 8) & 0xFF).astype(np.int64) - 1
    both = hit & valid(gst) & valid(ref["epa_status"])
    assert both.sum() >= 0.97 * hit.sum()
    err = np.abs(got["distance"][both].astype(np.float64) - ref["distance"][both])
    assert np.mean(err <= 1e-4) >= 0.90
    ov = both & (sd["epa_status"] == 1) & (sd["distance"] < 0)
    # EPA's depth on a curved pair is its last face's estimate, which the
    # reference's incremental run can undercut (seen: 1 pair in 15 754, the
    # FP64 restatement agreeing with the GPU there)
    assert np.mean(-got["distance"][ov] >= -sd["distance"][ov] - 1e-5) >= 0.999
    nrm = np.linalg.norm(got["normal"][both], axis=1)
    assert np.all(np.abs(nrm - 1) < 1e-4)


def make_request_flags(flags):
    from fclg.api import make_request
    return make_request(flags=flags)


@pytest.mark.parametrize("workload,n", [("mixed", 60000), ("pareto", 60000)])
def test_boolean_collide_mpr_vs_oracle(gpu_ctx, oracle_lib, workload, n):
    """Boolean fcl::collide: MPR on the GPU (GJK where MPR fails) against the
    restated reference's MPR, and against the GJK boolean; flags identical
    outside the 1e-6 m band around contact."""
    from fclg.api import make_request
    BOOLEAN, GJK_BOOLEAN, NO_ANALYTIC, MPR_BIT = 1, 8, 16, 1 << 16
    b = getattr(workloads, workload)(n)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.collide(b.pairs, make_request(flags=BOOLEAN | NO_ANALYTIC))
    gjk = gpu_ctx.collide(b.pairs, make_request(flags=BOOLEAN | GJK_BOOLEAN | NO_ANALYTIC))
    ref = oracle_lib.collide(b, analytic=False)
    sd = oracle_lib.signed_distance(b)
    outside = np.abs(sd["distance"]) > BAND
    assert np.sum((got["collide"] != ref["ok"]) & outside) == 0
    assert np.sum((got["collide"] != gjk["collide"]) & outside) == 0
    assert np.mean((got["status"] & MPR_BIT) != 0) > 0.99   # MPR decided (almost) every pair
    assert np.all((gjk["status"] & MPR_BIT) == 0)


@pytest.mark.parametrize("workload,n", [("plain_small", 4096), ("mixed", 60000), ("pareto", 60000)])
def test_distance_vs_oracle(gpu_ctx, oracle_lib, workload, n):
    b = getattr(workloads, workload)(n)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.distance(b.pairs)
    ref = oracle_lib.signed_distance(b)
    check_parity(got, ref, b)
    # status words: GJK verdict identical wherever the reference is outside the band
    outside = np.abs(ref["distance"]) > BAND
    assert np.mean(gjk_status(got["status"])[outside] == ref["gjk_status"][outside]) > 0.999


@pytest.mark.parametrize("workload,n", [("mixed", 200000), ("pareto", 100000)])
def test_parity_tails_have_stated_causes(gpu_ctx, oracle_lib, workload, n):
    """Every pair outside the tight bars (|err| > 1e-5 m) is one of the cases
    the bar names, checked pair by pair instead of as a fraction:
    * separation: both answers lie at or above the exact distance (the FP64
      oracle run to a 1e-12 tolerance, 1000 iterations; 1e-6 m of FP32 slack
      on the GPU side) -- GJK's |v| bounds the distance from above, and the
      two distance loops stopped on the reference's small-improvement rule
      (gjk_distance.hpp:78-90) at different iterates above it (curved shapes,
      and hulls of many vertices where one step improves little);
    * depth: EPA ended on its face capacity or iteration limit on at least one
      side (the reference's MallocFailed / IterationLimit results are its
      partial polytope's nearest face, epa.hpp:220-234); otherwise a curved
      shape is involved and both depths lie at or below the converged depth
      (the oracle's EPA with 4096 faces and a 1e-9 tolerance): the nearest
      face of a polytope inside the Minkowski difference bounds the depth from
      below, and the two runs met their stopping test on different faces."""
    b = getattr(workloads, workload)(n)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.distance(b.pairs)
    ref = oracle_lib.signed_distance(b)
    both = (got["ok"] == 1) & (ref["ok"] == 1)
    rd = ref["distance"]
    gd = got["distance"].astype(np.float64)
    err = np.abs(gd - rd)
    tail = np.nonzero(both & (rd > BAND) & (err > 1e-5))[0]
    if len(tail):
        ex = oracle_lib.signed_distance(b.subset(tail), gjk_max_iter=1000, gjk_tol=1e-12)
        assert np.all(ex["ok"] == 1)
        assert np.all(gd[tail] >= ex["distance"] - 1e-6), "GPU separation below the exact distance"
        assert np.all(rd[tail] >= ex["distance"] - 1e-9)
    tail = np.nonzero(both & (rd < -BAND) & (err > 1e-5))[0]
    if len(tail):
        limits = (EPA_ITER_LIMIT, EPA_MALLOC_FAILED)
        limited = np.isin(epa_status(got["status"][tail]), limits) | np.isin(ref["epa_status"][tail], limits)
        rest = tail[~limited]
        if len(rest):
            assert np.all(_curved(b)[rest]), "depth tails on polyhedra with EPA converged: %s" % rest[:8]
            big = oracle_lib.signed_distance(b.subset(rest), epa_max_faces=4096, epa_max_iter=20000, epa_tol=1e-9)
            assert np.all(big["epa_status"] == EPA_OK)
            assert np.all(-gd[rest] <= -big["distance"] + 1e-6), "GPU depth beyond the converged depth"
            assert np.all(-rd[rest] <= -big["distance"] + 1e-9)


def test_launch_shapes_agree(gpu_ctx, oracle_lib):
    b = workloads.mixed(20000, seed=5)
    gpu_ctx.set_batch(b)
    ref = oracle_lib.signed_distance(b)
    outs = []
    for lanes in (1, 4, 32):
        gpu_ctx.set_launch(gjk_lanes=lanes)
        outs.append(gpu_ctx.distance(b.pairs))
        check_parity(outs[-1], ref, b)
    gpu_ctx.set_launch(gjk_lanes=1)
    for o in outs[1:]:
        assert np.mean(np.abs(o["distance"] - outs[0]["distance"]) <= 1e-5) > 0.995


def test_device_entry_point_matches_host(gpu_ctx):
    import torch
    b = workloads.mixed(5000, seed=6)
    gpu_ctx.set_batch(b)
    host = gpu_ctx.distance(b.pairs)
    d_pairs = torch.from_numpy(b.pairs.view(np.uint8).copy()).cuda()
    d_res = torch.empty(len(b.pairs) * 48, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    gpu_ctx.distance_device(d_pairs.data_ptr(), len(b.pairs), d_res.data_ptr(), None, s.cuda_stream)
    s.synchronize()
    dev = d_res.cpu().numpy().view(host.dtype)
    assert np.array_equal(dev.view(np.uint8), host.view(np.uint8))


def _one(shape_a, shape_b, R, t, verts=None):
    s = np.concatenate([shape_a, shape_b])
    p = np.zeros(len(t), PAIR_DTYPE)
    p["shape_b"] = 1
    p["rot"] = np.asarray(R).reshape(-1, 9)
    p["trans"] = t
    v = np.zeros((1, 4), np.float32) if verts is None else verts
    return workloads.Batch("edge", s, v, p)


def _sh(t, *param, vc=0, vo=0):
    s = np.zeros(1, SHAPE_DTYPE)
    s["type"] = t
    s["param"][0, :len(param)] = param
    s["vert_count"] = vc
    s["vert_offset"] = vo
    return s


def test_edge_cases(gpu_ctx, oracle_lib):
    # empty batch
    b = _one(_sh(SPHERE, 0.1), _sh(SPHERE, 0.1), np.eye(3)[None], np.zeros((1, 3)))
    gpu_ctx.set_batch(b)
    assert len(gpu_ctx.distance(b.pairs[:0])) == 0
    # coincident spheres, face-touching boxes, separated boxes, deep box-in-box
    eye = np.repeat(np.eye(3)[None], 4, axis=0)
    t = np.array([[0, 0, 0], [0.2, 0, 0], [0.5, 0, 0], [0.01, 0.02, 0]], np.float64)
    b = _one(_sh(BOX, 0.2, 0.2, 0.2), _sh(BOX, 0.2, 0.2, 0.2), eye, t)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.distance(b.pairs)
    ref = oracle_lib.signed_distance(b)
    assert np.all(got["ok"] == ref["ok"])
    assert np.allclose(got["distance"], ref["distance"], atol=1e-5)
    # NaN pose: must return (no hang) and must not claim a valid distance
    p = b.pairs.copy()
    p["trans"][0] = np.nan
    got = gpu_ctx.distance(p)
    assert got["ok"][0] == 0 or np.isnan(got["distance"][0])
    # out-of-range shape index: rejected per pair, not read
    p = b.pairs.copy()
    p["shape_b"][1] = 1000
    got = gpu_ctx.distance(p)
    assert got["ok"][1] == 0 and gjk_status(got["status"][1]) == 4
    # one-vertex convex (a point) against a sphere, and a flat (coplanar) hull against a box
    verts = np.array([[0.3, 0, 0, 0], [-0.1, -0.1, 0, 0], [0.1, -0.1, 0, 0], [0.1, 0.1, 0, 0], [-0.1, 0.1, 0, 0]],
                     np.float32)
    s = np.concatenate([_sh(CONVEX, vc=1, vo=0), _sh(SPHERE, 0.1), _sh(CONVEX, vc=4, vo=1), _sh(BOX, 0.1, 0.1, 0.1)])
    p = np.zeros(3, PAIR_DTYPE)
    p["rot"] = np.eye(3).ravel()
    p[0]["shape_a"], p[0]["shape_b"] = 0, 1
    p[1]["shape_a"], p[1]["shape_b"] = 2, 3
    p[2]["shape_a"], p[2]["shape_b"] = 2, 3
    p["trans"] = [[0, 0, 0], [0, 0, 0.3], [0.02, 0.01, 0.03]]
    b = workloads.Batch("edge2", s, verts, p)
    gpu_ctx.set_batch(b)
    got = gpu_ctx.distance(b.pairs)
    ref = oracle_lib.signed_distance(b)
    assert np.all(got["ok"] == ref["ok"])
    ok = ref["ok"] == 1
    assert np.allclose(got["distance"][ok], ref["distance"][ok], atol=1e-5)


def test_large_hulls(gpu_ctx, oracle_lib):
    # Pareto tail: up to 1024-vertex hulls
    b = workloads.pareto(200000, seed=12)
    big = np.nonzero(np.maximum(b.shapes["vert_count"][b.pairs["shape_a"]],
                                b.shapes["vert_count"][b.pairs["shape_b"]]) >= 256)[0][:3000]
    sub = b.subset(big)
    gpu_ctx.set_batch(sub)
    check_parity(gpu_ctx.distance(sub.pairs), oracle_lib.signed_distance(sub), sub)


def test_invalid_shapes_rejected(gpu_ctx):
    from fclg.api import FclgError
    s = _sh(CONVEX, vc=10, vo=0)
    with pytest.raises(FclgError, match="vertex range"):
        gpu_ctx.set_shapes(s, np.zeros((4, 4), np.float32))
    with pytest.raises(FclgError, match="unsupported type"):
        gpu_ctx.set_shapes(_sh(7, 1.0), np.zeros((1, 4), np.float32))


def test_epa_resume_equals_restart(gpu_ctx):
    """A pair whose EPA polytope outgrows the 128-face layout continues in the
    256-face layout from its saved state (fclg_tuning.epa_resume, the
    default); rerunning it from the GJK simplex instead gives byte-identical
    results, since both layouts assign slots the same way until the smaller
    one fills."""
    b = workloads.mixed(200000, seed=workloads.SEED_BASE + 51)
    gpu_ctx.set_batch(b)
    keep = gpu_ctx.get_tuning()
    try:
        gpu_ctx.set_tuning(epa_resume=True)
        resumed = gpu_ctx.distance(b.pairs)
        gpu_ctx.set_tuning(epa_resume=False)
        restarted = gpu_ctx.distance(b.pairs)
    finally:
        gpu_ctx.set_tuning(**keep)
    assert resumed.tobytes() == restarted.tobytes()
    # the batch does reach the large layout (about 64 expansions fill 128 faces)
    assert np.sum((resumed["distance"] < 0) & (resumed["iterations"] > 90)) > 100


@pytest.mark.parametrize("workload", ["mixed", "pareto"])
def test_split_gjk_launches_equal_one_pass(gpu_ctx, workload):
    """The bucketed one-lane distance query runs GJK as two launches (boolean
    phase, then the distance loop over the separated pairs it hands over);
    the results equal the single-pass launch's (bucketing off) byte for byte,
    with and without EPA."""
    from fclg.api import FCLG_REQ_NO_EPA, make_request
    b = getattr(workloads, workload)(100_000, seed=workloads.SEED_BASE + 43)
    keep = gpu_ctx.get_tuning()
    gpu_ctx.set_batch(b)
    try:
        for req in (None, make_request(flags=FCLG_REQ_NO_EPA)):
            out = []
            for bucketing in (True, False):
                gpu_ctx.set_tuning(bucketing=bucketing, gjk_lanes_small=1, gjk_lanes_large=1, gjk_refill=False,
                                   large_hull_vertices=1024)
                out.append(gpu_ctx.distance(b.pairs, req))
            assert np.array_equal(out[0].view(np.uint8), out[1].view(np.uint8))
    finally:
        gpu_ctx.set_tuning(**keep)
