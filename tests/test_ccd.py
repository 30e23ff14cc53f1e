"""Translational continuous collision of shape pairs (fcl::translational_ccd,
narrowphase/continuous_collision.h:13-19; ShapePairTranslationalCollisionSolver,
narrowphase/detail/ccd/shape_pair_ccd-inl.h).

CPU: the FP64 restatement (oracle/orc_ccd.hpp) pinned two ways --
* the swept-volume MPR and its portal bit for bit against the reference's own
  MPR::Intersect with IntersectData (oracle/_ref, where it is built);
* the box interval test and the one-sample time of collision against the
  properties the reference's tests check (test/ccd/test_box_pair_ccd.cpp,
  test/ccd/test_shape_pair_interface.cpp): interval symmetry and endpoints,
  zero displacement = the static box test, boxes by interval = boxes by
  swept MPR, a swept sphere = a capsule, and the moving shape touching the
  other at the sampled time.
GPU (marked): the library's pass against the restatement on the same pairs.
"""
import os

import numpy as np
import pytest

from fclg import workloads
from fclg.layout import BOX, CAPSULE, SHAPE_DTYPE, SPHERE

import oracle


def _rot(rng, n):
    return workloads.random_rotations(rng, n).reshape(n, 3, 3)


def _obb_overlap(h1, R, t, h2, eps=0.0):
    """Static separating-axis test of box 1 (half sizes h1, at the origin,
    axis-aligned) and box 2 (half sizes h2, rotation R, centre t): True when
    no axis separates them by more than eps."""
    Ra = np.abs(R)
    for k in range(3):  # box 1's axes
        if abs(t[k]) > h1[k] + Ra[k] @ h2 + eps:
            return False
    for k in range(3):  # box 2's axes
        if abs(R[:, k] @ t) > Ra[:, k] @ h1 + h2[k] + eps:
            return False
    for k in range(3):
        for i in range(3):
            a = np.cross(np.eye(3)[k], R[:, i])
            if np.linalg.norm(a) < 1e-12:
                continue
            if abs(a @ t) > np.abs(a) @ h1 + np.abs(R.T @ a) @ h2 + eps * np.linalg.norm(a):
                return False
    return True


def test_box_axis_interval_random_and_symmetric():
    """testTocIntervalOnAxisRandom / testTocIntervalOnAxisSymmetry: boxes of
    half sizes 0.5 and 0.8, displacement and offset uniform in [-10, 10].  An
    empty interval means the boxes are apart at both ends of the motion; a
    non-empty one touches at both of its (unscaled) ends; mirroring both
    inputs keeps the interval; at offset 0 it is [0, min(|d|, 1.3)]."""
    rng = np.random.default_rng(1)
    h1, h2 = 0.5, 0.8
    for d, off in (rng.random((20000, 2)) * 20 - 10):
        e, lo, hi = oracle.box_axis(h1, d, h2, off)
        lb2, ub2 = off - h2, off + h2
        if e:
            assert -h1 > ub2 or lb2 > h1
            assert d - h1 > ub2 or lb2 > d + h1
        else:
            sg = 1.0 if d > 0 else -1.0
            for s in (lo, hi):
                assert not (sg * s - h1 > ub2 + 1e-9 or lb2 > sg * s + h1 + 1e-9)
        e2, lo2, hi2 = oracle.box_axis(h1, -d, h2, -off)
        assert e == e2 and (e or (abs(lo - lo2) < 1e-12 and abs(hi - hi2) < 1e-12))
        e3, _, _ = oracle.box_axes3(h1, d, h2, off)
        assert e3 == e
        e0, lo0, hi0 = oracle.box_axis(h1, d, h2, 0.0)
        assert not e0 and lo0 == 0.0 and abs(hi0 - min(abs(d), h1 + h2)) < 1e-12


def test_box_pair_interval_properties():
    """boxPairIntersectTest: AABB [-0.1, 0.2]^3 boxes at random poses in a
    cube of half size 0.5 -- zero displacement gives the static box test; with
    a random unit axis and distance, box 1 moved to either end of the interval
    overlaps box 2, and a disjoint verdict leaves ten samples along the motion
    apart."""
    rng = np.random.default_rng(2)
    n = 3000
    h = np.full(3, 0.15)
    c = np.full(3, 0.05)  # centre of [-0.1, 0.2]^3
    R1, R2 = _rot(rng, n), _rot(rng, n)
    T1, T2 = rng.random((n, 3)) - 0.5, rng.random((n, 3)) - 0.5
    U = _rot(rng, n)[:, :, 0]
    D = np.abs(rng.random(n) - 0.5)
    hits = 0
    for i in range(n):
        To1, To2 = R1[i] @ c + T1[i], R2[i] @ c + T2[i]
        R = R1[i].T @ R2[i]
        t = R1[i].T @ (To2 - To1)
        e, lo, hi = oracle.box_pair_ccd(h, [1, 0, 0], 0.0, R, t, h)
        assert (not e) == _obb_overlap(h, R, t, h, 1e-9) or _obb_overlap(h, R, t, h, 1e-7) != _obb_overlap(
            h, R, t, h, -1e-7)
        e, lo, hi = oracle.box_pair_ccd(h, U[i], D[i], R, t, h)
        if not e:
            hits += 1
            assert hi >= lo
            for s in (lo, hi):
                assert _obb_overlap(h, R, t - U[i] * D[i] * s, h, 1e-9)
        else:
            for s in np.arange(10) / 10.0:
                assert not _obb_overlap(h, R, t - U[i] * D[i] * s, h, -1e-9)
    assert 0.2 < hits / n < 0.9


def _box_batch(rng, n, s1=0.2, s2=0.25):
    s = np.zeros(2, SHAPE_DTYPE)
    s["type"] = BOX
    s["param"][0, :3] = s1
    s["param"][1, :3] = s2
    p = np.zeros(n, workloads.PAIR_DTYPE)
    p["shape_a"], p["shape_b"] = 0, 1
    R1, R2 = _rot(rng, n), _rot(rng, n)
    T1, T2 = rng.random((n, 3)) - 0.5, rng.random((n, 3)) - 0.5
    p["rot"] = np.einsum("nji,njk->nik", R1, R2).reshape(n, 9)
    p["trans"] = np.einsum("nji,nj->ni", R1, T2 - T1)
    d = np.zeros((n, 4), np.float32)
    d[:, :3] = _rot(rng, n)[:, :, 0]
    d[:, 3] = np.abs(rng.random(n) - 0.5)
    return workloads.Batch("boxes", s, np.zeros((1, 4), np.float32), p, {}), d


def test_box_interval_equals_swept_mpr():
    """boxPairIntersectTestCompareMPR: cubes of sides 0.2 and 0.25 -- the box
    interval test and MPR on the swept volume give the same verdict (outside
    a 1e-9 band of the swept boxes' contact, which neither decides reliably)."""
    b, d = _box_batch(np.random.default_rng(3), 20000)
    got = oracle.translational_ccd(b, d, oracle.TOC_NONE)
    assert np.all(got["box_tested"] == 1) and np.all(got["mpr_status"] == -1)
    mpr = oracle.swept_portal(b, d)[:, 0]
    assert np.all(mpr != 2)
    diff = np.nonzero(got["collide"] != (mpr == 0))[0]
    assert len(diff) <= 2, diff
    assert 0.05 < got["collide"].mean() < 0.9
    hit = got["collide"] == 1
    assert np.all((got["toc_lo"][hit] >= 0) & (got["toc_lo"][hit] <= got["toc_hi"][hit]) & (got["toc_hi"][hit] <= 1))


def test_swept_sphere_equals_capsule():
    """sphereCapsuleTest: a sphere of radius 0.1 moving along its z axis by
    |t| (t uniform in [-0.5, 0.5]) against a sphere of radius 0.125 hits
    exactly when the capsule its motion sweeps (radius 0.1, length |t|,
    centred halfway) collides statically; the sampled time of collision puts
    the two spheres in touch."""
    rng = np.random.default_rng(4)
    n = 4000
    dist = np.abs(rng.random(n) - 0.5).astype(np.float32)
    s = np.zeros(2 + n, SHAPE_DTYPE)
    s["type"][0], s["type"][1] = SPHERE, SPHERE
    s["param"][0, 0], s["param"][1, 0] = 0.1, 0.125
    s["type"][2:] = CAPSULE
    s["param"][2:, 0] = 0.1
    s["param"][2:, 1] = dist
    R1, R2 = _rot(rng, n), _rot(rng, n)
    T1, T2 = rng.random((n, 3)) - 0.5, rng.random((n, 3)) - 0.5
    p = np.zeros(n, workloads.PAIR_DTYPE)
    p["shape_a"], p["shape_b"] = 0, 1
    p["rot"] = np.einsum("nji,njk->nik", R1, R2).reshape(n, 9)
    p["trans"] = np.einsum("nji,nj->ni", R1, T2 - T1)
    d = np.zeros((n, 4), np.float32)
    d[:, 2] = 1.0
    d[:, 3] = dist
    b = workloads.Batch("spheres", s, np.zeros((1, 4), np.float32), p, {})
    got = oracle.translational_ccd(b, d, oracle.TOC_SAMPLE)
    cap = p.copy()
    cap["shape_a"] = np.arange(2, 2 + n)
    cap["trans"] = p["trans"] - np.array([0, 0, 1.0]) * (0.5 * dist[:, None])
    ref = oracle.collide(workloads.Batch("caps", s, b.vertices, cap, {}), analytic=True)
    gap = np.linalg.norm(p["trans"].astype(np.float64) - np.array([0, 0, 1.0]) * np.clip(
        p["trans"][:, 2:3], 0, dist[:, None]), axis=1) - 0.225
    clear = np.abs(gap) > 1e-6
    assert np.array_equal(got["collide"][clear], ref["ok"][clear])
    assert 0.03 < got["collide"].mean() < 0.9
    hit = got["collide"] == 1
    ts = got["toc_lo"][hit]
    assert np.array_equal(ts, got["toc_hi"][hit]) and np.all((ts >= 0) & (ts <= 1))
    c = p["trans"][hit].astype(np.float64) - np.array([0, 0, 1.0]) * (ts * dist[hit])[:, None]
    assert np.all(np.linalg.norm(c, axis=1) <= 0.225 + 1e-6)


def test_toc_sample_touches_mixed():
    """The sampled time of collision on the mixed kinds: shape a moved by the
    sampled fraction of its displacement touches shape b (signed distance
    <= 1e-6 m by the FP64 oracle) -- the origin lies in the final portal
    tetrahedron, so the barycentric mix of the portal's support points is a
    common point of both shapes at that time (gjk_ccd-inl.h:106-187)."""
    b, d = workloads.ccd(20000, seed=workloads.SEED_BASE + 91)
    got = oracle.translational_ccd(b, d, oracle.TOC_SAMPLE)
    hit = (got["collide"] == 1) & (got["mpr_status"] == 0)
    assert hit.mean() > 0.2
    ts = got["toc_lo"]
    assert np.all((ts[hit] >= 0) & (ts[hit] <= 1))
    moved = b.pairs.copy()
    moved["trans"] = (b.pairs["trans"].astype(np.float64) - d[:, :3] * (ts * d[:, 3])[:, None]).astype(np.float32)
    sd = oracle.signed_distance(workloads.Batch("moved", b.shapes, b.vertices, moved[hit], {}))
    ok = sd["ok"] == 1
    assert ok.mean() > 0.999
    assert np.mean(sd["distance"][ok] <= 1e-6) >= 0.999, np.sort(sd["distance"][ok])[-5:]
    # the box pre-check never drops a swept-MPR hit
    bx = oracle.translational_ccd(b, d, oracle.TOC_BOX)
    assert np.array_equal(bx["collide"], got["collide"])
    assert np.all(bx["box_tested"] == 1)


@pytest.mark.skipif(not os.path.exists(oracle.REF_PATH), reason="reference driver not built")
@pytest.mark.parametrize("workload", ["ccd", "boxes"])
def test_swept_portal_pinned_to_reference(workload):
    """The restated swept-volume MPR (status and IntersectData: interior point,
    portal vertices and directions) equals the reference's MPR::Intersect on
    the same difference bit for bit."""
    if workload == "ccd":
        b, d = workloads.ccd(20000, seed=workloads.SEED_BASE + 92)
    else:
        b, d = _box_batch(np.random.default_rng(5), 5000)
    a, r = oracle.swept_portal(b, d), oracle.ref_swept_portal(b, d)
    same = np.all((a == r) | (np.isnan(a) & np.isnan(r)), axis=1)
    assert same.all(), np.nonzero(~same)[0][:5]
    assert np.mean(a[:, 0] == 0) > 0.1


@pytest.mark.gpu
@pytest.mark.parametrize("toc", [0, 1, 2])
def test_gpu_ccd_vs_oracle(toc):
    """The library's pass (fclg_translational_ccd) against the restatement:
    box-box pairs and the box pre-check bit for bit in their decision and
    within float rounding in their interval (FP64 on both sides); swept MPR
    (FP32) verdicts equal outside a 1e-6 m band of contact at either end of
    the motion for >= 99.9 % of pairs; sampled times within 1e-3 of the
    oracle's for >= 99 % of hits on both sides, and the GPU's sampled time
    puts the shapes in touch (signed distance <= 1e-4 m) for >= 99.5 %."""
    from fclg.api import Context
    b, d = workloads.ccd(50000, seed=workloads.SEED_BASE + 93)
    ctx = Context(0)
    try:
        ctx.set_batch(b)
        got = ctx.translational_ccd(b.pairs, d, toc_type=toc)
    finally:
        ctx.close()
    ref = oracle.translational_ccd(b, d, toc)
    boxes = (b.shapes["type"][b.pairs["shape_a"]] == BOX) & (b.shapes["type"][b.pairs["shape_b"]] == BOX)
    tested = (got["status"] & 4) != 0
    assert np.array_equal(tested, ref["box_tested"] == 1)
    disj = (got["status"] & 8) != 0
    ref_disj = (ref["box_tested"] == 1) & np.where(boxes, ref["collide"] == 0, ref["mpr_status"] == -1)
    assert np.array_equal(disj, ref_disj)
    assert np.array_equal(got["collide"][boxes], ref["collide"][boxes])
    hb = boxes & (ref["collide"] == 1)
    assert np.allclose(got["toc_lower"][hb], ref["toc_lo"][hb], rtol=1e-6, atol=1e-7)
    assert np.allclose(got["toc_upper"][hb], ref["toc_hi"][hb], rtol=1e-6, atol=1e-7)
    # MPR verdicts outside a band: signed distance at the start and at the end of the motion
    sd0 = oracle.signed_distance(b)["distance"]
    end = b.pairs.copy()
    end["trans"] = (b.pairs["trans"].astype(np.float64) - d[:, :3] * d[:, 3:4]).astype(np.float32)
    sd1 = oracle.signed_distance(workloads.Batch("end", b.shapes, b.vertices, end, {}))["distance"]
    clear = (np.abs(sd0) > 1e-6) & (np.abs(sd1) > 1e-6)
    m = ~boxes
    assert np.mean(got["collide"][m & clear] == ref["collide"][m & clear]) >= 0.999
    if toc == 2:
        both = m & (got["collide"] == 1) & (ref["collide"] == 1)
        err = np.abs(got["toc_lower"][both].astype(np.float64) - ref["toc_lo"][both])
        assert np.mean(err <= 1e-3) >= 0.99
        ts = got["toc_lower"].astype(np.float64)
        moved = b.pairs.copy()
        moved["trans"] = (b.pairs["trans"].astype(np.float64) - d[:, :3] * (ts * d[:, 3])[:, None]).astype(np.float32)
        h = m & (got["collide"] == 1)
        sd = oracle.signed_distance(workloads.Batch("moved", b.shapes, b.vertices, moved[h], {}))
        assert np.mean((sd["ok"] == 1) & (sd["distance"] <= 1e-4)) >= 0.995


@pytest.mark.gpu
def test_gpu_ccd_edge_cases():
    """An empty batch is a no-op; a pair naming a shape outside the set gets
    collide 0, no interval and status bit 4 (shape id out of range) while its
    neighbours are unaffected; zero displacement reduces to the static
    collide (MPR flags of the oracle's static boolean)."""
    from fclg.api import Context
    b, d = workloads.ccd(2000, seed=workloads.SEED_BASE + 94)
    ctx = Context(0)
    try:
        ctx.set_batch(b)
        assert len(ctx.translational_ccd(b.pairs[:0], d[:0])) == 0
        bad = b.pairs.copy()
        bad["shape_b"][::7] = len(b.shapes) + 5
        got = ctx.translational_ccd(bad, d, toc_type=2)
        ref = ctx.translational_ccd(b.pairs, d, toc_type=2)
        z = d.copy()
        z[:, 3] = 0.0
        still = ctx.translational_ccd(b.pairs, z)
    finally:
        ctx.close()
    m = np.zeros(len(bad), bool)
    m[::7] = True
    assert np.all(got["collide"][m] == 0) and np.all((got["status"][m] & 16) != 0)
    assert np.all(got["toc_lower"][m] == -1)
    assert np.array_equal(got.view(np.uint8).reshape(len(bad), -1)[~m], ref.view(np.uint8).reshape(len(bad), -1)[~m])
    static = oracle.collide(b, analytic=False)
    sd = oracle.signed_distance(b)["distance"]
    clear = np.abs(sd) > 1e-6
    assert np.mean(still["collide"][clear] == static["ok"][clear]) >= 0.999
