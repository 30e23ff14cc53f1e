"""The FP64 oracle (oracle/) pinned against the reference.

* bit-for-bit against outputs of the reference itself (tests/golden/
  convex_ref.npz, written by tests/golden/make_golden.py from the reference's
  own GJK / EPA / MPR), and against oracle/_ref directly where it was built;
* the known-answer and analytic cross-checks of the reference's tests:
  sphere separation 0.2 (test/cvx_collide/test_gjk2_distance.cpp:18-68),
  sphere penetration 0.2 (test_epa2_with_gjk2.cpp:21-73), capsule distance vs
  the analytic segment distance (test_gjk2_distance.cpp:156-219), the
  hard-coded capsule pair (:70-154), box flags vs a 15-axis separating-axis
  test (test_gjk2.cpp:19-77) and the hard-coded box pose (:129-223), box EPA
  depth never deeper than the SAT depth (test_epa2_with_gjk2.cpp:75-161), and
  the escape-by-1.05-depth property (test_fcl_collision_penetration.cpp:14-82).
"""
import os

import numpy as np
import pytest

from fclg import workloads
from fclg.layout import BOX, CAPSULE, CONVEX, CYLINDER, PAIR_DTYPE, SHAPE_DTYPE, SPHERE

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "convex_ref.npz")
FIELDS = ["distance", "p0", "p1", "normal", "ok", "gjk_status", "epa_status"]


def _batch(shapes, vertices, pairs, name="case"):
    return workloads.Batch(name, np.asarray(shapes, SHAPE_DTYPE), np.asarray(vertices, np.float32).reshape(-1, 4),
                           np.asarray(pairs, PAIR_DTYPE))


def _same(a, b):
    return np.all(np.stack([np.all((a[f] == b[f]).reshape(len(a), -1), axis=1) for f in FIELDS]), axis=0)


def _golden(name):
    g = np.load(GOLDEN)
    return _batch(g[name + "/shapes"], g[name + "/vertices"], g[name + "/pairs"], name), g


@pytest.mark.parametrize("name", ["plain_small", "mixed", "pareto"])
def test_oracle_matches_reference_golden(oracle_lib, name):
    b, g = _golden(name)
    assert np.all(_same(oracle_lib.signed_distance(b, threads=2), g[name + "/signed_distance"]))
    # the goldens ran the reference's cvx_collide path (MPR / GJK+EPA) for every pair
    assert np.all(_same(oracle_lib.collide(b, False, threads=2, analytic=False), g[name + "/collide_bool"]))
    assert np.all(_same(oracle_lib.collide(b, True, threads=2, analytic=False), g[name + "/collide_contact"]))


def test_oracle_matches_reference_build(oracle_lib):
    if not oracle_lib.ref_available():
        pytest.skip("oracle/_ref not built (reference sources absent)")
    for b in (workloads.mixed(3000, seed=7), workloads.pareto(3000, seed=8)):
        assert np.all(_same(oracle_lib.signed_distance(b), oracle_lib.ref_signed_distance(b)))
        assert np.all(_same(oracle_lib.collide(b, True, analytic=False), oracle_lib.ref_collide(b, True)))


def _rot_from_euler(rng, n):
    # the reference tests' generateRandomTransform uses Euler angles in [0, 2pi)
    a, b, c = (rng.random(n) * 2 * np.pi for _ in range(3))
    R = np.zeros((n, 3, 3))
    ca, sa, cb, sb, cc, sc = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    R[:, 0, 0] = cb * cc
    R[:, 0, 1] = -cb * sc
    R[:, 0, 2] = sb
    R[:, 1, 0] = ca * sc + sa * sb * cc
    R[:, 1, 1] = ca * cc - sa * sb * sc
    R[:, 1, 2] = -sa * cb
    R[:, 2, 0] = sa * sc - ca * sb * cc
    R[:, 2, 1] = sa * cc + ca * sb * sc
    R[:, 2, 2] = ca * cb
    return R


def _relative(R1, t1, R2, t2):
    R = np.einsum("nji,njk->nik", R1, R2)
    t = np.einsum("nji,nj->ni", R1, t2 - t1)
    return R, t


def _pairs_of(R, t):
    p = np.zeros(len(R), PAIR_DTYPE)
    p["shape_a"] = 0
    p["shape_b"] = 1
    p["rot"] = R.reshape(-1, 9)
    p["trans"] = t
    return p


def _shape(type_, *param):
    s = np.zeros(1, SHAPE_DTYPE)
    s["type"] = type_
    s["param"][0, :len(param)] = param
    return s


def test_sphere_separation_known_answer(oracle_lib):
    rng = np.random.default_rng(1)
    n = 2000
    R1, R2 = _rot_from_euler(rng, n), _rot_from_euler(rng, n)
    t1 = rng.random((n, 3)) * 6 - 3
    d = _rot_from_euler(rng, n)[:, :, 0]
    t2 = t1 + d * 2.2
    R, t = _relative(R1, t1, R2, t2)
    b = _batch(np.concatenate([_shape(SPHERE, 1.0), _shape(SPHERE, 1.0)]), np.zeros((1, 4)), _pairs_of(R, t))
    o = oracle_lib.signed_distance(b)
    assert np.all(o["gjk_status"] == 1)
    assert np.max(np.abs(o["distance"] - 0.2)) < 1e-3


def test_sphere_penetration_known_answer(oracle_lib):
    rng = np.random.default_rng(2)
    n = 500
    d = _rot_from_euler(rng, n)[:, :, 0]
    R = np.repeat(np.eye(3)[None], n, axis=0)
    b = _batch(np.concatenate([_shape(SPHERE, 1.0), _shape(SPHERE, 1.0)]), np.zeros((1, 4)), _pairs_of(R, d * 1.8))
    o = oracle_lib.signed_distance(b)
    assert np.all(o["ok"] == 1)
    assert np.max(np.abs(-o["distance"] - 0.2)) < 1e-4


def _segment_distance(p1, q1, p2, q2):
    """Closest distance between segments (Ericson, Real-Time Collision Detection 5.1.9), vectorised."""
    d1, d2, r = q1 - p1, q2 - p2, p1 - p2
    a = np.einsum("ij,ij->i", d1, d1)
    e = np.einsum("ij,ij->i", d2, d2)
    f = np.einsum("ij,ij->i", d2, r)
    c = np.einsum("ij,ij->i", d1, r)
    b = np.einsum("ij,ij->i", d1, d2)
    den = a * e - b * b
    s = np.where(den > 1e-15, np.clip((b * f - c * e) / np.where(den > 1e-15, den, 1), 0, 1), 0.0)
    t = (b * s + f) / e
    s = np.where(t < 0, np.clip(-c / a, 0, 1), np.where(t > 1, np.clip((b - c) / a, 0, 1), s))
    t = np.clip(t, 0, 1)
    c1 = p1 + d1 * s[:, None]
    c2 = p2 + d2 * t[:, None]
    return np.linalg.norm(c1 - c2, axis=1)


def _capsule_distance(R, t, r, lz):
    n = len(R)
    h = np.array([0, 0, lz / 2])
    p1, q1 = np.tile(h, (n, 1)), np.tile(-h, (n, 1))
    p2 = np.einsum("nij,j->ni", R, h) + t
    q2 = np.einsum("nij,j->ni", R, -h) + t
    return _segment_distance(p1, q1, p2, q2) - 2 * r


def test_capsule_distance_vs_analytic(oracle_lib):
    rng = np.random.default_rng(3)
    n = 3000
    R1, R2 = _rot_from_euler(rng, n), _rot_from_euler(rng, n)
    t1, t2 = rng.random((n, 3)) * 4 - 2, rng.random((n, 3)) * 4 - 2
    R, t = _relative(R1, t1, R2, t2)
    b = _batch(np.concatenate([_shape(CAPSULE, 0.5, 1.3), _shape(CAPSULE, 0.5, 1.3)]), np.zeros((1, 4)),
               _pairs_of(R.astype(np.float32).astype(np.float64), t.astype(np.float32).astype(np.float64)))
    o = oracle_lib.signed_distance(b)
    ref = _capsule_distance(b.pairs["rot"].reshape(-1, 3, 3).astype(np.float64),
                            b.pairs["trans"].astype(np.float64), 0.5, 1.3)
    sep = ref > 1e-6
    assert np.all(o["gjk_status"][sep] == 1)
    assert np.sum(np.abs(o["distance"][sep] - ref[sep]) > 5e-3) <= 2


def test_capsule_pair_known_answer(oracle_lib):
    """The hard-coded capsule pair of test_gjk2_distance.cpp:70-154 with the
    GJK2(1000, 1e-7) that test uses.  The reference's GJK stops about 6.8e-3
    above the analytic segment distance here (that test only prints the gap);
    the oracle must reproduce the reference's own answer bit for bit."""
    b, g = _golden("capsule_pair")
    o = oracle_lib.signed_distance(b, gjk_max_iter=1000, gjk_tol=1e-7)
    assert np.all(_same(o, g["capsule_pair/signed_distance"]))
    ref = _capsule_distance(b.pairs["rot"].reshape(-1, 3, 3).astype(np.float64),
                            b.pairs["trans"].astype(np.float64), 0.5, 1.3)
    assert o["gjk_status"][0] == 1
    assert 0.0 < o["distance"][0] - ref[0] < 1e-2


def _box_sat(R, t, h1, h2):
    """15-axis separating-axis test for boxes a (at origin) and b (R, t); returns
    (overlap flag, minimum overlap depth over the axes)."""
    A = np.eye(3)
    axes = [A[i] for i in range(3)] + [R[:, i] for i in range(3)]
    axes += [np.cross(A[i], R[:, j]) for i in range(3) for j in range(3)]
    depth = np.inf
    for ax in axes:
        nl = np.linalg.norm(ax)
        if nl < 1e-9:
            continue
        ax = ax / nl
        ra = np.sum(h1 * np.abs(ax))
        rb = np.sum(h2 * np.abs(R.T @ ax))
        dist = abs(ax @ t)
        ov = ra + rb - dist
        if ov < 0:
            return False, 0.0
        depth = min(depth, ov)
    return True, depth


def test_box_flags_vs_sat(oracle_lib):
    rng = np.random.default_rng(4)
    n = 3000
    R1, R2 = _rot_from_euler(rng, n), _rot_from_euler(rng, n)
    t1, t2 = rng.random((n, 3)) * 0.4 - 0.2, rng.random((n, 3)) * 0.4 - 0.2
    R, t = _relative(R1, t1, R2, t2)
    b = _batch(np.concatenate([_shape(BOX, 0.1, 0.1, 0.1), _shape(BOX, 0.2, 0.2, 0.2)]), np.zeros((1, 4)),
               _pairs_of(R, t))
    Rf = b.pairs["rot"].reshape(-1, 3, 3).astype(np.float64)
    tf = b.pairs["trans"].astype(np.float64)
    sat = np.array([_box_sat(Rf[i], tf[i], np.full(3, 0.05), np.full(3, 0.1))[0] for i in range(n)])
    mpr = oracle_lib.collide(b, False)["ok"] == 1
    gjk = oracle_lib.signed_distance(b)["distance"] < 0
    assert np.all(mpr == sat)
    assert np.all(gjk == sat)


def test_box_known_pose(oracle_lib):
    R1 = np.array([[-0.6001922922342994848, -0.6452300220595174052, 0.4727022646186623822],
                   [-0.6144479604359862623, 0.750289910702751861, 0.2439646568946272354],
                   [-0.5120770608595877071, -0.1440252357426682894, -0.8467784924114895029]])
    t1 = np.array([0.1331561010330915562, -0.04835435003042221069, -0.08343856278806925653])
    R2 = np.array([[0.7155820814515156947, 0.2218768144779907359, -0.6623541076362519098],
                   [0.5764451852026616363, -0.7231199678065238778, 0.3805370686492457466],
                   [-0.3945291284077582228, -0.6541163438996084878, -0.6453515131160874052]])
    t2 = np.array([-0.00932837892323731821, 0.08853187374770643547, -0.05020954832434654236])
    R, t = _relative(R1[None], t1[None], R2[None], t2[None])
    b = _batch(np.concatenate([_shape(BOX, 0.1, 0.1, 0.1), _shape(BOX, 0.2, 0.2, 0.2)]), np.zeros((1, 4)),
               _pairs_of(R, t))
    sat = _box_sat(b.pairs["rot"].reshape(3, 3).astype(np.float64), b.pairs["trans"][0].astype(np.float64),
                   np.full(3, 0.05), np.full(3, 0.1))[0]
    assert (oracle_lib.collide(b, False)["ok"][0] == 1) == sat
    assert (oracle_lib.signed_distance(b)["distance"][0] < 0) == sat


def test_box_epa_depth_vs_sat(oracle_lib):
    rng = np.random.default_rng(5)
    n = 3000
    R1, R2 = _rot_from_euler(rng, n), _rot_from_euler(rng, n)
    t1, t2 = rng.random((n, 3)) * 4 - 2, rng.random((n, 3)) * 4 - 2
    R, t = _relative(R1, t1, R2, t2)
    t = t * 0.25
    b = _batch(np.concatenate([_shape(BOX, 2, 1, 0.5), _shape(BOX, 1, 1, 1)]), np.zeros((1, 4)), _pairs_of(R, t))
    Rf = b.pairs["rot"].reshape(-1, 3, 3).astype(np.float64)
    tf = b.pairs["trans"].astype(np.float64)
    o = oracle_lib.signed_distance(b)
    hit = 0
    for i in range(n):
        ov, depth = _box_sat(Rf[i], tf[i], np.array([1, 0.5, 0.25]), np.full(3, 0.5))
        if not ov:
            continue
        hit += 1
        assert o["ok"][i] == 1
        epa = -o["distance"][i]
        assert not (abs(depth - epa) > 1e-4 and depth < epa)
    assert hit > 100


def test_escape_moves_out_of_collision(oracle_lib):
    """Moving b by 1.05 x depth along the contact normal separates the pair.
    Box pairs are left out: fcl::collide answers them with boxBox2, whose
    contact depth is that of the deepest clipped manifold point, at most the
    separating-axis overlap (test_box_box.py checks that bound)."""
    b = workloads.mixed(3000, seed=11)
    o = oracle_lib.collide(b, True)
    t = b.shapes["type"]
    box_box = (t[b.pairs["shape_a"]] == BOX) & (t[b.pairs["shape_b"]] == BOX)
    hit = np.nonzero((o["ok"] == 1) & (o["distance"] < -1e-6) & ~box_box)[0]
    assert len(hit) > 500
    moved = b.subset(hit)
    depth = -o["distance"][hit]
    moved.pairs["trans"] = (moved.pairs["trans"].astype(np.float64) + 1.05 * depth[:, None] * o["normal"][hit]).astype(
        np.float32)
    again = oracle_lib.collide(moved, False)
    assert np.mean(again["ok"] == 0) > 0.995


def test_convex_support_known_answers(oracle_lib):
    # A tetrahedron (test/geometry/shape/test_convex.cpp:537-603 style): the
    # distance from a far sphere along each axis pins the extreme vertex.
    verts = np.array([[0, 0, 0, 0], [1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32)
    s = np.zeros(2, SHAPE_DTYPE)
    s[0]["type"] = CONVEX
    s[0]["vert_count"] = 4
    s[1]["type"] = SPHERE
    s[1]["param"][0] = 0.1
    dirs = np.array([[5, 0, 0], [0, 5, 0], [0, 0, 5], [-5, 0, 0], [3, 3, 3.0]])
    p = np.zeros(len(dirs), PAIR_DTYPE)
    p["shape_b"] = 1
    p["rot"] = np.eye(3).ravel()
    p["trans"] = dirs
    o = oracle_lib.signed_distance(_batch(s, verts, p))
    expect = [4 - 0.1, 4 - 0.1, 4 - 0.1, 5 - 0.1, np.linalg.norm(dirs[4] - np.array([1, 1, 1]) / 3) - 0.1]
    assert np.allclose(o["distance"], expect, atol=1e-5)


def test_analytic_sphere_solvers_known_answers(oracle_lib):
    """The oracle's closed-form sphere solvers (oracle/orc_analytic.hpp, the
    ones fcl::collide dispatches to) against hand-computed contacts:
    sphere-sphere, sphere-box (face, edge, centre inside), sphere-capsule,
    sphere-cylinder (cap, barrel, inside) and reversed orders."""
    S, B, C, Y = SPHERE, BOX, CAPSULE, CYLINDER
    shapes = np.zeros(8, SHAPE_DTYPE)
    shapes["type"] = [S, S, B, C, Y, S, S, S]
    shapes["param"][0, 0] = 0.5                    # sphere r 0.5
    shapes["param"][1, 0] = 0.3                    # sphere r 0.3
    shapes["param"][2, :3] = [2.0, 2.0, 2.0]       # box, half extent 1
    shapes["param"][3, :2] = [0.2, 1.0]            # capsule r 0.2, lz 1
    shapes["param"][4, :2] = [0.4, 1.0]            # cylinder r 0.4, lz 1
    shapes["param"][5, 0] = 0.2
    shapes["param"][6, 0] = 0.2
    shapes["param"][7, 0] = 0.2
    cases = [
        # (a, b, trans of b, hit, depth, normal)
        (0, 1, [0.7, 0, 0], True, 0.1, [1, 0, 0]),          # sphere-sphere
        (0, 1, [0.81, 0, 0], False, None, None),
        (0, 2, [1.3, 0, 0], True, 0.2, [1, 0, 0]),          # sphere outside the box's -x face
        (0, 2, [0, 0, -1.3], True, 0.2, [0, 0, -1]),
        (0, 2, [0.8, 0.0, 0.0], True, 0.7, [1, 0, 0]),      # centre inside, nearest face -x: n into box = +x
        (2, 5, [1.1, 0, 0], True, 0.1, [1, 0, 0]),          # box-sphere (reversed), sphere beyond +x face
        (0, 3, [0.6, 0, 0.3], True, 0.1, [1, 0, 0]),        # sphere-capsule, barrel side
        (0, 3, [0, 0, 1.15], True, 0.05, [0, 0, 1]),        # sphere-capsule, end cap
        (0, 4, [0.8, 0, 0], True, 0.1, [1, 0, 0]),          # sphere-cylinder barrel
        (0, 4, [0, 0, 0.95], True, 0.05, [0, 0, 1]),        # sphere-cylinder cap
        (4, 6, [0.3, 0, 0], True, 0.3, [1, 0, 0]),          # cylinder-sphere, centre inside, nearer the barrel
    ]
    p = np.zeros(len(cases), PAIR_DTYPE)
    for i, (a, b, t, *_ ) in enumerate(cases):
        p[i]["shape_a"], p[i]["shape_b"] = a, b
        p[i]["rot"] = np.eye(3).ravel()
        p[i]["trans"] = t
    from fclg import workloads
    batch = workloads.Batch("analytic", shapes, np.zeros((0, 4), np.float32), p)
    r = oracle_lib.collide(batch, want_contact=True)
    assert np.all(r["gjk_status"] == 20)
    for i, (a, b, t, hit, depth, normal) in enumerate(cases):
        assert bool(r["ok"][i]) == hit, i
        if hit:
            assert abs(-r["distance"][i] - depth) < 1e-6, (i, r["distance"][i])  # FP32 inputs
            assert np.allclose(r["normal"][i], normal, atol=1e-6), (i, r["normal"][i])


def test_directed_penetration_pinned_to_reference(oracle_lib):
    """The restated MPR::DirectedPenetration against the reference's own
    RunDirectedPenetration (mpr.hpp:495-701) on random unit directions: the
    same status everywhere, bit-identical depth and witness points wherever it
    succeeds."""
    if not oracle_lib.ref_available():
        pytest.skip("reference build unavailable")
    from fclg import workloads
    for b in (workloads.mixed(6000, seed=31), workloads.pareto(4000, seed=32)):
        rng = np.random.default_rng(3)
        u = rng.normal(size=(b.n_pairs, 3))
        u = (u / np.linalg.norm(u, axis=1, keepdims=True)).astype(np.float32)
        o = oracle_lib.directed_raw(b, u, threads=2)
        r = oracle_lib.ref_directed(b, u, threads=2)
        assert np.array_equal(o["epa_status"], r["epa_status"])
        ok = o["epa_status"] == 0
        assert ok.mean() > 0.3
        assert np.array_equal(o["distance"][ok], r["distance"][ok])
        assert np.array_equal(o["p0"][ok], r["p0"][ok]) and np.array_equal(o["p1"][ok], r["p1"][ok])


def test_directed_penetration_properties(oracle_lib):
    """Depth along the EPA normal equals the EPA depth; along any direction it
    is no smaller than the minimum depth (fcl::collide, directed mode)."""
    from fclg import workloads
    b = workloads.mixed(8000, seed=33)
    sd = oracle_lib.signed_distance(b, threads=2)
    ov = (sd["distance"] < -1e-5) & (sd["epa_status"] == 1)
    r = oracle_lib.collide_directed(b, sd["normal"].astype(np.float32), threads=2)
    m = ov & (r["epa_status"] == 0)
    assert m.sum() > 1000
    err = np.abs(r["distance"][m] - sd["distance"][m])
    assert np.mean(err <= 1e-5) >= 0.99
    rng = np.random.default_rng(4)
    u = rng.normal(size=(b.n_pairs, 3))
    u = (u / np.linalg.norm(u, axis=1, keepdims=True)).astype(np.float32)
    r2 = oracle_lib.collide_directed(b, u, threads=2)
    m2 = ov & (r2["epa_status"] == 0)
    assert np.all(-r2["distance"][m2] >= -sd["distance"][m2] - 1e-6)
    assert np.array_equal(r2["ok"] == 1, oracle_lib.collide(b, threads=2)["ok"] == 1)


def test_incremental_penetration_pinned_to_reference(oracle_lib):
    """The restated incremental minimum-distance penetration against the
    reference's own RunIncrementalMinimumPenetrationDistance
    (mpr_incremental_penetration.hpp:176-288) from random unit hints: the same
    status everywhere, bit-identical depth, direction and witness points
    wherever the run is valid (OK or at its iteration limit)."""
    if not oracle_lib.ref_available():
        pytest.skip("reference build unavailable")
    from fclg import workloads
    for b in (workloads.mixed(6000, seed=34), workloads.pareto(4000, seed=35)):
        rng = np.random.default_rng(5)
        u = rng.normal(size=(b.n_pairs, 3))
        u = (u / np.linalg.norm(u, axis=1, keepdims=True)).astype(np.float32)
        o = oracle_lib.incremental_raw(b, u, threads=2)
        r = oracle_lib.ref_incremental(b, u, threads=2)
        assert np.array_equal(o["epa_status"], r["epa_status"])
        ok = o["ok"] == 1
        assert ok.mean() > 0.3
        for f in ("distance", "normal", "p0", "p1"):
            # a zero-area final portal (depth 0) gives NaN witnesses on both sides
            assert np.array_equal(o[f][ok], r[f][ok], equal_nan=True), f


def test_incremental_penetration_properties(oracle_lib):
    """fcl::collide, incremental mode: started on the EPA normal the run
    returns the EPA depth (within 1e-5 m for >= 99 %); from a random hint it
    descends to a direction whose depth is not below EPA's by more than
    1e-6 m for >= 99.9 % (the depth along any direction bounds the minimum
    from above; EPA's own depth on curved pairs is an estimate).
    The reference stops at the first converged subroutine
    (return_on_subroutine_converge), a local minimum over directions: about
    70 % of random hints end within 1e-4 m of EPA's global minimum."""
    from fclg import workloads
    b = workloads.mixed(8000, seed=36)
    sd = oracle_lib.signed_distance(b, threads=2)
    ov = (sd["distance"] < -1e-5) & (sd["epa_status"] == 1)
    r = oracle_lib.collide_incremental(b, sd["normal"].astype(np.float32), threads=2)
    m = ov & (r["ok"] == 1) & np.isin(r["epa_status"], (0, 4))
    assert m.sum() > 1000
    assert np.mean(np.abs(r["distance"][m] - sd["distance"][m]) <= 1e-5) >= 0.99
    rng = np.random.default_rng(6)
    u = rng.normal(size=(b.n_pairs, 3))
    u = (u / np.linalg.norm(u, axis=1, keepdims=True)).astype(np.float32)
    r2 = oracle_lib.collide_incremental(b, u, threads=2)
    m2 = ov & np.isin(r2["epa_status"], (0, 4))
    assert m2.mean() / ov.mean() > 0.95
    depth, epa = -r2["distance"][m2], -sd["distance"][m2]
    # EPA's depth on a curved pair is its last face's estimate, which the
    # incremental run can undercut on a rare pair
    assert np.mean(depth >= epa - 1e-6) >= 0.999
    assert np.mean(depth - epa <= 1e-4) >= 0.6
    assert np.array_equal(r2["ok"] == 1, oracle_lib.collide(b, threads=2)["ok"] == 1)
