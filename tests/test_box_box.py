"""fcl::collide on box pairs: the oracle's boxBox2 restatement
(primitive_shape_algorithm/box_box-inl.h) against the reference's own
box-box scenarios (test/test_fcl_box_box.cpp:203-457), in FP64 on posed boxes.

Each scenario runs, as the reference's BoxBoxTest does, for the six
orientations of the cube box 2 that leave it unchanged as a set (top, bottom,
back, front, left, right) and for both query orders; the expected contact
normal flips with the order.  The contact checked is the one a single-contact
request reports: the first of maximal depth (the partial sort by depth in
narrowphase/detail/shape_pair_intersect-inl.h:92-104).
"""
import numpy as np
import pytest


def aa(angle, axis):
    """Rotation matrix of angle about a unit axis (Rodrigues)."""
    k = np.asarray(axis, np.float64)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * (K @ K)


PI = np.pi
ISO = {"top": np.eye(3), "bottom": aa(PI, [1, 0, 0]), "back": aa(PI / 2, [1, 0, 0]),
       "front": aa(3 * PI / 2, [1, 0, 0]), "left": aa(PI / 2, [0, 1, 0]), "right": aa(3 * PI / 2, [0, 1, 0])}


def run_cases(oracle_lib, box1, box2, normal12, depth, pos_test, tol):
    (s1, R1, T1), (s2, R2, T2) = box1, box2
    for name, pre in ISO.items():
        R2p = R2 @ pre
        for order, (a, b, n_exp) in {"12": ((s1, R1, T1), (s2, R2p, T2), normal12),
                                     "21": ((s2, R2p, T2), (s1, R1, T1), -normal12)}.items():
            code, normal, d, contacts = oracle_lib.box_box(a[0], a[1], a[2], b[0], b[1], b[2])
            where = "%s %s" % (name, order)
            assert code != 0, where
            assert len(contacts) >= 1, where
            k = int(np.argmax(contacts[:, 3]))  # first of maximal depth
            assert abs(contacts[k, 3] - depth) <= tol, where
            assert np.allclose(normal, n_exp, rtol=0, atol=tol), where
            pos_test(contacts[k, :3], tol, where)


def test_box_box_all_contacts(oracle_lib):
    """test_fcl_box_box.cpp:203-290: unit cube tilted 45 deg about y sinking into
    the top face of a 3-cube; depth sqrt(2)/2, contact on the edge x = 0,
    z = -sqrt(2)/4."""
    box1 = (np.ones(3), aa(PI / 4, [0, 1, 0]), np.zeros(3))
    box2 = (np.full(3, 3.0), np.eye(3), np.array([0, 0, -1.5]))

    def pos_test(p, tol, where):
        assert abs(p[2] + np.sqrt(2) / 4) <= tol, where
        assert abs(p[0]) <= tol, where
        assert -0.5 <= p[1] <= 0.5, where

    run_cases(oracle_lib, box1, box2, np.array([0, 0, -1.0]), np.sqrt(2) / 2, pos_test, 1e-12)


def test_box_box_cull_contacts(oracle_lib):
    """test_fcl_box_box.cpp:297-379: an eight-sided contact polygon culled to
    four points; depth sqrt(2)/2 cos(pi/4 - pi/8) - 0.25, the contact on the
    segment y = -sqrt(2)/2 sin(pi/4 - pi/8), z = -0.25 - depth / 2."""
    tilt = PI / 8
    box1 = (np.ones(3), aa(tilt, [1, 0, 0]), np.zeros(3))
    box2 = (np.ones(3), aa(PI / 4, [0, 0, 1]), np.array([0, 0, -0.75]))
    depth = np.sqrt(2) / 2 * np.cos(PI / 4 - tilt) - 0.25

    def pos_test(p, tol, where):
        ey = -np.sqrt(2) / 2 * np.sin(PI / 4 - tilt)
        ex = np.sqrt(2) / 2 + ey + np.finfo(np.float64).eps
        assert abs(p[2] - (-0.25 - depth / 2)) <= tol, where
        assert abs(p[1] - ey) <= tol, where
        assert -ex <= p[0] <= ex, where

    run_cases(oracle_lib, box1, box2, np.array([0, 0, -1.0]), depth, pos_test, 1e-14)


def test_box_box_edge_contact(oracle_lib):
    """test_fcl_box_box.cpp:386-447: edge-edge contact (codes 7-15) of a cube
    turned 45 deg about z then -45 deg about y, pushed 0.1 into a unit cube."""
    d = np.array([np.sqrt(2) / 2, 0, np.sqrt(2) / 2])
    box1 = (np.ones(3), aa(-PI / 4, [0, 1, 0]) @ aa(PI / 4, [0, 0, 1]), d * (np.sqrt(2) - 0.1))
    box2 = (np.ones(3), np.eye(3), np.zeros(3))

    def pos_test(p, tol, where):
        want = d * (np.sqrt(2) / 2 - 0.05)
        assert np.linalg.norm(p - want) <= tol * max(np.linalg.norm(want), 1.0), where

    run_cases(oracle_lib, box1, box2, -d, 0.1, pos_test, 1e-14)


def test_box_box_separated_and_touching(oracle_lib):
    """Apart by 1 mm along x: no collision, the gap of the separating face axis;
    coincident boxes collide at full depth."""
    code, _, gap, contacts = oracle_lib.box_box(np.ones(3), np.eye(3), np.zeros(3), np.ones(3), np.eye(3),
                                                [1.001, 0, 0])
    assert code == 0 and len(contacts) == 0 and abs(gap - 0.001) < 1e-12
    code, normal, depth, contacts = oracle_lib.box_box([1, 2, 3], np.eye(3), np.zeros(3), [1, 2, 3], np.eye(3),
                                                       np.zeros(3))
    assert code in (1, 2, 3, 4, 5, 6) and abs(depth - 1.0) < 1e-12 and len(contacts) >= 1


def test_collide_batch_uses_box_box(oracle_lib):
    """The batch collide (shape a at the origin, b posed in a's frame) answers
    box pairs with boxBox2: the edge-contact scenario in a's frame."""
    from fclg import workloads
    from fclg.layout import BOX, PAIR_DTYPE, SHAPE_DTYPE
    d = np.array([np.sqrt(2) / 2, 0, np.sqrt(2) / 2])
    Ra = aa(-PI / 4, [0, 1, 0]) @ aa(PI / 4, [0, 0, 1])
    ta = d * (np.sqrt(2) - 0.1)
    s = np.zeros(2, SHAPE_DTYPE)
    s["type"] = BOX
    s["param"][:, :3] = 1.0
    p = np.zeros(1, PAIR_DTYPE)
    p["shape_a"], p["shape_b"] = 0, 1
    p["rot"] = Ra.T.ravel()                     # identity box b in a's frame
    p["trans"] = Ra.T @ (np.zeros(3) - ta)
    b = workloads.Batch("box", s, np.zeros((1, 4), np.float32), p, {})
    r = oracle_lib.collide(b, want_contact=True)
    assert r["ok"][0] == 1 and r["gjk_status"][0] == 20
    assert abs(r["distance"][0] + 0.1) < 1e-6
    assert np.allclose(Ra @ r["normal"][0], -d, atol=1e-6)
    pos = Ra @ (0.5 * (r["p0"][0] + r["p1"][0])) + ta
    assert np.allclose(pos, d * (np.sqrt(2) / 2 - 0.05), atol=1e-6)


def test_box_box_flags_and_depth_vs_sat(oracle_lib):
    """Random box pairs through the batch collide: the flag equals a plain
    15-axis separating-axis test outside a 1e-9 band, the contact normal is
    unit, and the contact depth is at most the separating-axis overlap along
    the reported normal (both to 1e-6: the FP32 rotations of the pair records
    are orthonormal to about 1e-7)."""
    from fclg import workloads
    from fclg.layout import BOX, PAIR_DTYPE, SHAPE_DTYPE
    rng = np.random.default_rng(21)
    n = 4000
    s = np.zeros(2, SHAPE_DTYPE)
    s["type"] = BOX
    s["param"][0, :3] = [2.0, 1.0, 0.5]
    s["param"][1, :3] = [1.0, 1.0, 1.0]
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                  2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                  2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], axis=1)
    p = np.zeros(n, PAIR_DTYPE)
    p["shape_a"], p["shape_b"] = 0, 1
    p["rot"] = R
    p["trans"] = rng.uniform(-1.6, 1.6, size=(n, 3))
    b = workloads.Batch("boxes", s, np.zeros((1, 4), np.float32), p, {})
    r = oracle_lib.collide(b, want_contact=True)
    Rf = p["rot"].astype(np.float64).reshape(-1, 3, 3)
    tf = p["trans"].astype(np.float64)
    ha, hb = np.array([1.0, 0.5, 0.25]), np.full(3, 0.5)
    hits = 0
    for i in range(n):
        axes = [np.eye(3)[k] for k in range(3)] + [Rf[i][:, k] for k in range(3)]
        axes += [np.cross(np.eye(3)[k], Rf[i][:, m]) for k in range(3) for m in range(3)]
        gap = -np.inf
        for ax in axes:
            nl = np.linalg.norm(ax)
            if nl < 1e-9:
                continue
            ax = ax / nl
            gap = max(gap, abs(ax @ tf[i]) - np.sum(ha * np.abs(ax)) - np.sum(hb * np.abs(Rf[i].T @ ax)))
        if abs(gap) < 1e-9:
            continue
        assert (r["ok"][i] == 1) == (gap < 0), i
        if gap < 0:
            hits += 1
            nrm = r["normal"][i]
            assert abs(np.linalg.norm(nrm) - 1) < 1e-6
            over = np.sum(ha * np.abs(nrm)) + np.sum(hb * np.abs(Rf[i].T @ nrm)) - abs(nrm @ tf[i])
            assert -r["distance"][i] <= over + 1e-6, i
    assert hits > 1000


def test_epa_depth_vs_box_box(oracle_lib):
    """test/cvx_collide/test_epa2_with_gjk2.cpp:75-161 (testBoxPenetration) at
    20 k poses: boxes of sides (2, 1, 0.5) and (1, 1, 1) at random poses in a
    4 m cube; wherever boxBox2 reports contacts, EPA's depth may not exceed
    boxBox2's separating-axis depth by more than 1e-4 (no mismatches)."""
    from fclg import workloads
    from fclg.layout import BOX, PAIR_DTYPE, SHAPE_DTYPE
    rng = np.random.default_rng(77)
    n = 20000

    def rot(k):
        q = rng.normal(size=(k, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        w, x, y, z = q.T
        return np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                         2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                         2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], axis=1).reshape(k, 3, 3)

    R1, R2 = rot(n), rot(n)
    t1, t2 = rng.uniform(-2, 2, size=(n, 3)), rng.uniform(-2, 2, size=(n, 3))
    # b in a's frame, rounded to the FP32 pair record; boxBox2 runs on the same rounded pose
    R = np.einsum("nji,njk->nik", R1, R2).astype(np.float32).astype(np.float64)
    t = np.einsum("nji,nj->ni", R1, t2 - t1).astype(np.float32).astype(np.float64)
    side1, side2 = np.array([2.0, 1.0, 0.5]), np.ones(3)
    sat_depth = np.full(n, np.nan)
    for i in range(n):
        code, _, depth, contacts = oracle_lib.box_box(side1, np.eye(3), np.zeros(3), side2, R[i], t[i])
        if len(contacts) > 0:
            sat_depth[i] = depth
    hit = np.nonzero(~np.isnan(sat_depth))[0]
    assert len(hit) > 1000
    s = np.zeros(2, SHAPE_DTYPE)
    s["type"] = BOX
    s["param"][0, :3] = side1
    s["param"][1, :3] = side2
    p = np.zeros(len(hit), PAIR_DTYPE)
    p["shape_a"], p["shape_b"] = 0, 1
    p["rot"] = R[hit].reshape(-1, 9)
    p["trans"] = t[hit]
    b = workloads.Batch("box_pen", s, np.zeros((1, 4), np.float32), p, {})
    o = oracle_lib.signed_distance(b)
    ok = (o["ok"] == 1) & (o["distance"] < 0)
    epa = -o["distance"]
    mismatch = ok & (np.abs(sat_depth[hit] - epa) > 1e-4) & (sat_depth[hit] < epa)
    assert mismatch.sum() == 0
    assert ok.mean() > 0.99
