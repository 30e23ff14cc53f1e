"""Broadphase feed: BinaryAABB_Tree::SelfCollision over CollisionObject AABBs
(broadphase/binary_AABB_tree-inl.h; narrowphase/collision_object-inl.h:
141-154), then the narrowphase on the candidate pairs.

CPU: the oracle's AABBs (FP64 restatement of computeAABB and computeBV<AABB>)
against closed forms; its brute-force pair set.
GPU: the library's boxes within FP32 rounding of the oracle's; its sort-and-
sweep pair set identical to brute force over the same (GPU) boxes and to the
oracle's pairs except boxes within 1e-5 m of touching; candidate records fed
to the distance query equal the oracle's relative poses.
"""
import numpy as np
import pytest

from fclg import workloads
from fclg.layout import BOX, CAPSULE, CYLINDER, SHAPE_DTYPE, SPHERE


def test_oracle_aabbs_closed_forms(oracle_lib):
    s = np.zeros(4, SHAPE_DTYPE)
    s["type"] = [BOX, SPHERE, CAPSULE, CYLINDER]
    s["param"][0, :3] = [2, 1, 0.5]
    s["param"][1, 0] = 0.3
    s["param"][2, :2] = [0.1, 0.6]
    s["param"][3, :2] = [0.2, 0.4]
    b = workloads.Batch("s", s, np.zeros((1, 4), np.float32), np.zeros(0, workloads.PAIR_DTYPE), {})
    eye = [1, 0, 0, 0, 1, 0, 0, 0, 1]
    c, sn = np.cos(0.3), np.sin(0.3)
    rz = [c, -sn, 0, sn, c, 0, 0, 0, 1]
    poses = np.array([eye + [1, 2, 3], rz + [1, 2, 3], eye + [0, 0, 0], eye + [0, 0, 1], rz + [0, 0, 0]], np.float32)
    ids = np.array([0, 0, 1, 2, 3], np.uint32)
    a = oracle_lib.object_aabbs(b, ids, poses)
    # identity: the local box translated
    assert np.allclose(a[0], [0, 1.5, 2.75, 2, 2.5, 3.25])
    # rotated: the cube of the local half diagonal about the moved centre
    r = np.sqrt(1 + 0.25 + 0.0625)
    assert np.allclose(a[1], [1 - r, 2 - r, 3 - r, 1 + r, 2 + r, 3 + r])
    assert np.allclose(a[2], [-0.3, -0.3, -0.3, 0.3, 0.3, 0.3])
    assert np.allclose(a[3], [-0.1, -0.1, 0.6, 0.1, 0.1, 1.4])
    r = np.sqrt(0.04 + 0.04 + 0.04)
    assert np.allclose(a[4], [-r, -r, -r, r, r, r])


def test_oracle_pairs_touching_counts(oracle_lib):
    boxes = np.array([[0, 0, 0, 1, 1, 1], [1, 0, 0, 2, 1, 1], [2.0001, 0, 0, 3, 1, 1], [0.5, 0.5, 1, 0.6, 0.6, 2]])
    pairs = {tuple(p) for p in oracle_lib.aabb_pairs(boxes)}
    assert pairs == {(0, 1), (0, 3)}
    assert {tuple(p) for p in oracle_lib.sweep_pairs(boxes)} == pairs


def test_oracle_sweep_equals_brute_force(oracle_lib):
    b, ids, poses = workloads.scene(3000, seed=5)
    boxes = oracle_lib.object_aabbs(b, ids, poses)
    brute = {tuple(p) for p in oracle_lib.aabb_pairs(boxes).tolist()}
    assert len(brute) > 500
    assert {tuple(p) for p in oracle_lib.sweep_pairs(boxes).tolist()} == brute


@pytest.mark.gpu
def test_gpu_broadphase_vs_oracle(oracle_lib):
    from fclg.api import Context, broadphase
    b, ids, poses = workloads.scene(20000, seed=workloads.SEED_BASE + 71)
    ctx = Context(0)
    try:
        ctx.set_batch(b)
        pairs, boxes = broadphase(ctx, ids, poses)
        ref = oracle_lib.object_aabbs(b, ids, poses)
        scale = 1 + np.abs(ref).max(axis=1, keepdims=True)
        assert np.all(np.abs(boxes.astype(np.float64) - ref) <= 2e-6 * scale)
        got = {tuple(p) for p in pairs.tolist()}
        assert len(got) == len(pairs) and all(i < j for i, j in got)
        # exact against brute force over the same boxes
        brute = {tuple(p) for p in oracle_lib.aabb_pairs(boxes.astype(np.float64)).tolist()}
        assert got == brute
        assert len(got) > 5000
        # against the FP64 boxes: differences only where boxes nearly touch
        r64 = {tuple(p) for p in oracle_lib.aabb_pairs(ref).tolist()}
        for i, j in got ^ r64:
            gap = np.max(np.maximum(ref[i, :3] - ref[j, 3:], ref[j, :3] - ref[i, 3:]))
            assert abs(gap) <= 1e-5
        # a capped call reports the total and a subset of the pairs
        import ctypes
        few = np.zeros((100, 2), np.uint32)
        total = ctypes.c_uint32(0)
        ctx._check(ctx.lib.fclg_broadphase(ctx.h, ids.ctypes.data_as(ctypes.c_void_p),
                                           poses.ctypes.data_as(ctypes.c_void_p), len(ids),
                                           few.ctypes.data_as(ctypes.c_void_p), 100, ctypes.byref(total), None),
                   "fclg_broadphase")
        assert total.value == len(got)
        assert {tuple(p) for p in few.tolist()} <= got
    finally:
        ctx.close()


@pytest.mark.gpu
def test_gpu_broadphase_feeds_the_narrowphase(oracle_lib):
    """Broadphase -> fclg_object_pairs_device -> fclg_distance_device, all on
    the device: the records equal the relative poses computed on the host and
    the distances match the oracle's on them."""
    import ctypes
    import torch
    from fclg.api import Context
    from fclg.layout import PAIR_DTYPE, RESULT_DTYPE
    from test_gpu_convex import check_parity
    b, ids, poses = workloads.scene(6000, seed=workloads.SEED_BASE + 72)
    ctx = Context(0)
    try:
        ctx.set_batch(b)
        d_ids = torch.from_numpy(ids.view(np.int32)).cuda()
        d_poses = torch.from_numpy(poses).cuda()
        cap = 1 << 16
        d_cand = torch.zeros(2 * cap, dtype=torch.int32, device="cuda")
        d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        vp = ctypes.c_void_p
        assert ctx.lib.fclg_broadphase_device(ctx.h, vp(d_ids.data_ptr()), vp(d_poses.data_ptr()), len(ids),
                                              vp(d_cand.data_ptr()), cap, vp(d_cnt.data_ptr()), None, None,
                                              None) == 0
        m = int(d_cnt.item())
        assert 0 < m <= cap
        d_pairs = torch.zeros(m * PAIR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        assert ctx.lib.fclg_object_pairs_device(ctx.h, vp(d_ids.data_ptr()), vp(d_poses.data_ptr()),
                                                vp(d_cand.data_ptr()), m, vp(d_pairs.data_ptr()), None) == 0
        d_res = torch.zeros(m * RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        ctx.distance_device(d_pairs.data_ptr(), m, d_res.data_ptr())
        torch.cuda.synchronize()
        rec = d_pairs.cpu().numpy().view(PAIR_DTYPE)
        cand = d_cand[:2 * m].cpu().numpy().view(np.uint32).reshape(-1, 2)
        P = poses.astype(np.float64)
        Ri, Rj = P[cand[:, 0], :9].reshape(-1, 3, 3), P[cand[:, 1], :9].reshape(-1, 3, 3)
        R = np.einsum("nki,nkj->nij", Ri, Rj)
        t = np.einsum("nki,nk->ni", Ri, P[cand[:, 1], 9:] - P[cand[:, 0], 9:])
        assert np.array_equal(rec["shape_a"], ids[cand[:, 0]]) and np.array_equal(rec["shape_b"], ids[cand[:, 1]])
        assert np.allclose(rec["rot"].reshape(-1, 3, 3), R, atol=1e-6)
        assert np.allclose(rec["trans"], t, atol=1e-5)
        q = workloads.Batch("cand", b.shapes, b.vertices, rec, {})
        got = d_res.cpu().numpy().view(RESULT_DTYPE)
        check_parity(got, oracle_lib.signed_distance(q), q)
    finally:
        ctx.close()


@pytest.mark.gpu
def test_gpu_broadphase_two_sets(oracle_lib):
    """TreeCollision / SingleObjectCollision: the pairs across two object sets
    equal the cross pairs of the joint self query."""
    import ctypes
    import torch
    from fclg.api import Context, broadphase
    b, ids, poses = workloads.scene(8000, seed=workloads.SEED_BASE + 73)
    na = 3000
    ctx = Context(0)
    try:
        ctx.set_batch(b)
        joint, _ = broadphase(ctx, ids, poses)
        want = {(int(i), int(j) - na) for i, j in joint.tolist() if i < na <= j}
        vp = ctypes.c_void_p
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        da, pa, db, pb = dev(ids[:na].view(np.int32)), dev(poses[:na]), dev(ids[na:].view(np.int32)), dev(poses[na:])
        cap = 1 << 16
        out = torch.zeros(2 * cap, dtype=torch.int32, device="cuda")
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        assert ctx.lib.fclg_broadphase_cross_device(ctx.h, vp(da.data_ptr()), vp(pa.data_ptr()), na,
                                                    vp(db.data_ptr()), vp(pb.data_ptr()), len(ids) - na,
                                                    vp(out.data_ptr()), cap, vp(cnt.data_ptr()), None) == 0
        m = int(cnt.item())
        got = {tuple(p) for p in out[:2 * m].cpu().numpy().reshape(-1, 2).tolist()}
        assert m == len(got) == len(want) and got == want and m > 100
        # a single object against the set
        assert ctx.lib.fclg_broadphase_cross_device(ctx.h, vp(da.data_ptr()), vp(pa.data_ptr()), 1,
                                                    vp(db.data_ptr()), vp(pb.data_ptr()), len(ids) - na,
                                                    vp(out.data_ptr()), cap, vp(cnt.data_ptr()), None) == 0
        m1 = int(cnt.item())
        one = {tuple(p) for p in out[:2 * m1].cpu().numpy().reshape(-1, 2).tolist()}
        assert one == {p for p in want if p[0] == 0}
    finally:
        ctx.close()
