"""The mesh-mesh path pinned to the reference itself.

CPU (no GPU):
  * the oracle's FP64 restatement of BVHModel<OBBRSS<double>>::endModel
    (oracle/orc_mesh.hpp buildRefTree) is bit-identical to the reference's own
    build compiled from its sources (oracle/_ref/libfcl_ref_mesh.so): every
    node's OBB axes, centre, extents, |extent|^2, children and primitive range;
  * the restated MeshIntersect over that tree reports the reference's contact
    lists, in the reference's order, for caps 1, 64 and "all";
  * the restatement reproduces the golden lists of tests/golden/mesh_ref.npz
    (the reference's own outputs on its test meshes env.obj / rob.obj and on
    bumpy spheres of the mesh-mesh workload's kind);
  * the library's host build (fclg_bvh_build, fclg_bvh_node_sizes) gives the
    reference's tree: same children and leaf triangles in every slot, the
    same FP64 |extent|^2 per node (the traversal's descend key), FP32 boxes
    that contain their triangles;
  * the reference's test_mesh_mesh property (test_fcl_collision.cpp:318-360):
    the contact set of the full request equals every colliding triangle pair
    (brute force);
  * MeshShapeIntersect (mesh against sphere, box, capsule, cylinder, hull):
    the restatement (oracle/orc_mesh_shape.hpp) over the library's tree gives
    the compiled reference's ordered triangle lists and the golden ones.
The GPU side (tests/test_mesh.py, tests/test_mesh_shape.py) checks the kernels
against the same lists.
"""
import os

import numpy as np
import pytest

from fclg import workloads

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mesh_ref.npz")
CASES = ("env_rob", "spheres")
ALL = 1 << 30


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN))


def _case(g, name):
    a = (g[name + "/va"].astype(np.float64), g[name + "/ta"])
    b = (g[name + "/vb"].astype(np.float64), g[name + "/tb"])
    return a, b, g[name + "/poses"]


def _lists(counts, flat):
    off = np.concatenate([[0], np.cumsum(counts)])
    return [flat[off[i]:off[i + 1]] for i in range(len(counts))]


def _need_ref(oracle_lib):
    if not oracle_lib.ref_mesh_available():
        pytest.skip("reference sources not available: oracle/_ref/libfcl_ref_mesh.so not built")


@pytest.mark.parametrize("name", CASES)
def test_restated_tree_equals_reference(oracle_lib, golden, name):
    _need_ref(oracle_lib)
    a, b, _ = _case(golden, name)
    for mesh in (a, b):
        rf, ri = oracle_lib.ref_tree(*mesh)
        of, oi, _ = oracle_lib.orc_tree(*mesh)
        assert np.array_equal(ri, oi)
        assert np.array_equal(rf.view(np.uint64), of.view(np.uint64))  # bit for bit


@pytest.mark.parametrize("name", CASES)
def test_restated_traversal_equals_reference(oracle_lib, golden, name):
    _need_ref(oracle_lib)
    a, b, poses = _case(golden, name)
    # poses other than the golden ones: rotate the golden set's translations
    P = poses.astype(np.float64).copy()
    P[:, 9:] = np.roll(P[:, 9:], 7, axis=0) * 0.9
    for cap in (1, 64, ALL):
        stride = 64 if cap != ALL else 8192
        rc, rp = oracle_lib.ref_mesh_collide(a, b, P[:64], cap, stride=stride)
        oc, op = oracle_lib.orc_mesh_collide_ref(a, b, P[:64], cap, stride=stride)
        assert np.array_equal(rc, oc)
        assert rc.max() <= stride
        assert np.array_equal(rp, op)


@pytest.mark.parametrize("name", CASES)
def test_restated_traversal_equals_golden(oracle_lib, golden, name):
    a, b, poses = _case(golden, name)
    for tag, cap, n in (("cap1", 1, len(poses)), ("cap64", 64, len(poses)), ("all", ALL, 48)):
        counts = golden["%s/%s/counts" % (name, tag)]
        want = _lists(counts, golden["%s/%s/pairs" % (name, tag)])
        stride = max(int(counts.max()), 1)
        oc, op = oracle_lib.orc_mesh_collide_ref(a, b, poses[:n].astype(np.float64), cap, stride=stride)
        assert np.array_equal(oc, counts)
        for i in range(n):
            assert np.array_equal(op[i, :oc[i]], want[i])
    assert golden[name + "/cap1/counts"].sum() > 0.3 * len(poses)


@pytest.mark.parametrize("name", CASES)
def test_library_build_is_the_reference_tree(golden, name):
    from fclg.api import bvh_build, bvh_node_sizes
    for side in ("a", "b"):
        v = golden["%s/v%s" % (name, side)]
        t = golden["%s/t%s" % (name, side)]
        ref_i32 = golden["%s/tree_%s_i32" % (name, side)]
        ref_size = golden["%s/tree_%s_size" % (name, side)]
        nodes, soup = bvh_build(v, t)
        sizes, depth = bvh_node_sizes(v, t)
        assert len(nodes) == len(ref_i32)
        internal = ref_i32[:, 0] >= 0
        assert np.array_equal(nodes["child"][internal], ref_i32[internal, 0])
        assert np.array_equal(nodes["child"][~internal], ref_i32[~internal, 0])  # -(triangle + 1)
        assert np.array_equal(sizes.view(np.uint64), ref_size.view(np.uint64))
        assert 0 < depth < 40
        # every FP32 box holds its triangles (leaf boxes checked directly, inner
        # boxes through their leaves' triangles)
        first = ref_i32[:, 1]
        count = ref_i32[:, 2]
        leaf_tri = np.full(len(nodes), -1)
        leaf_tri[~internal] = -(ref_i32[~internal, 0] + 1)
        # primitive order after the build: leaves in slot order give each node's block
        order = np.zeros(len(t), np.int64)
        order[first[~internal]] = leaf_tri[~internal]
        for i in range(0, len(nodes), max(1, len(nodes) // 400)):
            tri = order[first[i]:first[i] + count[i]]
            pts = soup[tri, :, :3].reshape(-1, 3).astype(np.float64)
            A = nodes[i]["axis"].reshape(3, 3).astype(np.float64)
            loc = (pts - nodes[i]["center"].astype(np.float64)) @ A
            assert np.all(np.abs(loc) <= nodes[i]["extent"].astype(np.float64))


def test_reference_full_request_is_every_colliding_pair(oracle_lib, golden):
    _need_ref(oracle_lib)
    a, b, poses = _case(golden, "env_rob")
    soup = lambda m: np.concatenate([m[0][m[1]].astype(np.float32), np.zeros((len(m[1]), 3, 1), np.float32)], 2)
    sa, sb = soup(a), soup(b)
    rc, rp = oracle_lib.ref_mesh_collide(a, b, poses[:48].astype(np.float64), ALL, stride=2048)
    hits = 0
    for i in range(48):
        bf = oracle_lib.mesh_allpairs(sa, sb, poses[i])
        assert set(map(tuple, bf)) == set(map(tuple, rp[i, :rc[i]]))
        hits += rc[i] > 0
    assert hits > 10


def test_restated_traversal_c2_sized(oracle_lib):
    """Full-size bumpy spheres (2 x 50k triangles): restated tree and lists
    equal the compiled reference's on a few poses."""
    _need_ref(oracle_lib)
    ma, mb = workloads.mesh_pair()
    a = (ma.vertices.astype(np.float64), ma.triangles)
    b = (mb.vertices.astype(np.float64), mb.triangles)
    rf, ri = oracle_lib.ref_tree(*a)
    of, oi, _ = oracle_lib.orc_tree(*a)
    assert np.array_equal(ri, oi) and np.array_equal(rf.view(np.uint64), of.view(np.uint64))
    poses = workloads.mesh_poses(24, seed=workloads.SEED_BASE + 40).astype(np.float64)
    for cap in (1, 64):
        rc, rp = oracle_lib.ref_mesh_collide(a, b, poses, cap)
        oc, op = oracle_lib.orc_mesh_collide_ref(a, b, poses, cap)
        assert np.array_equal(rc, oc) and np.array_equal(rp, op)


def _mesh_shape_case(g):
    from fclg.api import bvh_build
    b = workloads.Batch("mesh_shapes", g["mesh_shape/shapes"], g["mesh_shape/vertices"],
                        np.zeros(0, workloads.PAIR_DTYPE), {})
    nodes, soup = bvh_build(g["spheres/va"], g["spheres/ta"])
    return b, nodes, soup, g["mesh_shape/ids"], g["mesh_shape/poses"]


def test_restated_mesh_shape_equals_golden(oracle_lib, golden):
    """MeshShapeIntersect restated (oracle/orc_mesh_shape.hpp) over the
    library's tree (the reference's own) gives the reference's golden lists:
    triangle ids in order, caps 1 and 16 and every contact."""
    b, nodes, soup, ids, poses = _mesh_shape_case(golden)
    every = np.arange(len(ids)) % 6 == 0
    for tag, cap, sel in (("cap1", 1, slice(None)), ("cap16", 16, slice(None)), ("all", 0, every)):
        counts = golden["mesh_shape/%s/counts" % tag]
        want = _lists(counts, golden["mesh_shape/%s/tris" % tag])
        pc = max(int(counts.max()), 1)
        f, c, t = oracle_lib.mesh_shape_collide(nodes, soup, b, ids[sel], poses[sel], max_contacts=cap, pair_cap=pc)
        assert np.array_equal(c.astype(np.int32), counts)
        for i in range(len(counts)):
            assert np.array_equal(t[i, :c[i]], want[i]), (tag, i)


def test_restated_mesh_shape_equals_reference(oracle_lib, golden):
    """The same against the compiled reference on other poses, every shape type."""
    _need_ref(oracle_lib)
    b, nodes, soup, _, _ = _mesh_shape_case(golden)
    mesh = (golden["spheres/va"].astype(np.float64), golden["spheres/ta"])
    for k in range(len(b.shapes)):
        P = workloads.mesh_poses(6, max_dist=0.7, seed=workloads.SEED_BASE + 500 + k)
        for cap in (1, 16):
            rc, rt = oracle_lib.ref_mesh_shape_collide(mesh, b, k, P.astype(np.float64), cap)
            f, c, t = oracle_lib.mesh_shape_collide(nodes, soup, b, np.full(len(P), k, np.uint32), P,
                                                    max_contacts=cap)
            assert np.array_equal(c.astype(np.int32), rc)
            for i in range(len(P)):
                assert np.array_equal(t[i, :c[i]], rt[i, :rc[i]]), (k, cap, i)
