"""Mesh-mesh BVH collision (OBB hierarchy, boolean contacts).

CPU: the host BVH build (every triangle inside every box on its root path;
2 n - 1 nodes) and the FP64 oracle's traversal (the restated
OrientedNodeBVHSolver::MeshIntersect, bvh_solver-inl.h:74-164) against brute
force over all triangle pairs, plus the oracle's triangle-triangle test
against an independent interval-overlap test.

GPU: the warp-per-pose kernel through the C ABI against the restated
reference traversal over the reference's own tree (oracle/orc_mesh.hpp
meshIntersectRef, pinned to the compiled reference by tests/test_mesh_ref.py)
and against the reference's own golden lists: per pose the contact count and
the ordered (b1, b2) list identical, for first contact, a cap of 64, a cap
above the shared-memory buffer and every contact.
"""
import os

import numpy as np
import pytest

from fclg import workloads


@pytest.fixture(scope="module")
def small_meshes():
    from fclg.api import bvh_build
    a = workloads.geodesic_sphere(10, 0.3, 0.05, seed=1)
    b = workloads.geodesic_sphere(8, 0.3, 0.05, seed=2)
    na, ta = bvh_build(a.vertices, a.triangles)
    nb, tb = bvh_build(b.vertices, b.triangles)
    return a, b, (na, ta), (nb, tb)


def _ancestors(nodes):
    parent = np.full(len(nodes), -1)
    for i, n in enumerate(nodes):
        if n["child"] >= 0:
            parent[n["child"]] = i
            parent[n["child"] + 1] = i
    return parent


def test_bvh_contains_triangles(small_meshes):
    for nodes, tris in (small_meshes[2], small_meshes[3]):
        assert len(nodes) == 2 * len(tris) - 1
        parent = _ancestors(nodes)
        leaves = np.nonzero(nodes["child"] < 0)[0]
        assert sorted(-(nodes["child"][leaves] + 1)) == list(range(len(tris)))
        for i in leaves:
            pts = tris[-(nodes["child"][i] + 1), :, :3].astype(np.float64)
            j = i
            while j >= 0:
                A = nodes[j]["axis"].reshape(3, 3).astype(np.float64)
                loc = (pts - nodes[j]["center"].astype(np.float64)) @ A
                assert np.all(np.abs(loc) <= nodes[j]["extent"].astype(np.float64))
                j = parent[j]


def test_oracle_traversal_equals_brute_force(oracle_lib, small_meshes):
    _, _, (na, ta), (nb, tb) = small_meshes
    poses = workloads.mesh_poses(120, seed=5)
    flags, counts, pairs = oracle_lib.mesh_collide(na, ta, nb, tb, poses, max_contacts=0, pair_cap=4096)
    assert 0.2 < flags.mean() < 0.95
    for i in range(len(poses)):
        bf = oracle_lib.mesh_allpairs(ta, tb, poses[i])
        assert set(map(tuple, bf)) == set(map(tuple, pairs[i, :counts[i]]))
    f1, _, p1 = oracle_lib.mesh_collide(na, ta, nb, tb, poses, max_contacts=1)
    assert np.array_equal(f1, flags)


def _intervals_overlap_tri_tri(P, Q):
    """Independent check: triangles intersect iff no separating axis among the
    edge-edge cross products, the two normals and the in-plane edge normals,
    evaluated here in numpy with np.cross (touching counts as intersecting)."""
    e = [P[1] - P[0], P[2] - P[1], P[0] - P[2]]
    f = [Q[1] - Q[0], Q[2] - Q[1], Q[0] - Q[2]]
    n = np.cross(e[0], e[1])
    m = np.cross(f[0], f[1])
    axes = [n, m] + [np.cross(a, b) for a in e for b in f] + [np.cross(a, n) for a in e] + [np.cross(b, m) for b in f]
    for ax in axes:
        p = P @ ax
        q = Q @ ax
        if p.min() > q.max() or q.min() > p.max():
            return False
    return True


def test_tri_tri_vs_independent(oracle_lib):
    rng = np.random.default_rng(9)
    agree = 0
    for _ in range(3000):
        P = rng.random((3, 3))
        Q = rng.random((3, 3)) * 0.8 + rng.random(3) * 0.5
        pose = np.concatenate([np.eye(3).ravel(), np.zeros(3)])
        got = oracle_lib.tri_tri(P, Q, pose)
        assert got == _intervals_overlap_tri_tri(P, Q)
        agree += 1
    assert agree == 3000


def _gpu_lists(ctx, va, ta, vb, tb, poses, cap):
    from fclg.api import GpuMesh, mesh_collide
    ga, gb = GpuMesh(ctx, va, ta), GpuMesh(ctx, vb, tb)
    try:
        f, c, p, st = mesh_collide(ctx, ga, gb, poses, max_contacts=cap)
    finally:
        ga.close()
        gb.close()
    assert np.all(st == 0)
    assert np.array_equal(f, (c > 0).astype(np.uint8))
    return c, p


def _check_gpu_vs_oracle(oracle_lib, ctx, mesh_a, mesh_b, poses, caps=(1, 64)):
    """The kernel's contact lists equal, pose by pose and in order, the
    restated reference traversal's over the reference's own tree."""
    A = (mesh_a.vertices.astype(np.float64), mesh_a.triangles)
    B = (mesh_b.vertices.astype(np.float64), mesh_b.triangles)
    rate = None
    for cap in caps:
        c, p = _gpu_lists(ctx, mesh_a.vertices, mesh_a.triangles, mesh_b.vertices, mesh_b.triangles, poses, cap)
        oc, op = oracle_lib.orc_mesh_collide_ref(A, B, poses.astype(np.float64), cap)
        assert np.array_equal(c.astype(np.int32), oc)
        for i in range(len(poses)):
            assert np.array_equal(p[i, :c[i]], op[i, :oc[i]]), (cap, i)
        if rate is None:
            rate = (c > 0).mean()
    return rate


@pytest.mark.gpu
def test_gpu_mesh_small_vs_oracle(gpu_ctx, oracle_lib):
    a = workloads.geodesic_sphere(10, 0.3, 0.05, seed=1)
    b = workloads.geodesic_sphere(8, 0.3, 0.05, seed=2)
    rate = _check_gpu_vs_oracle(oracle_lib, gpu_ctx, a, b, workloads.mesh_poses(1500, seed=6), caps=(1, 64, 200))
    assert 0.2 < rate < 0.95


@pytest.mark.gpu
def test_gpu_mesh_full_size_vs_oracle(gpu_ctx, oracle_lib):
    a, b = workloads.mesh_pair()
    rate = _check_gpu_vs_oracle(oracle_lib, gpu_ctx, a, b, workloads.mesh_poses(600, seed=7))
    assert 0.2 < rate < 0.99


@pytest.mark.gpu
@pytest.mark.parametrize("name", ("env_rob", "spheres"))
def test_gpu_mesh_reference_golden(gpu_ctx, name):
    """The reference's own contact lists (tests/golden/mesh_ref.npz: its test
    meshes env.obj / rob.obj and bumpy spheres), first contact, cap 64 and
    every contact: counts and ordered (b1, b2) lists identical."""
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mesh_ref.npz"))
    va, ta, vb, tb = (g[name + "/" + k] for k in ("va", "ta", "vb", "tb"))
    poses = g[name + "/poses"]
    for tag, cap, n in (("cap1", 1, len(poses)), ("cap64", 64, len(poses)), ("all", None, 48)):
        counts = g["%s/%s/counts" % (name, tag)]
        flat = g["%s/%s/pairs" % (name, tag)]
        cap = cap or max(int(counts.max()), 1)
        c, p = _gpu_lists(gpu_ctx, va, ta, vb, tb, poses[:n], cap)
        assert np.array_equal(c.astype(np.int32), counts)
        off = np.concatenate([[0], np.cumsum(counts)])
        for i in range(n):
            assert np.array_equal(p[i, :c[i]], flat[off[i]:off[i + 1]]), (tag, i)


@pytest.mark.gpu
def test_gpu_mesh_edge_cases(gpu_ctx):
    from fclg.api import FclgError, GpuMesh, mesh_collide
    a = workloads.geodesic_sphere(4, 0.3, 0.0)
    ga = GpuMesh(gpu_ctx, a.vertices, a.triangles)
    # far apart: no contact; identical pose: contact
    poses = np.zeros((2, 12), np.float32)
    poses[:, :9] = np.eye(3).ravel()
    poses[0, 9] = 5.0
    f, c, p, st = mesh_collide(gpu_ctx, ga, ga, poses, max_contacts=4)
    assert f[0] == 0 and c[0] == 0 and f[1] == 1 and c[1] == 4
    with pytest.raises(FclgError):
        GpuMesh(gpu_ctx, a.vertices, np.array([[0, 1, 10 ** 6]], np.int32))
    ga.close()
