"""Writes tests/golden/mesh_ref.npz: mesh-mesh inputs with the outputs of the
reference itself — its BVHModel<OBBRSS<double>> tree and
OrientedNodeBVHSolver::MeshIntersect contact lists, compiled from the
reference sources into oracle/_ref by oracle/build_ref.sh.  Run where the
reference sources exist (REF_ROOT, else the recipe's default checkout):

    python tests/golden/make_mesh_golden.py

Cases:
  env_rob   the reference's own test meshes test/fcl_resources/env.obj and
            rob.obj (test_fcl_collision.cpp: test_mesh_mesh), vertices rounded
            to FP32 (the library's input type), with 96 seeded poses: 48 in the
            reference test's translation box [-3000, 3000]^2 x [0, 3000], 48
            within 1500 of the origin, uniform rotations;
  spheres   two bumpy geodesic spheres of the mesh-mesh workload's kind at a
            smaller frequency (16: 5120 triangles each; radius 0.3 m, radial
            noise 0.05 m), 192 poses within 0.8 m.
For each case and each cap in (1, 64): per pose the contact count and the
(b1, b2) triangle pairs in the reference's order, stored flat (the counts give
the offsets); every contact ("all") for the first 48 poses of each case.
The reference receives the FP32 vertices and poses as doubles.

mesh_shape: the spheres case's first mesh against 40 shapes (8 each of
sphere, box, capsule, cylinder and convex hull of the mixed workload's kind)
at 12 poses each within 0.6 m of the mesh centre: the reference's
MeshShapeIntersect contact lists (triangle ids) for caps 1 and 16, and every
contact for each sixth query.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "mind-fcl_gb300"))

import oracle  # noqa: E402
from fclg import workloads  # noqa: E402

ALL = 1 << 30  # "every contact": a cap no pose reaches


def load_obj(path):
    """Vertices and triangles of a Wavefront OBJ file (v / f records; faces
    with more than three corners are fanned; 1-based indices, '/'-suffixes
    ignored)."""
    verts, tris = [], []
    with open(path) as fh:
        for line in fh:
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "v":
                verts.append([float(x) for x in tok[1:4]])
            elif tok[0] == "f":
                idx = [int(t.split("/")[0]) - 1 for t in tok[1:]]
                for k in range(1, len(idx) - 1):
                    tris.append([idx[0], idx[k], idx[k + 1]])
    return np.array(verts, np.float32), np.array(tris, np.int32)


def poses_in_box(rng, n, lo, hi):
    R = workloads.random_rotations(rng, n)
    t = lo + (hi - lo) * rng.random((n, 3))
    return np.concatenate([R, t], axis=1).astype(np.float32)


def main():
    oracle.build()
    if not oracle.ref_mesh_available():
        raise SystemExit("oracle/_ref/libfcl_ref_mesh.so missing: the reference sources are needed")
    ref_root = os.environ.get("REF_ROOT", "/root/reference")
    res = os.path.join(ref_root, "test", "fcl_resources")
    rng = np.random.default_rng(20240655)
    env = load_obj(os.path.join(res, "env.obj"))
    rob = load_obj(os.path.join(res, "rob.obj"))
    poses_er = np.concatenate([
        poses_in_box(rng, 48, np.array([-3000.0, -3000.0, 0.0]), np.array([3000.0, 3000.0, 3000.0])),
        poses_in_box(rng, 48, np.array([-1500.0, -1500.0, -1500.0]), np.array([1500.0, 1500.0, 1500.0]))])
    sa = workloads.geodesic_sphere(16, 0.3, 0.05, seed=workloads.SEED_BASE + 31)
    sb = workloads.geodesic_sphere(16, 0.3, 0.05, seed=workloads.SEED_BASE + 32)
    poses_sp = workloads.mesh_poses(192, max_dist=0.8, seed=workloads.SEED_BASE + 33)
    out = {}
    for name, a, b, poses in (("env_rob", env, rob, poses_er),
                              ("spheres", (sa.vertices, sa.triangles), (sb.vertices, sb.triangles), poses_sp)):
        out[name + "/va"], out[name + "/ta"] = a
        out[name + "/vb"], out[name + "/tb"] = b
        out[name + "/poses"] = poses
        A = (a[0].astype(np.float64), a[1])
        B = (b[0].astype(np.float64), b[1])
        for side, M in (("a", A), ("b", B)):
            f64, i32 = oracle.ref_tree(*M)
            out["%s/tree_%s_i32" % (name, side)] = i32
            out["%s/tree_%s_size" % (name, side)] = f64[:, 15]
        P_all = poses.astype(np.float64)
        for cap, tag in ((1, "cap1"), (64, "cap64"), (ALL, "all")):
            P = P_all[:48] if cap == ALL else P_all
            stride = cap if cap != ALL else 1
            counts, _ = oracle.ref_mesh_collide(A, B, P, cap, stride=stride)
            stride = max(int(counts.max()), 1)
            counts, pairs = oracle.ref_mesh_collide(A, B, P, cap, stride=stride)
            flat = np.concatenate([pairs[i, :counts[i]] for i in range(len(P))] + [np.zeros((0, 2), np.int32)])
            out["%s/%s/counts" % (name, tag)] = counts
            out["%s/%s/pairs" % (name, tag)] = flat.astype(np.int32)
            print(name, tag, "colliding poses", int((counts > 0).sum()), "of", len(P), "contacts", int(counts.sum()))
    # mesh against shapes
    from fclg.layout import BOX, CAPSULE, CONVEX, CYLINDER, SPHERE
    shapes = workloads.mixed(4000, seed=workloads.SEED_BASE + 34)
    sel = np.concatenate([np.nonzero(shapes.shapes["type"] == t)[0][:8] for t in (SPHERE, BOX, CAPSULE, CYLINDER,
                                                                                 CONVEX)])
    ids = np.repeat(sel, 12).astype(np.uint32)
    poses = workloads.mesh_poses(len(ids), max_dist=0.6, seed=workloads.SEED_BASE + 35)
    M = (sa.vertices.astype(np.float64), sa.triangles)
    every = np.arange(len(ids)) % 6 == 0
    for cap, tag in ((1, "cap1"), (16, "cap16"), (ALL, "all")):
        counts = np.zeros(len(ids), np.int32)
        lists = []
        for sid in sel:
            q = np.nonzero((ids == sid) & (every if cap == ALL else True))[0]
            if len(q) == 0:
                continue
            c, _ = oracle.ref_mesh_shape_collide(M, shapes, int(sid), poses[q].astype(np.float64), cap, stride=1)
            st = max(int(c.max()), 1)
            c, t = oracle.ref_mesh_shape_collide(M, shapes, int(sid), poses[q].astype(np.float64), cap, stride=st)
            counts[q] = c
            lists += [(qi, t[j, :c[j]]) for j, qi in enumerate(q)]
        lists.sort(key=lambda x: x[0])
        if cap == ALL:
            counts = counts[every]
        out["mesh_shape/%s/counts" % tag] = counts
        out["mesh_shape/%s/tris" % tag] = np.concatenate([l for _, l in lists] + [np.zeros(0, np.int32)]).astype(
            np.int32)
        print("mesh_shape", tag, "colliding", int((counts > 0).sum()), "of", len(ids), "contacts", int(counts.sum()))
    # the 40 shapes alone, their hull vertices packed
    sh = shapes.shapes[sel].copy()
    verts = []
    off = 0
    for k, sid in enumerate(sel):
        s0 = shapes.shapes[sid]
        if s0["type"] == CONVEX:
            verts.append(shapes.vertices[s0["vert_offset"]:s0["vert_offset"] + s0["vert_count"]])
            sh["vert_offset"][k] = off
            off += int(s0["vert_count"])
    out["mesh_shape/shapes"] = sh
    out["mesh_shape/vertices"] = np.concatenate(verts).astype(np.float32)
    remap = {int(sid): k for k, sid in enumerate(sel)}
    out["mesh_shape/ids"] = np.array([remap[int(i)] for i in ids], np.uint32)
    out["mesh_shape/poses"] = poses
    np.savez_compressed(os.path.join(HERE, "mesh_ref.npz"), **out)
    print("wrote", os.path.join(HERE, "mesh_ref.npz"))


if __name__ == "__main__":
    main()
