"""ORACLE — test infrastructure only.

ctypes access to the FP64 CPU restatement of mind-fcl's convex query engine
(oracle/orc_convex.hpp, built into oracle/liboracle.so) and, where it was
built, to the reference itself (oracle/_ref/libfcl_ref.so, see
oracle/build_ref.sh).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this package; the product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libfcl_ref.so")
REF_MESH_PATH = os.path.join(HERE, "_ref", "libfcl_ref_mesh.so")

RESULT_DTYPE = np.dtype(
    [("distance", "<f8"), ("p0", "<f8", (3,)), ("p1", "<f8", (3,)), ("normal", "<f8", (3,)),
     ("ok", "<i4"), ("gjk_status", "<i4"), ("epa_status", "<i4"), ("gjk_iters", "<i4"),
     ("epa_iters", "<i4"), ("reserved", "<i4")]
)
assert RESULT_DTYPE.itemsize == 104

_CXXFLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared"]


def build(force=False):
    """Compile the restatement (always) and the reference driver (only where the
    reference sources exist)."""
    srcs = [os.path.join(HERE, f) for f in ("oracle.cpp", "orc_convex.hpp", "orc_mesh.hpp", "orc_analytic.hpp",
                                            "orc_mesh_shape.hpp", "orc_ccd.hpp") if
            os.path.exists(os.path.join(HERE, f))]
    if force or not os.path.exists(LIB_PATH) or any(os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in srcs):
        subprocess.check_call(["g++", *_CXXFLAGS, os.path.join(HERE, "oracle.cpp"), "-o", LIB_PATH, "-lpthread"])
    # the recipe decides where the reference sources are and skips when absent
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")])


_lib = None
_ref = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = ctypes.CDLL(LIB_PATH)
        vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        lib.orc_signed_distance.argtypes = [vp, i, vp, vp, i, vp, vp, i, i, d, i, i, d]
        lib.orc_signed_distance.restype = i
        lib.orc_collide.argtypes = [vp, i, vp, vp, i, i, i, vp, i]
        lib.orc_collide_directed.argtypes = [vp, i, vp, vp, i, vp, vp, i]
        lib.orc_collide_directed.restype = i
        lib.orc_directed_raw.argtypes = [vp, i, vp, vp, i, vp, vp, i]
        lib.orc_directed_raw.restype = i
        lib.orc_collide_incremental.argtypes = [vp, i, vp, vp, i, vp, vp, i]
        lib.orc_collide_incremental.restype = i
        lib.orc_incremental_raw.argtypes = [vp, i, vp, vp, i, vp, vp, i]
        lib.orc_incremental_raw.restype = i
        lib.orc_collide.restype = i
        lib.orc_time_signed_distance.argtypes = [vp, i, vp, vp, i, vp, i]
        lib.orc_time_signed_distance.restype = d
        lib.orc_mesh_collide.argtypes = [vp, vp, vp, vp, vp, i, i, i, vp, vp, vp, i]
        lib.orc_mesh_collide.restype = i
        lib.orc_mesh_allpairs.argtypes = [vp, i, vp, i, vp, vp, i]
        lib.orc_mesh_allpairs.restype = i
        lib.orc_ref_tree.argtypes = [vp, vp, i, vp, vp, vp]
        lib.orc_ref_tree.restype = i
        lib.orc_ref_mesh_collide.argtypes = [vp, vp, i, vp, vp, i, vp, i, i, vp, vp, i, i]
        lib.orc_ref_mesh_collide.restype = i
        lib.orc_tri_tri.argtypes = [vp, vp, vp]
        lib.orc_tri_tri.restype = i
        lib.orc_set_walk.argtypes = [vp, i, vp]
        lib.orc_set_walk.restype = None
        lib.orc_support.argtypes = [vp, i, vp, i, vp, i, vp]
        lib.orc_support.restype = i
        lib.orc_box_box.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        lib.orc_box_box.restype = i
        lib.orc_mesh_shape_collide.argtypes = [vp, vp, vp, i, vp, vp, vp, i, i, i, vp, vp, vp, i]
        lib.orc_mesh_shape_collide.restype = i
        lib.orc_mesh_shape_all.argtypes = [vp, i, vp, i, vp, ctypes.c_uint32, vp, vp, i]
        lib.orc_mesh_shape_all.restype = i
        lib.orc_object_aabbs.argtypes = [vp, i, vp, vp, vp, i, vp]
        lib.orc_object_aabbs.restype = i
        lib.orc_aabb_pairs.argtypes = [vp, i, vp, i]
        lib.orc_aabb_pairs.restype = i
        lib.orc_sweep_pairs.argtypes = [vp, i, vp, i]
        lib.orc_sweep_pairs.restype = i
        _lib = lib
    return _lib


def ref_available():
    return os.path.exists(REF_PATH)


def _load_ref():
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_PATH)
        vp, i = ctypes.c_void_p, ctypes.c_int
        lib.ref_signed_distance.argtypes = [vp, i, vp, vp, i, vp, vp, i, i, ctypes.c_double]
        lib.ref_signed_distance.restype = i
        lib.ref_collide.argtypes = [vp, i, vp, vp, i, i, vp, i]
        lib.ref_directed.argtypes = [vp, i, vp, vp, i, vp, vp, i]
        lib.ref_directed.restype = i
        lib.ref_incremental.argtypes = [vp, i, vp, vp, i, vp, vp, i]
        lib.ref_incremental.restype = i
        lib.ref_swept_portal.argtypes = [vp, i, vp, vp, i, vp, i, ctypes.c_double, vp, i]
        lib.ref_swept_portal.restype = i
        lib.ref_collide.restype = i
        _ref = lib
    return _ref


def ref_mesh_available():
    return os.path.exists(REF_MESH_PATH)


_ref_mesh = None


def _load_ref_mesh():
    global _ref_mesh
    if _ref_mesh is None:
        lib = ctypes.CDLL(REF_MESH_PATH)
        vp, i = ctypes.c_void_p, ctypes.c_int
        lib.refm_build.argtypes = [vp, i, vp, i]
        lib.refm_build.restype = vp
        lib.refm_free.argtypes = [vp]
        lib.refm_free.restype = None
        lib.refm_num_nodes.argtypes = [vp]
        lib.refm_num_nodes.restype = i
        lib.refm_export.argtypes = [vp, vp, vp]
        lib.refm_export.restype = None
        lib.refm_mesh_collide.argtypes = [vp, vp, vp, i, i, vp, vp, i, i]
        lib.refm_mesh_collide.restype = i
        lib.refm_analytic.argtypes = [vp, vp, vp, i, vp, vp, i]
        lib.refm_analytic.restype = i
        lib.refm_mesh_shape_collide.argtypes = [vp, i, vp, vp, i, vp, i, i, vp, i, i, vp, vp, i, i]
        lib.refm_mesh_shape_collide.restype = i
        _ref_mesh = lib
    return _ref_mesh


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _prep(batch):
    s = np.ascontiguousarray(batch.shapes)
    v = np.ascontiguousarray(batch.vertices, np.float32)
    if len(v) == 0:
        v = np.zeros((1, 4), np.float32)
    p = np.ascontiguousarray(batch.pairs)
    return s, v, p


# fcl::Convex walks hulls of more than this many vertices
# (kMinVertCountForEdgeWalking, include/fcl/geometry/shape/convex.h:60-61).
WALK_MIN_VERTICES = 32


def neighbor_table(nv, faces):
    """Convex::FindVertexNeighbors (convex-inl.h:379-405) over a face list
    (an [m, k] array or sequences of vertex indices; consecutive vertices of a
    face and its last and first are neighbours): the neighbors_ layout, int32
    -- nv row offsets, then per vertex its neighbour count and the neighbours
    ascending."""
    if isinstance(faces, np.ndarray) and faces.ndim == 2:
        f = faces.astype(np.int64)
        a, b = f.reshape(-1), np.roll(f, -1, axis=1).reshape(-1)
    else:
        a = np.asarray([int(v) for face in faces for v in face], np.int64)
        b = np.asarray([int(face[(k + 1) % len(face)]) for face in faces for k in range(len(face))], np.int64)
    e = np.unique(np.concatenate([a * nv + b, b * nv + a]))  # sorted: by vertex, then neighbour
    src, dst = e // nv, e % nv
    deg = np.bincount(src, minlength=nv)
    row = nv + np.concatenate([[0], np.cumsum(deg + 1)[:-1]])  # each row: count, then neighbours
    table = np.zeros(nv + int(np.sum(deg + 1)), np.int32)
    table[:nv] = row
    table[row] = deg
    starts = np.concatenate([[0], np.cumsum(deg)[:-1]])
    table[row[src] + 1 + (np.arange(len(src)) - starts[src])] = dst
    return table


def walk_tables(batch, min_vertices=WALK_MIN_VERTICES, faces=None):
    """Neighbour tables of the batch's hulls with more than min_vertices
    vertices, as fcl::Convex builds them from a face list: faces[shape] where
    given, else the triangles of the hull's qhull convex hull (scipy).
    Returns (off int64[n_shapes], -1 = scan; nbr int32[])."""
    from scipy.spatial import ConvexHull
    s = batch.shapes
    off = np.full(len(s), -1, np.int64)
    parts, total, seen = [], 0, {}
    for i in range(len(s)):
        if int(s["type"][i]) != 100 or int(s["vert_count"][i]) <= min_vertices:
            continue
        o, c = int(s["vert_offset"][i]), int(s["vert_count"][i])
        key = (o, c)
        if faces is None and key in seen:
            off[i] = seen[key]
            continue
        if faces is not None and i in faces:
            f = faces[i]
        else:
            f = ConvexHull(np.asarray(batch.vertices[o:o + c, :3], np.float64)).simplices
        t = neighbor_table(c, f)
        off[i] = seen[key] = total
        parts.append(t)
        total += len(t)
    nbr = np.concatenate(parts) if parts else np.zeros(1, np.int32)
    return off, nbr


class _Walk:
    """Installs walk tables in the restatement for one call."""

    def __init__(self, lib, tables, n_shapes):
        self.lib, self.tables, self.n = lib, tables, n_shapes

    def __enter__(self):
        if self.tables is not None:
            off, nbr = self.tables
            assert len(off) == self.n
            self.off = np.ascontiguousarray(off, np.int64)
            self.nbr = np.ascontiguousarray(nbr, np.int32)
            self.lib.orc_set_walk(_ptr(self.off), self.n, _ptr(self.nbr))
        return self

    def __exit__(self, *exc):
        if self.tables is not None:
            self.lib.orc_set_walk(None, 0, None)
        return False


def default_threads():
    return max(1, os.cpu_count() or 1)


def signed_distance(batch, guess=None, threads=None, gjk_max_iter=0, gjk_tol=0.0, epa_max_faces=0,
                    epa_max_iter=0, epa_tol=0.0, walk=None):
    """GJKSolver::shapeSignedDistance per pair (restatement); walk = tables of
    walk_tables() for the hill-climbing convex support, None for the scan."""
    lib = _load()
    s, v, p = _prep(batch)
    out = np.zeros(len(p), RESULT_DTYPE)
    g = None if guess is None else np.ascontiguousarray(guess, np.float32)
    with _Walk(lib, walk, len(s)):
            rc = lib.orc_signed_distance(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(g), _ptr(out),
                                     threads or default_threads(), gjk_max_iter, gjk_tol, epa_max_faces,
                                     epa_max_iter, epa_tol)
    assert rc == 0
    return out


def collide(batch, want_contact=False, threads=None, analytic=True, walk=None):
    """fcl::collide on shape pairs (restatement): the closed-form sphere-pair
    solvers (analytic=True, as fcl::collide dispatches), else MPR boolean or
    GJK+EPA contact; walk as in signed_distance."""
    lib = _load()
    s, v, p = _prep(batch)
    out = np.zeros(len(p), RESULT_DTYPE)
    with _Walk(lib, walk, len(s)):
        rc = lib.orc_collide(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), int(want_contact), int(analytic),
                             _ptr(out), threads or default_threads())
    assert rc == 0
    return out


def collide_directed(batch, dirs, threads=None):
    """fcl::collide with useDirectedPenetration: boolean collide, then
    MPR::DirectedPenetration along dirs (unit, shape b's escape direction in
    shape a's frame) for colliding pairs; epa_status = the directed status."""
    lib = _load()
    s, v, p = _prep(batch)
    d = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(len(p), RESULT_DTYPE)
    rc = lib.orc_collide_directed(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(d), _ptr(out),
                                  threads or default_threads())
    assert rc == 0
    return out


def directed_raw(batch, dirs, threads=None):
    """Restated MPR::DirectedPenetration on every pair (status in epa_status)."""
    lib = _load()
    s, v, p = _prep(batch)
    d = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(len(p), RESULT_DTYPE)
    assert lib.orc_directed_raw(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(d), _ptr(out),
                                threads or default_threads()) == 0
    return out


def collide_incremental(batch, dirs, threads=None):
    """fcl::collide with useIncrementalMinimumDistancePenetration: boolean
    collide, then MPR::IncrementalMinimumPenetrationDistance from the hint dirs
    (unit, shape b's escape direction in shape a's frame) for colliding pairs;
    epa_status = the incremental status, normal = the converged direction."""
    return _dir_call("orc_collide_incremental", batch, dirs, threads)


def incremental_raw(batch, dirs, threads=None):
    """Restated incremental penetration on every pair (depth in distance)."""
    return _dir_call("orc_incremental_raw", batch, dirs, threads)


def ref_incremental(batch, dirs, threads=None):
    """The reference's RunIncrementalMinimumPenetrationDistance on every pair."""
    lib = _load_ref()
    s, v, p = _prep(batch)
    d = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(len(p), RESULT_DTYPE)
    assert lib.ref_incremental(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(d), _ptr(out),
                               threads or default_threads()) == 0
    return out


def _dir_call(name, batch, dirs, threads):
    lib = _load()
    s, v, p = _prep(batch)
    d = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(len(p), RESULT_DTYPE)
    assert getattr(lib, name)(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(d), _ptr(out),
                              threads or default_threads()) == 0
    return out


def ref_directed(batch, dirs, threads=None):
    """The reference's MPR::RunDirectedPenetration on every pair."""
    lib = _load_ref()
    s, v, p = _prep(batch)
    d = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(len(p), RESULT_DTYPE)
    assert lib.ref_directed(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(d), _ptr(out),
                            threads or default_threads()) == 0
    return out


def box_box(side1, R1, T1, side2, R2, T2):
    """boxBox2 in FP64 on two posed boxes (world frame), as boxBoxIntersect calls
    it: (code, normal, depth or separation, contacts [n, 4] = pos, depth)."""
    lib = _load()
    a = [np.ascontiguousarray(x, np.float64).reshape(-1) for x in (side1, R1, T1, side2, R2, T2)]
    out = np.zeros(6 + 16)
    n = lib.orc_box_box(*[_ptr(x) for x in a], _ptr(out))
    return int(out[4]), out[0:3].copy(), float(out[3]), out[6:6 + 4 * n].reshape(n, 4).copy()


def support(batch, shape, dirs, walk=None):
    """Support points [n, 3] of one shape of the batch for directions [n, 3]."""
    lib = _load()
    s, v, _ = _prep(batch)
    d = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
    out = np.zeros((len(d), 3), np.float64)
    with _Walk(lib, walk, len(s)):
        assert lib.orc_support(_ptr(s), len(s), _ptr(v), int(shape), _ptr(d), len(d), _ptr(out)) == 0
    return out


def time_signed_distance(batch, threads=None, walk=None):
    """Seconds the restatement takes for the whole batch (wall clock, C++ side)."""
    lib = _load()
    s, v, p = _prep(batch)
    out = np.zeros(len(p), RESULT_DTYPE)
    with _Walk(lib, walk, len(s)):
        t = lib.orc_time_signed_distance(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(out),
                                         threads or default_threads())
    return t, out


def ref_signed_distance(batch, guess=None, threads=None, gjk_max_iter=0, gjk_tol=0.0):
    """The reference's own GJK/EPA (oracle/_ref) on the same inputs."""
    lib = _load_ref()
    s, v, p = _prep(batch)
    out = np.zeros(len(p), RESULT_DTYPE)
    g = None if guess is None else np.ascontiguousarray(guess, np.float32)
    assert lib.ref_signed_distance(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(g), _ptr(out),
                                   threads or default_threads(), gjk_max_iter, gjk_tol) == 0
    return out


def ref_collide(batch, want_contact=False, threads=None):
    lib = _load_ref()
    s, v, p = _prep(batch)
    out = np.zeros(len(p), RESULT_DTYPE)
    assert lib.ref_collide(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), int(want_contact), _ptr(out),
                           threads or default_threads()) == 0
    return out


def mesh_collide(nodes_a, tris_a, nodes_b, tris_b, poses, max_contacts=1, pair_cap=None, threads=None):
    """MeshIntersect per pose over the given flattened trees (restatement).

    max_contacts = 0: every colliding pair (up to pair_cap stored per pose).
    Returns (flags, counts, pairs[n, pair_cap, 2])."""
    lib = _load()
    poses = np.ascontiguousarray(poses, np.float32).reshape(-1, 12)
    n = len(poses)
    cap = pair_cap if pair_cap is not None else max(max_contacts, 1)
    flags = np.zeros(n, np.uint8)
    counts = np.zeros(n, np.uint32)
    pairs = np.full((n, cap, 2), -1, np.int32)
    na = np.ascontiguousarray(nodes_a)
    nb = np.ascontiguousarray(nodes_b)
    ta = np.ascontiguousarray(tris_a, np.float32)
    tb = np.ascontiguousarray(tris_b, np.float32)
    assert lib.orc_mesh_collide(_ptr(na), _ptr(ta), _ptr(nb), _ptr(tb), _ptr(poses), n, int(max_contacts), cap,
                                _ptr(flags), _ptr(counts), _ptr(pairs), threads or default_threads()) == 0
    return flags, counts, pairs


def mesh_shape_collide(nodes, tris, batch, shape_ids, poses, max_contacts=1, pair_cap=None, threads=None):
    """fcl::collide(mesh, shape) per query (MeshShapeIntersect, penetration
    off): the batch's shape shape_ids[i] posed by poses[i] (12 floats) in the
    mesh frame.  Returns (flags, counts, tri_ids[n, pair_cap])."""
    lib = _load()
    s, v, _ = _prep(batch)
    ids = np.ascontiguousarray(shape_ids, np.uint32)
    poses = np.ascontiguousarray(poses, np.float32).reshape(-1, 12)
    n = len(poses)
    cap = pair_cap if pair_cap is not None else max(max_contacts, 1)
    flags = np.zeros(n, np.uint8)
    counts = np.zeros(n, np.uint32)
    out = np.full((n, cap), -1, np.int32)
    nd = np.ascontiguousarray(nodes)
    tr = np.ascontiguousarray(tris, np.float32)
    assert lib.orc_mesh_shape_collide(_ptr(nd), _ptr(tr), _ptr(s), len(s), _ptr(v), _ptr(ids), _ptr(poses), n,
                                      int(max_contacts), cap, _ptr(flags), _ptr(counts), _ptr(out),
                                      threads or default_threads()) == 0
    return flags, counts, out


def mesh_shape_contacts(nodes, tris, batch, shape_ids, poses, max_contacts=1, pair_cap=None, threads=None):
    """fcl::collide(mesh, shape) with penetration on: per query (counts,
    tri_ids[n, pair_cap], contacts[n, pair_cap, 8] = pos, normal (mesh frame,
    the reference's reversed normal), depth, EPA status or -1 for a sphere)."""
    lib = _load()
    s, v, _ = _prep(batch)
    ids = np.ascontiguousarray(shape_ids, np.uint32)
    poses = np.ascontiguousarray(poses, np.float32).reshape(-1, 12)
    n = len(poses)
    cap = pair_cap if pair_cap is not None else max(max_contacts, 1)
    counts = np.zeros(n, np.uint32)
    out = np.full((n, cap), -1, np.int32)
    con = np.zeros((n, cap, 8))
    nd = np.ascontiguousarray(nodes)
    tr = np.ascontiguousarray(tris, np.float32)
    assert lib.orc_mesh_shape_contacts(_ptr(nd), _ptr(tr), _ptr(s), len(s), _ptr(v), _ptr(ids), _ptr(poses), n,
                                       int(max_contacts), cap, _ptr(counts), _ptr(out), _ptr(con),
                                       threads or default_threads()) == 0
    return counts, out, con


def mesh_shape_all(tris, batch, shape_id, pose, cap=1 << 20):
    """Every colliding triangle of one query by brute force."""
    lib = _load()
    s, v, _ = _prep(batch)
    tr = np.ascontiguousarray(tris, np.float32)
    p = np.ascontiguousarray(pose, np.float32).reshape(12)
    out = np.zeros(cap, np.int32)
    n = lib.orc_mesh_shape_all(_ptr(tr), len(tr), _ptr(s), len(s), _ptr(v), int(shape_id), _ptr(p), _ptr(out), cap)
    return out[:min(n, cap)]


def object_aabbs(batch, shape_ids, poses):
    """CollisionObject::computeAABB per object in FP64: [n, 6] lo, hi."""
    lib = _load()
    s, v, _ = _prep(batch)
    ids = np.ascontiguousarray(shape_ids, np.uint32)
    p = np.ascontiguousarray(poses, np.float32).reshape(-1, 12)
    out = np.zeros((len(p), 6), np.float64)
    assert lib.orc_object_aabbs(_ptr(s), len(s), _ptr(v), _ptr(ids), _ptr(p), len(p), _ptr(out)) == 0
    return out


def aabb_pairs(boxes, cap=None):
    """Every overlapping pair (i < j) of the boxes [n, 6] by brute force."""
    lib = _load()
    b = np.ascontiguousarray(boxes, np.float64).reshape(-1, 6)
    cap = len(b) * 8 if cap is None else cap
    while True:
        out = np.zeros((max(cap, 1), 2), np.uint32)
        m = lib.orc_aabb_pairs(_ptr(b), len(b), _ptr(out), cap)
        if m <= cap:
            return out[:m]
        cap = m


def sweep_pairs(boxes, cap=None):
    """The overlapping pairs by sort-and-sweep (CPU baseline of the broadphase)."""
    lib = _load()
    b = np.ascontiguousarray(boxes, np.float64).reshape(-1, 6)
    cap = len(b) * 8 if cap is None else cap
    while True:
        out = np.zeros((max(cap, 1), 2), np.uint32)
        m = lib.orc_sweep_pairs(_ptr(b), len(b), _ptr(out), cap)
        if m <= cap:
            return out[:m]
        cap = m


def mesh_allpairs(tris_a, tris_b, pose, cap=1 << 20):
    """Every colliding triangle pair of one pose by brute force."""
    lib = _load()
    ta = np.ascontiguousarray(tris_a, np.float32)
    tb = np.ascontiguousarray(tris_b, np.float32)
    p = np.ascontiguousarray(pose, np.float32).reshape(12)
    out = np.zeros((cap, 2), np.int32)
    n = lib.orc_mesh_allpairs(_ptr(ta), len(ta), _ptr(tb), len(tb), _ptr(p), _ptr(out), cap)
    return out[:min(n, cap)]


def tri_tri(p, q, pose):
    lib = _load()
    p = np.ascontiguousarray(p, np.float64).reshape(9)
    q = np.ascontiguousarray(q, np.float64).reshape(9)
    pose = np.ascontiguousarray(pose, np.float64).reshape(12)
    return bool(lib.orc_tri_tri(_ptr(p), _ptr(q), _ptr(pose)))


# ------------------------------------------------------- translational CCD --
CCD_DTYPE = np.dtype([("collide", np.int32), ("mpr_status", np.int32), ("box_tested", np.int32),
                      ("reserved", np.int32), ("toc_lo", np.float64), ("toc_hi", np.float64)])
TOC_NONE, TOC_BOX, TOC_SAMPLE = 0, 1, 2  # TimeOfCollisionRequestType order of the C ABI


def translational_ccd(batch, disp, toc_type=TOC_NONE, zero_tol=1e-4, max_iter=128, tol=1e-6, threads=None):
    """fcl::translational_ccd on every pair: shape a moving along disp[i] =
    (unit axis in a's frame, distance) against shape b (CCD_DTYPE rows;
    toc = (-1, -1) where the request computes none)."""
    lib = _load()
    s, v, p = _prep(batch)
    d = np.ascontiguousarray(disp, np.float32).reshape(-1, 4)
    assert len(d) == len(p)
    out = np.zeros(len(p), CCD_DTYPE)
    assert lib.orc_translational_ccd(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(d), int(toc_type),
                                     ctypes.c_double(zero_tol), int(max_iter), ctypes.c_double(tol), _ptr(out),
                                     threads or default_threads()) == 0
    return out


def _portal(fn, batch, disp, max_iter, tol, threads):
    s, v, p = _prep(batch)
    d = np.ascontiguousarray(disp, np.float32).reshape(-1, 4)
    out = np.zeros((len(p), 23))
    assert fn(_ptr(s), len(s), _ptr(v), _ptr(p), len(p), _ptr(d), int(max_iter), ctypes.c_double(tol), _ptr(out),
              threads or default_threads()) == 0
    return out


def swept_portal(batch, disp, max_iter=128, tol=1e-6, threads=None):
    """The restated MPR on the swept-volume difference with its portal data
    (rows of 23: status, count, v0, v1..v3, d1..d3; unset entries NaN)."""
    return _portal(_load().orc_swept_portal, batch, disp, max_iter, tol, threads)


def ref_swept_portal(batch, disp, max_iter=128, tol=1e-6, threads=None):
    """The reference's MPR::Intersect with IntersectData on the same difference."""
    return _portal(_load_ref().ref_swept_portal, batch, disp, max_iter, tol, threads)


def box_axis(h1, d, h2, off):
    """CheckEmptyTocIntervalOnAxis, scalar: (empty, lo, hi), unscaled."""
    out = np.zeros(2)
    e = _load().orc_box_axis(ctypes.c_double(h1), ctypes.c_double(d), ctypes.c_double(h2), ctypes.c_double(off),
                             _ptr(out))
    return bool(e), out[0], out[1]


def box_axes3(h1, d, h2, off, zero_tol=1e-4):
    """CheckEmptyTocIntervalOnAxis, three axes: (empty, lo, hi) scaled to [0, 1]."""
    a = [np.ascontiguousarray(np.broadcast_to(x, 3), np.float64) for x in (h1, d, h2, off)]
    out = np.zeros(2)
    e = _load().orc_box_axes3(*[_ptr(x) for x in a], ctypes.c_double(zero_tol), _ptr(out))
    return bool(e), out[0], out[1]


def box_pair_ccd(h1, axis, dist, R, t, h2, zero_tol=1e-4):
    """BoxPairTranslationalCCD::IsDisjoint with box 1 at the origin of its frame:
    (disjoint, lo, hi); R row-major (box 2 in box 1), t box 2's centre."""
    a = [np.ascontiguousarray(x, np.float64).reshape(-1) for x in (h1, axis, R, t, h2)]
    out = np.zeros(2)
    e = _load().orc_box_pair_ccd(_ptr(a[0]), _ptr(a[1]), ctypes.c_double(dist), _ptr(a[2]), _ptr(a[3]), _ptr(a[4]),
                                 ctypes.c_double(zero_tol), _ptr(out))
    return bool(e), out[0], out[1]


# ------------------------------------------------ mesh: the reference's tree --

def _mesh_arrays(vertices, triangles):
    V = np.ascontiguousarray(vertices, np.float64).reshape(-1, 3)
    T = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    return V, T


def ref_tree(vertices, triangles):
    """The reference's own BVHModel<OBBRSS<double>> over the mesh (compiled
    reference): (f64[n, 16] = axis row-major 9, To 3, extent 3, size;
    i32[n, 3] = first_child, first_primitive, num_primitives)."""
    lib = _load_ref_mesh()
    V, T = _mesh_arrays(vertices, triangles)
    h = lib.refm_build(_ptr(V), len(V), _ptr(T), len(T))
    assert h, "reference BVH build failed"
    try:
        n = lib.refm_num_nodes(h)
        f64 = np.zeros((n, 16))
        i32 = np.zeros((n, 3), np.int32)
        lib.refm_export(h, _ptr(f64), _ptr(i32))
    finally:
        lib.refm_free(h)
    return f64, i32


def orc_tree(vertices, triangles):
    """The restated build of the same tree: (f64, i32, primitive order)."""
    lib = _load()
    V, T = _mesh_arrays(vertices, triangles)
    n = max(2 * len(T) - 1, 0)
    f64 = np.zeros((n, 16))
    i32 = np.zeros((n, 3), np.int32)
    prim = np.zeros(len(T), np.uint32)
    assert lib.orc_ref_tree(_ptr(V), _ptr(T), len(T), _ptr(f64), _ptr(i32), _ptr(prim)) == n
    return f64, i32, prim


def _collide_out(n, stride):
    return np.zeros(n, np.int32), np.full((n, max(stride, 1), 2), -1, np.int32)


def ref_mesh_collide(mesh_a, mesh_b, poses, max_contacts=1, stride=None, threads=None):
    """The compiled reference's MeshIntersect per pose (mesh a at the identity,
    mesh b posed by poses[i]: 12 values, rotation row-major then translation)
    with CollisionRequest(max_contacts).  Returns (counts, pairs[n, stride, 2])
    in the reference's contact order."""
    lib = _load_ref_mesh()
    Va, Ta = _mesh_arrays(*mesh_a)
    Vb, Tb = _mesh_arrays(*mesh_b)
    P = np.ascontiguousarray(poses, np.float64).reshape(-1, 12)
    stride = max_contacts if stride is None else stride
    ha = lib.refm_build(_ptr(Va), len(Va), _ptr(Ta), len(Ta))
    hb = lib.refm_build(_ptr(Vb), len(Vb), _ptr(Tb), len(Tb))
    assert ha and hb
    try:
        counts, pairs = _collide_out(len(P), stride)
        assert lib.refm_mesh_collide(ha, hb, _ptr(P), len(P), int(max_contacts), _ptr(counts), _ptr(pairs),
                                     max(stride, 1), threads or default_threads()) == 0
    finally:
        lib.refm_free(ha)
        lib.refm_free(hb)
    return counts, pairs


def orc_mesh_collide_ref(mesh_a, mesh_b, poses, max_contacts=1, stride=None, threads=None):
    """The restated MeshIntersect over the restated reference trees (same
    interface as ref_mesh_collide)."""
    lib = _load()
    Va, Ta = _mesh_arrays(*mesh_a)
    Vb, Tb = _mesh_arrays(*mesh_b)
    P = np.ascontiguousarray(poses, np.float64).reshape(-1, 12)
    stride = max_contacts if stride is None else stride
    counts, pairs = _collide_out(len(P), stride)
    assert lib.orc_ref_mesh_collide(_ptr(Va), _ptr(Ta), len(Ta), _ptr(Vb), _ptr(Tb), len(Tb), _ptr(P), len(P),
                                    int(max_contacts), _ptr(counts), _ptr(pairs), max(stride, 1),
                                    threads or default_threads()) == 0
    return counts, pairs


ANALYTIC_SHAPE_DTYPE = np.dtype([("type", "<i4"), ("pad", "<i4"), ("p", "<f8", (3,))])


def ref_analytic(types_a, params_a, types_b, params_b, poses, threads=None):
    """The compiled reference's GJKSolver::shapeIntersect with contacts on
    closed-form pairs (types 0 sphere, 1 box, 2 capsule, 3 cylinder; params:
    radius / full sides / radius and full length), shape a at the identity and
    shape b posed by poses[i].  Returns (count[n] (-1: not a closed-form pair),
    contacts[n, 4, 7] = normal 3, pos 3, depth)."""
    lib = _load_ref_mesh()
    n = len(types_a)
    A = np.zeros(n, ANALYTIC_SHAPE_DTYPE)
    B = np.zeros(n, ANALYTIC_SHAPE_DTYPE)
    A["type"], A["p"] = types_a, params_a
    B["type"], B["p"] = types_b, params_b
    P = np.ascontiguousarray(poses, np.float64).reshape(-1, 12)
    out = np.zeros((n, 4, 7))
    ret = np.zeros(n, np.int32)
    assert lib.refm_analytic(_ptr(A), _ptr(B), _ptr(P), n, _ptr(out), _ptr(ret), threads or default_threads()) == 0
    return ret, out


def ref_mesh_shape_collide(mesh, batch, shape_id, poses, max_contacts=1, stride=None, threads=None):
    """The compiled reference's MeshShapeIntersect of a mesh (vertices,
    triangles) against one shape of `batch` (sphere, box, capsule, cylinder or
    convex hull; a hull gets scipy's triangulated hull faces) posed by
    poses[i] in the mesh frame.  Returns (counts, tris[n, stride]) in the
    reference's order."""
    from fclg.layout import BOX, CAPSULE, CONVEX, CYLINDER, SPHERE
    lib = _load_ref_mesh()
    s = batch.shapes[shape_id]
    t = int(s["type"])
    code = {SPHERE: 0, BOX: 1, CAPSULE: 2, CYLINDER: 3, CONVEX: 4}[t]
    params = np.ascontiguousarray(s["param"][:3], np.float64)
    hv = np.zeros((1, 3))
    faces = np.zeros(1, np.int32)
    n_faces = 0
    if t == CONVEX:
        from scipy.spatial import ConvexHull
        hv = np.ascontiguousarray(batch.vertices[s["vert_offset"]:s["vert_offset"] + s["vert_count"], :3],
                                  np.float64)
        hull = ConvexHull(hv)
        n_faces = len(hull.simplices)
        faces = np.concatenate([np.full((n_faces, 1), 3), hull.simplices], 1).astype(np.int32).ravel()
    V, T = _mesh_arrays(*mesh)
    P = np.ascontiguousarray(poses, np.float64).reshape(-1, 12)
    stride = max_contacts if stride is None else stride
    h = lib.refm_build(_ptr(V), len(V), _ptr(T), len(T))
    assert h
    try:
        counts = np.zeros(len(P), np.int32)
        tris = np.full((len(P), max(stride, 1)), -1, np.int32)
        rc = lib.refm_mesh_shape_collide(h, code, _ptr(params), _ptr(hv), len(hv), _ptr(faces), n_faces, len(faces),
                                         _ptr(P), len(P), int(max_contacts), _ptr(counts), _ptr(tris),
                                         max(stride, 1), threads or default_threads())
        assert rc == 0
    finally:
        lib.refm_free(h)
    return counts, tris
