"""Hull edge graphs and the hill-climbing convex support (host only, no GPU).

fcl::Convex finds the support vertex of a hull with more than 32 vertices by
walking its vertex-neighbour graph (include/fcl/geometry/shape/convex-inl.h:
201-283) instead of scanning every vertex; the reference checks the walk
against the naive scan over random directions (test/test_fcl_convex_primitive.cpp:
8-34) and pins one co-planar corner case (test/geometry/shape/test_convex.cpp:
584-605).  The same checks run here on:
* the library's own hull builder (fclg_hull_graph, the graph the GPU walk
  climbs), against scipy's qhull and through a Python walk of the reference rule;
* the oracle's walk (neighbour tables from face lists, as fcl::Convex builds them).
"""
import numpy as np
import pytest

from fclg import workloads


@pytest.fixture(scope="module")
def lib():
    import build as fclg_build
    fclg_build.build()
    from fclg import api
    return api


AXES = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float64)


def walk(points, starts, first, adj, d):
    """Convex::findExtremeVertexViaNeighbours (convex-inl.h:201-283) over a CSR graph."""
    init, best = -1, 0.0
    for k in range(6):
        v = float(AXES[k] @ d)
        if init < 0 or v > best:
            init, best = int(starts[k]), v
    ext = init
    ext_val = float(points[ext] @ d)
    p0 = p1 = init
    keep = True
    while keep:
        keep = False
        old = ext
        for n in adj[first[old]:first[old + 1]]:
            n = int(n)
            if n == p0 or n == p1:
                continue
            val = float(points[n] @ d)
            if val > ext_val:
                p1, ext, ext_val, keep = ext, n, val, True
        p0 = old
    return ext


def qhull_edges(points):
    from scipy.spatial import ConvexHull
    h = ConvexHull(points)
    e = set()
    for t in h.simplices:
        for k in range(3):
            a, b = int(t[k]), int(t[(k + 1) % 3])
            e.add((a, b))
            e.add((b, a))
    return e


def graph_edges(first, adj):
    return {(i, int(j)) for i in range(len(first) - 1) for j in adj[first[i]:first[i + 1]]}


def cloud(rng, kind, n):
    p = rng.normal(size=(n, 3))
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    if kind == "ellipsoid":
        p *= np.array([0.4, 0.1, 0.05])
    elif kind == "interior":
        p[n // 2:] *= rng.uniform(0.0, 0.9, size=(n - n // 2, 1))  # half the points strictly inside
    elif kind == "duplicates":
        p[n // 2:] = p[:n - n // 2]
    return p.astype(np.float32)


@pytest.mark.parametrize("kind", ["sphere", "ellipsoid", "interior", "duplicates"])
def test_hull_graph_matches_qhull(lib, kind):
    rng = np.random.default_rng(7)
    for n in (33, 64, 200, 600):
        p = cloud(rng, kind, n)
        starts, first, adj = lib.hull_graph(p)
        assert len(first) == n + 1
        for r in range(n):
            row = adj[first[r]:first[r + 1]]
            assert np.all(np.diff(row.astype(np.int64)) > 0)  # ascending, as the reference's std::set
        got = graph_edges(first, adj)
        ref = qhull_edges(p.astype(np.float64))
        if kind == "duplicates":
            # qhull and the builder may keep different copies of a repeated point
            uniq, inv = np.unique(p, axis=0, return_inverse=True)
            inv = inv.reshape(-1)
            assert {(inv[a], inv[b]) for a, b in got} == {(inv[a], inv[b]) for a, b in ref}
        else:
            assert got == ref
        deg = np.diff(first.astype(np.int64))
        for k in range(6):
            assert deg[starts[k]] > 0
            # the start corner is extreme along its axis
            assert np.isclose(p[starts[k]] @ AXES[k], np.max(p @ AXES[k]), rtol=0, atol=1e-7)


def test_walk_reaches_the_scan_maximum(lib):
    """test_fcl_convex_primitive.cpp:8-34 on the library's graphs: the walk
    from the six cached corners lands on a vertex of maximal support value."""
    rng = np.random.default_rng(11)
    for kind in ("sphere", "ellipsoid", "interior"):
        for n in (33, 120, 400):
            p = cloud(rng, kind, n).astype(np.float64)
            starts, first, adj = lib.hull_graph(p.astype(np.float32))
            dirs = rng.normal(size=(1000, 3))
            dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
            for d in dirs:
                v = walk(p, starts, first, adj, d)
                assert p[v] @ d >= np.max(p @ d) - 1e-12


def test_hull_graph_of_a_box_walks_to_a_corner(lib):
    """Co-planar faces (triangulated by the builder): every direction still ends
    on a corner of maximal value."""
    c = np.array([[x, y, z] for x in (-1, 1) for y in (-2, 2) for z in (-0.5, 0.5)], np.float32)
    extra = np.array([[0, 0, 0.5], [0, 2, 0], [0.3, 0.1, 0.2]], np.float32)  # face centre, edge midpoint, inside
    p = np.concatenate([c, extra])
    starts, first, adj = lib.hull_graph(p)
    deg = np.diff(first.astype(np.int64))
    assert np.all(deg[:8] >= 3) and np.all(deg[8:] == 0)
    rng = np.random.default_rng(3)
    for d in rng.normal(size=(500, 3)):
        v = walk(p.astype(np.float64), starts, first, adj, d)
        assert p[v].astype(np.float64) @ d >= np.max(p.astype(np.float64) @ d) - 1e-12


def test_hull_graph_rejects_flat_and_tiny_inputs(lib):
    rng = np.random.default_rng(5)
    flat = np.zeros((40, 3), np.float32)
    flat[:, :2] = rng.normal(size=(40, 2))
    assert lib.hull_graph(flat) is None
    assert lib.hull_graph(np.eye(3, dtype=np.float32)) is None
    line = np.outer(np.linspace(0, 1, 50), [1, 2, 3]).astype(np.float32)
    assert lib.hull_graph(line) is None


def _single_hull_batch(points):
    s = np.zeros(1, workloads.SHAPE_DTYPE)
    s["type"] = 100
    s["vert_count"] = len(points)
    v = np.zeros((len(points), 4), np.float32)
    v[:, :3] = points
    s["param"][0, :3] = v[:, :3].astype(np.float64).mean(axis=0)
    p = np.zeros(0, workloads.PAIR_DTYPE)
    return workloads.Batch("hull", s, v, p, {})


def test_oracle_walk_equals_the_scan(oracle_lib):
    """The oracle's walk over qhull face lists against its naive scan."""
    rng = np.random.default_rng(13)
    for kind in ("sphere", "ellipsoid", "interior"):
        b = _single_hull_batch(cloud(rng, kind, 150))
        tables = oracle_lib.walk_tables(b)
        assert tables[0][0] >= 0
        d = rng.normal(size=(2000, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        w = oracle_lib.support(b, 0, d, walk=tables)
        s = oracle_lib.support(b, 0, d)
        assert np.all(np.sum(w * d, axis=1) >= np.sum(s * d, axis=1) - 1e-12)
        assert np.mean(np.all(w == s, axis=1)) > 0.999  # a different vertex only on a tie


def test_oracle_walk_co_planar_known_answer(oracle_lib):
    """test_convex.cpp:551-605 (CoPlanarTetrahedron, SupportVertexCoPlanarFaces):
    vertex 0 sits in the middle of the bottom face; the walk, forced on for
    five vertices, returns the apex for the direction +z."""
    r3 = np.sqrt(3.0)
    tet = np.array([[0.5, -0.5 / r3, 0], [-0.5, -0.5 / r3, 0], [0, 1 / r3, 0], [0, 0, np.sqrt(3 / 8)]])
    pts = np.concatenate([tet[:3].mean(axis=0, keepdims=True), tet])
    faces = [[0, 1, 2], [0, 2, 3], [0, 3, 1], [1, 3, 4], [3, 2, 4], [1, 4, 2]]
    b = _single_hull_batch(pts.astype(np.float32))
    tables = oracle_lib.walk_tables(b, min_vertices=0, faces={0: faces})
    got = oracle_lib.support(b, 0, np.array([[0.0, 0.0, 1.0]]), walk=tables)[0]
    assert np.array_equal(got, pts[4].astype(np.float32).astype(np.float64))
    # and every other direction agrees with the scan on the value
    rng = np.random.default_rng(2)
    d = rng.normal(size=(500, 3))
    w = oracle_lib.support(b, 0, d, walk=tables)
    s = oracle_lib.support(b, 0, d)
    assert np.allclose(np.sum(w * d, axis=1), np.sum(s * d, axis=1), rtol=0, atol=1e-12)


def test_neighbor_table_layout(oracle_lib):
    """Convex::FindVertexNeighbors' encoding on a cube given as quads."""
    faces = [[0, 1, 2, 3], [4, 5, 6, 7], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [3, 0, 4, 7]]
    t = oracle_lib.neighbor_table(8, faces)
    for v, want in enumerate([[1, 3, 4], [0, 2, 5], [1, 3, 6], [0, 2, 7], [0, 5, 7], [1, 4, 6], [2, 5, 7],
                              [3, 4, 6]]):
        row = t[v]
        assert t[row] == 3
        assert list(t[row + 1:row + 4]) == want
