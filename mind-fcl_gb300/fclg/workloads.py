"""Seeded synthetic workloads for the batched narrowphase.

Every random number comes from ``Generator(Philox(seed)).random()`` and is
transformed here (Box-Muller, Shoemake quaternions, inverse CDFs), so a seed
gives the same batch on every numpy version and host.

Workloads (sizes as the project's benchmark configurations state them):

* ``plain_small``   4096 convex pairs, hulls of 32 points on the unit sphere
  scaled by r ~ U[0.05, 0.5] m, translation uniform in a 1 m cube, uniform
  random rotation.
* ``mixed``         pairs of shapes drawn uniformly from box / sphere /
  capsule / cylinder / convex; half extents, radii and half lengths
  ~ U[0.02, 0.4] m; convex hulls of V ~ log-uniform[8, 256] sphere points;
  about 40 % of the pairs overlap.
* ``pareto``        convex pairs with V ~ Pareto(alpha = 1.5, x_m = 4) clipped
  to [4, 1024]; about 30 % overlap.
* ``arm``           a 7-link serial arm (each link the hull of 64..256 points on
  an ellipsoid around the link) against 32 obstacle hulls of 64 points, every
  link-obstacle pair of each random joint configuration (224 pairs per
  configuration).

Every pair carries a shape-pair class for the warm-start model's embedding:
the type pair (5 x 5 classes) for ``mixed``, the pair of log2 vertex-count
buckets (9 x 9) for ``pareto``, link x 32 + obstacle (224) for ``arm``.

Overlap control: the translation of shape b is a uniform direction times
g * (rho_a + rho_b), rho the bounding-sphere radius and g ~ U[0, g_max]; g_max
was calibrated once with the FP64 oracle so that the overlap fraction lands on
the target (the achieved fraction is measured and reported by the bench).
"""
from dataclasses import dataclass, field

import numpy as np

from .layout import BOX, CAPSULE, CONVEX, CYLINDER, PAIR_DTYPE, SHAPE_DTYPE, SPHERE

SEED_BASE = 20240611
MIXED_CLASSES = 25
PARETO_CLASSES = 81
ARM_LINKS, ARM_OBSTACLES = 7, 32
ARM_CLASSES = ARM_LINKS * ARM_OBSTACLES
MIXED_G_MAX = 1.92   # calibrated: 40 % overlap on the mixed workload
CCD_G_MAX = 3.0      # translational CCD: start separations
CCD_REACH = 2.0      # and displacements (bounding-sphere sums)
PARETO_G_MAX = 1.66  # calibrated: 30 % overlap on the pareto workload


@dataclass
class Batch:
    name: str
    shapes: np.ndarray           # SHAPE_DTYPE [n_shapes]
    vertices: np.ndarray         # float32 [n_vertices, 4] (x, y, z, 0)
    pairs: np.ndarray            # PAIR_DTYPE [n_pairs]
    meta: dict = field(default_factory=dict)

    @property
    def n_pairs(self):
        return len(self.pairs)

    def subset(self, idx):
        """Pairs ``idx`` with only the shapes and vertices they use, re-indexed."""
        idx = np.asarray(idx)
        p = self.pairs[idx].copy()
        used = np.unique(np.concatenate([p["shape_a"], p["shape_b"]]))
        remap = np.full(len(self.shapes), -1, np.int64)
        remap[used] = np.arange(len(used))
        s = self.shapes[used].copy()
        counts = s["vert_count"].astype(np.int64)
        is_cvx = s["type"] == CONVEX
        counts[~is_cvx] = 0
        new_off = np.concatenate([[0], np.cumsum(counts)[:-1]])
        chunks = [self.vertices[o:o + c] for o, c in zip(s["vert_offset"].astype(np.int64), counts) if c > 0]
        verts = np.concatenate(chunks) if chunks else np.zeros((0, 4), np.float32)
        s["vert_offset"] = np.where(is_cvx, new_off, 0)
        p["shape_a"] = remap[p["shape_a"]]
        p["shape_b"] = remap[p["shape_b"]]
        return Batch(self.name + "[subset]", s, np.ascontiguousarray(verts, np.float32), p, dict(self.meta))


def _rng(seed):
    return np.random.Generator(np.random.Philox(seed))


def _normals(rng, shape):
    """Standard normals by Box-Muller from uniforms."""
    n = int(np.prod(shape))
    m = (n + 1) // 2
    u1 = rng.random(m)
    u2 = rng.random(m)
    rad = np.sqrt(-2.0 * np.log1p(-u1))
    z = np.concatenate([rad * np.cos(2 * np.pi * u2), rad * np.sin(2 * np.pi * u2)])[:n]
    return z.reshape(shape)


def unit_vectors(rng, n):
    v = _normals(rng, (n, 3))
    nrm = np.linalg.norm(v, axis=1, keepdims=True)
    nrm[nrm == 0] = 1.0
    return v / nrm


def random_rotations(rng, n):
    """Uniform random rotations (Shoemake's quaternion method), row-major 3x3."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    x, y = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    z, w = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    R = np.empty((n, 9))
    R[:, 0] = 1 - 2 * (y * y + z * z)
    R[:, 1] = 2 * (x * y - z * w)
    R[:, 2] = 2 * (x * z + y * w)
    R[:, 3] = 2 * (x * y + z * w)
    R[:, 4] = 1 - 2 * (x * x + z * z)
    R[:, 5] = 2 * (y * z - x * w)
    R[:, 6] = 2 * (x * z - y * w)
    R[:, 7] = 2 * (y * z + x * w)
    R[:, 8] = 1 - 2 * (x * x + y * y)
    return R


def log_uniform_counts(rng, n, lo, hi):
    u = rng.random(n)
    v = np.floor(np.exp(np.log(lo) + u * (np.log(hi + 1) - np.log(lo)))).astype(np.int64)
    return np.clip(v, lo, hi)


def pareto_counts(rng, n, alpha=1.5, xm=4, hi=1024):
    u = rng.random(n)
    v = np.floor(xm * (1.0 - u) ** (-1.0 / alpha)).astype(np.int64)
    return np.clip(v, xm, hi)


def _make_shapes(rng, types, lo, hi, counts):
    """Shapes of the given types; convex hull vertex counts from ``counts``."""
    n = len(types)
    s = np.zeros(n, SHAPE_DTYPE)
    s["type"] = types
    half = rng.random((n, 3)) * (hi - lo) + lo
    r = rng.random(n) * (hi - lo) + lo
    hl = rng.random(n) * (hi - lo) + lo
    rho = np.zeros(n)
    isb, iss, isc, isy, isx = (types == t for t in (BOX, SPHERE, CAPSULE, CYLINDER, CONVEX))
    s["param"][isb, :3] = 2 * half[isb]
    rho[isb] = np.linalg.norm(half[isb], axis=1)
    s["param"][iss, 0] = r[iss]
    rho[iss] = r[iss]
    s["param"][isc, 0] = r[isc]
    s["param"][isc, 1] = 2 * hl[isc]
    rho[isc] = r[isc] + hl[isc]
    s["param"][isy, 0] = r[isy]
    s["param"][isy, 1] = 2 * hl[isy]
    rho[isy] = np.sqrt(r[isy] ** 2 + hl[isy] ** 2)
    rho[isx] = r[isx]
    cvx_idx = np.nonzero(isx)[0]
    cnt = np.zeros(n, np.int64)
    cnt[cvx_idx] = counts(len(cvx_idx))
    off = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    s["vert_offset"] = np.where(isx, off, 0)
    s["vert_count"] = cnt
    nv = int(cnt.sum())
    verts = np.zeros((nv, 4), np.float32)
    if nv:
        pts = unit_vectors(rng, nv) * np.repeat(r, cnt)[:, None]
        verts[:, :3] = pts
        # interior point (vertex mean) for MPR-style queries, in param[0:3]
        sums = np.add.reduceat(verts[:, :3].astype(np.float64), off[cvx_idx], axis=0)
        s["param"][cvx_idx, :3] = sums / cnt[cvx_idx, None]
    s["param"][:, 3] = rho
    return s, verts, rho


def _pairs(rng, n, rho, translation):
    p = np.zeros(n, PAIR_DTYPE)
    p["shape_a"] = np.arange(0, 2 * n, 2)
    p["shape_b"] = np.arange(1, 2 * n, 2)
    p["rot"] = random_rotations(rng, n)
    if translation == "cube":
        p["trans"] = rng.random((n, 3)) - 0.5
    else:
        g_max = float(translation)
        d = unit_vectors(rng, n)
        g = rng.random(n) * g_max
        p["trans"] = d * (g * (rho[0::2] + rho[1::2]))[:, None]
    return p


def plain_small(n_pairs=4096, seed=SEED_BASE + 0):
    rng = _rng(seed)
    types = np.full(2 * n_pairs, CONVEX, np.int32)
    s, v, rho = _make_shapes(rng, types, 0.05, 0.5, lambda k: np.full(k, 32, np.int64))
    p = _pairs(rng, n_pairs, rho, "cube")
    return Batch("plain_small", s, v, p, {"seed": seed, "vertices_per_hull": 32})


def mixed(n_pairs=1_000_000, seed=SEED_BASE + 1, g_max=MIXED_G_MAX):
    rng = _rng(seed)
    choice = np.array([BOX, SPHERE, CAPSULE, CYLINDER, CONVEX], np.int32)
    types = choice[np.minimum((rng.random(2 * n_pairs) * 5).astype(np.int64), 4)]
    s, v, rho = _make_shapes(rng, types, 0.02, 0.4, lambda k: log_uniform_counts(rng, k, 8, 256))
    p = _pairs(rng, n_pairs, rho, g_max)
    cls = np.zeros(CONVEX + 1, np.uint32)
    cls[[BOX, SPHERE, CAPSULE, CYLINDER, CONVEX]] = np.arange(5)
    p["pair_class"] = 5 * cls[s["type"][p["shape_a"]]] + cls[s["type"][p["shape_b"]]]
    return Batch("mixed", s, v, p, {"seed": seed, "g_max": g_max})


def ccd(n_pairs=1_000_000, seed=SEED_BASE + 9, g_max=CCD_G_MAX, reach=CCD_REACH):
    """Translational continuous collision: pairs of the mixed workload's kinds
    and sizes, start separations as the mixed workload's at g_max, shape a
    moving along a uniform random unit axis of its frame by up to `reach`
    times the pair's bounding-sphere sum.  Returns (Batch, disp [n, 4]
    float32: axis, distance)."""
    rng = _rng(seed)
    choice = np.array([BOX, SPHERE, CAPSULE, CYLINDER, CONVEX], np.int32)
    types = choice[np.minimum((rng.random(2 * n_pairs) * 5).astype(np.int64), 4)]
    s, v, rho = _make_shapes(rng, types, 0.02, 0.4, lambda k: log_uniform_counts(rng, k, 8, 256))
    p = _pairs(rng, n_pairs, rho, g_max)
    cls = np.zeros(CONVEX + 1, np.uint32)
    cls[[BOX, SPHERE, CAPSULE, CYLINDER, CONVEX]] = np.arange(5)
    p["pair_class"] = 5 * cls[s["type"][p["shape_a"]]] + cls[s["type"][p["shape_b"]]]
    disp = np.zeros((n_pairs, 4), np.float32)
    disp[:, :3] = unit_vectors(rng, n_pairs)
    disp[:, 3] = rng.random(n_pairs) * reach * (rho[0::2] + rho[1::2])
    return Batch("ccd", s, v, p, {"seed": seed, "g_max": g_max, "reach": reach}), disp


def pareto(n_pairs=4_000_000, seed=SEED_BASE + 4, g_max=PARETO_G_MAX):
    rng = _rng(seed)
    types = np.full(2 * n_pairs, CONVEX, np.int32)
    s, v, rho = _make_shapes(rng, types, 0.02, 0.4, lambda k: pareto_counts(rng, k))
    p = _pairs(rng, n_pairs, rho, g_max)
    bucket = np.clip(np.floor(np.log2(np.maximum(s["vert_count"], 1))).astype(np.int64) - 2, 0, 8)
    p["pair_class"] = 9 * bucket[p["shape_a"]] + bucket[p["shape_b"]]
    return Batch("pareto", s, v, p, {"seed": seed, "g_max": g_max})


def scene(n_objects=100_000, seed=SEED_BASE + 7, density=0.25, identity_fraction=0.2):
    """A scene of posed objects for the broadphase feed: n_objects shapes of
    the mixed workload's kinds and sizes (one shape per object), world poses
    with uniform rotations (identity for identity_fraction of them: the
    CollisionObject::computeAABB shortcut) and translations uniform in a cube
    whose edge gives ``density`` objects per bounding-sphere volume.
    Returns (Batch of the shapes, shape_ids [n] uint32, poses [n, 12] float32)."""
    rng = _rng(seed)
    choice = np.array([BOX, SPHERE, CAPSULE, CYLINDER, CONVEX], np.int32)
    types = choice[np.minimum((rng.random(n_objects) * 5).astype(np.int64), 4)]
    s, v, rho = _make_shapes(rng, types, 0.02, 0.4, lambda k: log_uniform_counts(rng, k, 8, 256))
    vol = float(np.sum(4.0 / 3.0 * np.pi * rho ** 3)) / density
    edge = vol ** (1.0 / 3.0)
    R = random_rotations(rng, n_objects).reshape(-1, 9)
    ident = rng.random(n_objects) < identity_fraction
    R[ident] = np.eye(3).ravel()
    t = (rng.random((n_objects, 3)) - 0.5) * edge
    poses = np.concatenate([R, t], axis=1).astype(np.float32)
    ids = np.arange(n_objects, dtype=np.uint32)
    b = Batch("scene", s, v, np.zeros(0, PAIR_DTYPE), {"seed": seed, "edge": edge, "density": density})
    return b, ids, poses


def _rot(axis, ang):
    """Batched rotation matrices [n, 3, 3] about a coordinate axis."""
    c, s_ = np.cos(ang), np.sin(ang)
    R = np.zeros((len(ang), 3, 3))
    i, j = {"x": (1, 2), "z": (0, 1)}[axis]
    k = 3 - i - j
    R[:, k, k] = 1.0
    R[:, i, i] = c
    R[:, j, j] = c
    R[:, i, j] = -s_
    R[:, j, i] = s_
    return R


def arm(n_configs=100_000, seed=SEED_BASE + 3, chunk=8192):
    """7-link arm against 32 obstacles: every link-obstacle pair of n_configs
    random joint configurations (pair index (config * 7 + link) * 32 + obstacle;
    shape a the link, shape b the obstacle, posed in the link's frame)."""
    rng = _rng(seed)
    L, O = ARM_LINKS, ARM_OBSTACLES
    length = 0.20 + 0.15 * rng.random(L)        # joint-to-joint distance along the link's x axis
    radius = 0.04 + 0.03 * rng.random(L)
    link_nv = (64 + np.floor(rng.random(L) * 193)).astype(np.int64)  # 64..256
    d_off = 0.10 * rng.random(L)                # DH offsets along z
    twist = np.where(np.arange(L) % 2 == 0, np.pi / 2, -np.pi / 2)
    obs_r = 0.06 + 0.12 * rng.random(O)
    obs_dir = unit_vectors(rng, O)
    obs_dist = 0.3 + 0.6 * rng.random(O)
    obs_pos = obs_dir * obs_dist[:, None] + np.array([0.0, 0.0, 0.3])
    obs_rot = random_rotations(rng, O).reshape(O, 3, 3)
    # shapes: links are hulls of points on an ellipsoid spanning the link, obstacles of points on a sphere
    counts = np.concatenate([link_nv, np.full(O, 64, np.int64)])
    s = np.zeros(L + O, SHAPE_DTYPE)
    s["type"] = CONVEX
    s["vert_count"] = counts
    s["vert_offset"] = np.concatenate([[0], np.cumsum(counts)[:-1]])
    verts = np.zeros((int(counts.sum()), 4), np.float32)
    u = unit_vectors(rng, int(counts.sum()))
    for i in range(L + O):
        a, c = int(s["vert_offset"][i]), int(counts[i])
        if i < L:
            semi = np.array([0.5 * length[i] + 0.5 * radius[i], radius[i], radius[i]])
            pts = u[a:a + c] * semi + np.array([0.5 * length[i], 0.0, 0.0])
        else:
            pts = u[a:a + c] * obs_r[i - L]
        verts[a:a + c, :3] = pts
        s["param"][i, :3] = pts.mean(axis=0)
        s["param"][i, 3] = np.linalg.norm(pts, axis=1).max()
    # joint configurations and link frames
    q = (rng.random((n_configs, L)) * 2.0 - 1.0) * np.pi
    pairs = np.zeros(n_configs * L * O, PAIR_DTYPE)
    obs_R = obs_rot[None]                                       # [1, O, 3, 3]
    for c0 in range(0, n_configs, chunk):
        qc = q[c0:c0 + chunk]
        m = len(qc)
        R = np.broadcast_to(np.eye(3), (m, 3, 3)).copy()
        t = np.zeros((m, 3))
        link_R = np.empty((m, L, 3, 3))
        link_t = np.empty((m, L, 3))
        for j in range(L):
            R = R @ _rot("z", qc[:, j])
            t = t + R[:, :, 2] * d_off[j]
            link_R[:, j] = R
            link_t[:, j] = t
            t = t + R[:, :, 0] * length[j]
            R = R @ _rot("x", np.full(m, twist[j]))
        RT = np.swapaxes(link_R, -1, -2)                        # [m, L, 3, 3]
        rel_R = np.einsum("mlij,ojk->mloik", RT, obs_R[0])       # [m, L, O, 3, 3]
        rel_t = np.einsum("mlij,mloj->mloi", RT, obs_pos[None, None] - link_t[:, :, None, :])
        blk = pairs[c0 * L * O:(c0 + m) * L * O]
        blk["shape_a"] = np.broadcast_to(np.arange(L)[None, :, None], (m, L, O)).ravel()
        blk["shape_b"] = np.broadcast_to(L + np.arange(O)[None, None, :], (m, L, O)).ravel()
        blk["rot"] = rel_R.reshape(-1, 9)
        blk["trans"] = rel_t.reshape(-1, 3)
        blk["pair_class"] = np.broadcast_to(np.arange(L)[None, :, None] * O + np.arange(O)[None, None, :],
                                            (m, L, O)).ravel()
    return Batch("arm", s, verts, pairs, {"seed": seed, "configs": n_configs, "links": L, "obstacles": O,
                                          "link_vertices": link_nv.tolist()})


# ------------------------------------------------------------------ meshes --
_ICO_T = (1.0 + 5.0 ** 0.5) / 2.0
_ICO_V = np.array([(-1, _ICO_T, 0), (1, _ICO_T, 0), (-1, -_ICO_T, 0), (1, -_ICO_T, 0), (0, -1, _ICO_T),
                   (0, 1, _ICO_T), (0, -1, -_ICO_T), (0, 1, -_ICO_T), (_ICO_T, 0, -1), (_ICO_T, 0, 1),
                   (-_ICO_T, 0, -1), (-_ICO_T, 0, 1)], np.float64)
_ICO_F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
          (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
          (8, 6, 7), (9, 8, 1)]


@dataclass
class Mesh:
    vertices: np.ndarray   # float32 [nv, 3]
    triangles: np.ndarray  # int32 [nt, 3]


def geodesic_sphere(freq, radius=1.0, noise=0.0, seed=SEED_BASE + 2):
    """Class I geodesic sphere: every icosahedron face split into freq^2
    triangles (20 freq^2 triangles, 10 freq^2 + 2 vertices), projected to the
    sphere, each vertex then moved radially by N(0, noise) metres."""
    keys = {}
    verts = []
    tris = []

    def vid(face, i, j):
        a, b, c = face
        w = {a: freq - i - j, b: i, c: j}
        key = tuple(sorted((k, v) for k, v in w.items() if v > 0))
        if key not in keys:
            keys[key] = len(verts)
            p = (w[a] * _ICO_V[a] + w[b] * _ICO_V[b] + w[c] * _ICO_V[c]) / freq
            verts.append(p / np.linalg.norm(p))
        return keys[key]

    for face in _ICO_F:
        for i in range(freq):
            for j in range(freq - i):
                tris.append((vid(face, i, j), vid(face, i + 1, j), vid(face, i, j + 1)))
                if i + j + 1 < freq:
                    tris.append((vid(face, i + 1, j), vid(face, i + 1, j + 1), vid(face, i, j + 1)))
    v = np.array(verts)
    r = np.full(len(v), float(radius))
    if noise:
        r = r + noise * _normals(_rng(seed), (len(v),))
    return Mesh((v * r[:, None]).astype(np.float32), np.array(tris, np.int32))


def mesh_poses(n, max_dist=0.8, seed=SEED_BASE + 3):
    """Random relative poses: translation uniform in a ball of radius max_dist,
    uniform rotation; float32 [n, 12] (rotation row-major, translation)."""
    rng = _rng(seed)
    R = random_rotations(rng, n)
    d = unit_vectors(rng, n)
    t = d * (max_dist * rng.random(n) ** (1.0 / 3.0))[:, None]
    return np.concatenate([R, t], axis=1).astype(np.float32)


def mesh_pair(freq=50, radius=0.3, noise=0.05, seed=SEED_BASE + 2):
    """The two bumpy 50k-triangle spheres of the mesh-mesh workload."""
    return (geodesic_sphere(freq, radius, noise, seed), geodesic_sphere(freq, radius, noise, seed + 100))
