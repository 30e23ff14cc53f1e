"""Packed record layouts shared by the C ABI (include/fclg.h) and the host code.

Shape type codes are the reference's GJKShapeType values
(include/fcl/cvx_collide/gjk_shape.h:9-28).  Shape parameters follow the fcl
geometry classes: Box stores full side lengths (geometry/shape/box.h:63),
Sphere its radius (sphere.h:56), Capsule / Cylinder radius and full length lz
(capsule.h:57-60, cylinder.h:57-60).  A pair carries the pose of shape b in
shape a's frame, i.e. the reference's MinkowskiDiff::toshape0
(narrowphase/detail/gjk_solver-inl.h:84-85).
"""
import numpy as np

BOX, SPHERE, CAPSULE, CYLINDER, CONVEX = 0, 1, 3, 5, 100
TYPE_NAMES = {BOX: "box", SPHERE: "sphere", CAPSULE: "capsule", CYLINDER: "cylinder", CONVEX: "convex"}

SHAPE_DTYPE = np.dtype(
    [("type", "<i4"), ("vert_offset", "<u4"), ("vert_count", "<u4"), ("reserved", "<u4"), ("param", "<f4", (4,))],
    align=False,
)
PAIR_DTYPE = np.dtype(
    [("shape_a", "<u4"), ("shape_b", "<u4"), ("rot", "<f4", (9,)), ("trans", "<f4", (3,)),
     ("flags", "<u4"), ("pair_class", "<u4")],
    align=False,
)
# fclg_result: what the GPU writes per pair (48 bytes).
RESULT_DTYPE = np.dtype(
    [("distance", "<f4"), ("normal", "<f4", (3,)), ("p_a", "<f4", (3,)), ("p_b", "<f4", (3,)),
     ("status", "<i4"), ("iterations", "<u2"), ("collide", "u1"), ("ok", "u1")],
    align=False,
)
# fclg_result64: the FP64 separation distance (fclg_distance64)
RESULT64_DTYPE = np.dtype(
    [("distance", "<f8"), ("p_a", "<f8", (3,)), ("p_b", "<f8", (3,)), ("status", "<i4"), ("iterations", "<u2"),
     ("collide", "u1"), ("ok", "u1")],
    align=False,
)
assert SHAPE_DTYPE.itemsize == 32 and PAIR_DTYPE.itemsize == 64 and RESULT_DTYPE.itemsize == 48
assert RESULT64_DTYPE.itemsize == 64

# Status word of fclg_result: bits 0-7 GJK_Status (gjk.h:13-28), bits 8-15
# EPA_Status + 1 (epa.h:14; 0 = EPA not run), bit 16 = capacity overflow.
GJK_INTERSECT, GJK_SEPARATED, GJK_NO_PROGRESS, GJK_ITER_LIMIT, GJK_FAILED = 0, 1, 2, 3, 4
EPA_FAILED, EPA_OK, EPA_TOUCHING, EPA_ITER_LIMIT, EPA_MALLOC_FAILED = 0, 1, 2, 3, 4


def gjk_status(status):
    return np.asarray(status) & 0xFF


def epa_status(status):
    """EPA_Status per pair, -1 where EPA did not run."""
    return ((np.asarray(status) >> 8) & 0xFF).astype(np.int32) - 1
