"""The closed-form shape-pair solvers of fcl::collide pinned to the reference.

The reference's GJKSolver<double>::shapeIntersect, compiled from its sources
(oracle/_ref/libfcl_ref_mesh.so), dispatches sphere-sphere, sphere-box,
sphere-capsule, sphere-cylinder (either order) and box-box pairs to
sphereSphereIntersect (primitive_shape_algorithm/sphere_sphere-inl.h:49),
sphereBoxIntersect (sphere_box-inl.h:85), sphereCapsuleIntersect
(sphere_capsule-inl.h:71), sphereCylinderIntersect (sphere_cylinder-inl.h:96)
and boxBoxIntersect (box_box-inl.h:823-839).  The FP64 restatement
(oracle/orc_analytic.hpp, used by the GPU parity tests) must give the same
collision flags, and on colliding pairs the same contact normal and depth bit
for bit (box-box: the first deepest of the reference's contacts, the one a
one-contact request keeps) and the same position to rounding (the restatement
reports it as p_a / p_b = pos +- depth / 2 along the normal).
"""
import numpy as np
import pytest

from fclg import workloads
from fclg.layout import BOX, CAPSULE, CYLINDER, SPHERE

CODE = {SPHERE: 0, BOX: 1, CAPSULE: 2, CYLINDER: 3}


def _closed_form_pairs(n_max, seed):
    b = workloads.mixed(120000, seed=seed)
    s, p = b.shapes, b.pairs
    ta, tb = s["type"][p["shape_a"]], s["type"][p["shape_b"]]
    prim = np.isin(ta, list(CODE)) & np.isin(tb, list(CODE))
    keep = prim & (((ta == SPHERE) | (tb == SPHERE)) | ((ta == BOX) & (tb == BOX)))
    return b.subset(np.nonzero(keep)[0][:n_max])


@pytest.mark.parametrize("seed", (777, 778))
def test_closed_form_solvers_equal_reference(oracle_lib, seed):
    if not oracle_lib.ref_mesh_available():
        pytest.skip("reference sources not available: oracle/_ref/libfcl_ref_mesh.so not built")
    sub = _closed_form_pairs(20000, seed)
    s, p = sub.shapes, sub.pairs
    ca = np.array([CODE[t] for t in s["type"][p["shape_a"]]])
    cb = np.array([CODE[t] for t in s["type"][p["shape_b"]]])
    pa = s["param"][p["shape_a"], :3].astype(np.float64)
    pb = s["param"][p["shape_b"], :3].astype(np.float64)
    poses = np.concatenate([p["rot"].astype(np.float64).reshape(-1, 9),
                            p["trans"].astype(np.float64).reshape(-1, 3)], 1)
    ret, out = oracle_lib.ref_analytic(ca, pa, cb, pb, poses)
    orc = oracle_lib.collide(sub, want_contact=True)
    assert np.all(ret >= 0)
    hit = ret > 0
    assert np.array_equal(hit, orc["ok"] == 1)
    assert 0.2 < hit.mean() < 0.8
    # every type pair present, both orders
    assert len(set(zip(ca[hit], cb[hit]))) == 8
    depth = np.where(np.arange(4)[None, :] < ret[:, None], out[:, :, 6], -np.inf)
    k = np.argmax(depth, axis=1)  # first of maximal depth
    rc = out[np.arange(len(ret)), k]
    assert np.array_equal(rc[hit, :3], orc["normal"][hit])
    assert np.array_equal(rc[hit, 6], -orc["distance"][hit])
    pos = 0.5 * (orc["p0"] + orc["p1"])
    assert np.abs(rc[hit, 3:6] - pos[hit]).max() <= 1e-15
