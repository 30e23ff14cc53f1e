"""Writes tests/golden/convex_ref.npz: seeded inputs from the three convex
workloads together with the outputs of the reference itself (its own GJK / EPA /
MPR compiled from the reference sources into oracle/_ref by oracle/build_ref.sh)
for GJKSolver::shapeSignedDistance and for fcl::collide with and without
penetration.  Run where the reference sources exist:

    python tests/golden/make_golden.py
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


def capsule_pair_case():
    from fclg.layout import CAPSULE, PAIR_DTYPE, SHAPE_DTYPE
    R1 = np.array([[-0.1823781667231642312, 0.5834536857025155454, -0.7914038166087196124],
                   [-0.4082009544663793843, 0.6873272332027842157, 0.6007938542216808564],
                   [0.8944887842088544705, 0.4326234750195090406, 0.112812870660265227]])
    t1 = np.array([1.8916015625, 1.1961669921875, 1.0020751953125])
    R2 = np.array([[0.317527870519881128, -0.3295648710688394156, -0.8891361241117632375],
                   [-0.1094271233639760865, 0.9186616351567586936, -0.3795872821412688003],
                   [0.9419138793517136676, 0.217825149715291877, 0.2556373369367547776]])
    t2 = np.array([1.6461181640625, 0.496826171875, 0.091796875])
    s = np.zeros(2, SHAPE_DTYPE)
    s["type"] = CAPSULE
    s["param"][:, 0] = 0.5
    s["param"][:, 1] = 1.3
    p = np.zeros(1, PAIR_DTYPE)
    p["shape_b"] = 1
    p["rot"] = (R1.T @ R2).ravel()
    p["trans"] = R1.T @ (t2 - t1)
    return workloads.Batch("capsule_pair", s, np.zeros((1, 4), np.float32), p)


def main():
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libfcl_ref.so missing: the reference sources are needed")
    out = {}
    for name, batch in (("plain_small", workloads.plain_small().subset(np.arange(512))),
                        ("mixed", workloads.mixed(4096).subset(np.arange(1536))),
                        ("pareto", workloads.pareto(4096).subset(np.arange(512)))):
        sd = oracle.ref_signed_distance(batch)
        cb = oracle.ref_collide(batch, False)
        cc = oracle.ref_collide(batch, True)
        out[name + "/shapes"] = batch.shapes
        out[name + "/vertices"] = batch.vertices
        out[name + "/pairs"] = batch.pairs
        out[name + "/signed_distance"] = sd
        out[name + "/collide_bool"] = cb
        out[name + "/collide_contact"] = cc
    # test/cvx_collide/test_gjk2_distance.cpp:70-154: the hard-coded capsule
    # pair, run with GJK2(1000, 1e-7) as that test does.
    cap = capsule_pair_case()
    out["capsule_pair/shapes"] = cap.shapes
    out["capsule_pair/vertices"] = cap.vertices
    out["capsule_pair/pairs"] = cap.pairs
    out["capsule_pair/signed_distance"] = oracle.ref_signed_distance(cap, gjk_max_iter=1000, gjk_tol=1e-7)
    np.savez_compressed(os.path.join(HERE, "convex_ref.npz"), **out)
    print("wrote", os.path.join(HERE, "convex_ref.npz"))


if __name__ == "__main__":
    main()
