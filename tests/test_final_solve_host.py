"""EPA's FP64 final closest-face solve (epa_final_solve,
mind-fcl_gb300/csrc/device_math.cuh: the function the epa_finalize launch runs
a thread per pair), built for the CPU from the same header
(tests/cpp/final_solve_host.cu), against an independent FP64 computation of
the same quantities: the point of the face's triangle nearest the origin as
the best of the interior projection (when its barycentric weights are all
non-negative), the three edges' clamped projections and the three vertices,
the witness points interpolated with that point's barycentric weights, and
the depth |q|.  Cases: the origin projecting inside the face (EPA's usual
final face), onto an edge or vertex region, slivers, and collinear faces,
which fall back to the last support pair.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "final_solve_host.cu")
CSRC = os.path.join(ROOT, "mind-fcl_gb300", "csrc")

pytestmark = pytest.mark.skipif(shutil.which("nvcc") is None, reason="no nvcc")


@pytest.fixture(scope="module")
def solve(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("fs") / "libfs.so")
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2", "-Xcompiler", "-fPIC",
           "-shared", "-I", CSRC, SRC, "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(so)
    lib.fs_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.fs_run.restype = None

    def run(cases):
        c = np.ascontiguousarray(cases, np.float32).reshape(-1, 24)
        out = np.zeros((len(c), 7), np.float32)
        lib.fs_run(c.ctypes.data, len(c), out.ctypes.data)
        return out
    return run


def _closest(a, b, c):
    """Barycentric weights of the point of triangle abc nearest the origin:
    the best of the interior projection and the edge / vertex candidates."""
    best, lam = np.inf, None
    n = np.cross(b - a, c - a)
    nn = n @ n
    if nn > 0:
        p = n * ((a @ n) / nn)                       # projection of the origin onto the plane
        l1 = (np.cross(b - p, c - p) @ n) / nn
        l2 = (np.cross(c - p, a - p) @ n) / nn
        l3 = 1.0 - l1 - l2
        if min(l1, l2, l3) >= 0:
            best, lam = p @ p, np.array([l1, l2, l3])
    for i, j in ((0, 1), (1, 2), (2, 0)):
        P = (a, b, c)
        e = P[j] - P[i]
        t = 0.0 if e @ e == 0 else float(np.clip(-(P[i] @ e) / (e @ e), 0.0, 1.0))
        q = P[i] + t * e
        if q @ q < best - 1e-300:
            best = q @ q
            lam = np.zeros(3)
            lam[i], lam[j] = 1.0 - t, t
    return lam


def _expected(case):
    v = case.reshape(8, 3).astype(np.float64)
    a, b, c, pa = v[0], v[1], v[2], v[3:6]
    lam = _closest(a, b, c)
    q = lam @ v[0:3]
    p0 = lam @ pa
    return p0, p0 - q, np.sqrt(q @ q)


def _cases(rng, n):
    out = []
    for k in range(n):
        kind = k % 4
        a, b, c = rng.normal(size=(3, 3)) * rng.uniform(0.01, 0.5)
        if kind == 0:
            # EPA's final face: the origin projects inside, at depth d below the face
            nrm = rng.normal(size=3)
            nrm /= np.linalg.norm(nrm)
            u = np.cross(nrm, [1.0, 0.0, 0.0] if abs(nrm[0]) < 0.9 else [0.0, 1.0, 0.0])
            u /= np.linalg.norm(u)
            w = np.cross(nrm, u)
            d = rng.uniform(1e-4, 0.2)
            ang = np.sort(rng.uniform(0, 2 * np.pi, 3))
            r = rng.uniform(0.02, 0.5, 3)
            a, b, c = [d * nrm + ri * (np.cos(t) * u + np.sin(t) * w) for ri, t in zip(r, ang)]
        elif kind == 1:
            # a sliver: c close to the line ab
            c = a + rng.uniform(0.2, 0.8) * (b - a) + rng.normal(size=3) * 1e-5
        pa = rng.normal(size=(3, 3)) * 0.3
        cand = rng.normal(size=(2, 3)) * 0.3
        out.append(np.concatenate([a, b, c, pa.ravel(), cand.ravel()]))
    return np.array(out, np.float32)


def test_final_solve_against_closest_point(solve):
    rng = np.random.default_rng(11)
    cases = _cases(rng, 4000)
    got = solve(cases)
    scale = np.abs(cases[:, :18].astype(np.float64)).max(axis=1) + 1e-3
    for i, case in enumerate(cases):
        p0, p1, depth = _expected(case)
        # float outputs of FP64 values: a few FP32 roundings of the inputs' magnitude
        tol = 4e-7 * scale[i]
        assert abs(got[i, 6] - depth) <= tol, (i, got[i, 6], depth)
        assert np.all(np.abs(got[i, 0:3] - p0) <= 8 * tol), (i, got[i, 0:3], p0)
        assert np.all(np.abs(got[i, 3:6] - p1) <= 8 * tol), (i, got[i, 3:6], p1)


def test_final_solve_degenerate_face_falls_back(solve):
    rng = np.random.default_rng(12)
    cases = _cases(rng, 64)
    # collinear (a, 2a, 4a: exact in FP32 and their FP64 cross product exactly
    # zero) and coincident faces: the last support pair is the answer
    a = cases[:, 0:3]
    cases[:, 3:6] = a * 2.0
    cases[:, 6:9] = a * 4.0
    cases[32:, 3:6] = a[32:]
    cases[32:, 6:9] = a[32:]
    got = solve(cases)
    fa, fb = cases[:, 18:21], cases[:, 21:24]
    assert np.array_equal(got[:, 0:3], fa) and np.array_equal(got[:, 3:6], fb)
    assert np.allclose(got[:, 6], np.linalg.norm(fa.astype(np.float64) - fb, axis=1), rtol=1e-6, atol=0)
