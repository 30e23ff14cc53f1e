"""The FP64 GJK of the FP64 distance kernel (mind-fcl_gb300/csrc/gjk64.cuh),
built for the CPU (tests/cpp/gjk64_host.cpp, no contraction), against the
reference's own outputs (tests/golden/convex_ref.npz): every GJK status equal,
and on every pair the reference solved as separated with valid witness points
the same distance and points, bit for bit.  The GPU build of the same header
is checked against the same outputs in tests/test_gpu_fp64.py; this test pins
the restatement itself without a GPU.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from fclg import workloads
from fclg.layout import GJK_INTERSECT, GJK_SEPARATED, RESULT64_DTYPE, gjk_status

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "gjk64_host.cpp")
CSRC = os.path.join(ROOT, "mind-fcl_gb300", "csrc")
GOLDEN = os.path.join(ROOT, "tests", "golden", "convex_ref.npz")

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")


@pytest.fixture(scope="module")
def g64(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("g64") / "libg64.so")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Werror", "-Wno-unknown-pragmas", "-shared", "-fPIC",
           "-I", CSRC, SRC, "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(so)
    vp = ctypes.c_void_p
    lib.g64_run.argtypes = [vp, ctypes.c_uint32, vp, vp, ctypes.c_uint32, ctypes.c_double, ctypes.c_int, vp]
    lib.g64_run.restype = None

    def run(batch, tol=1e-6, max_iter=128):
        sh = np.ascontiguousarray(batch.shapes)
        v = np.ascontiguousarray(batch.vertices, np.float32)
        p = np.ascontiguousarray(batch.pairs)
        out = np.zeros(len(p), RESULT64_DTYPE)
        lib.g64_run(sh.ctypes.data, len(sh), v.ctypes.data, p.ctypes.data, len(p), tol, max_iter, out.ctypes.data)
        return out
    return run


@pytest.mark.parametrize("name", ["plain_small", "mixed", "pareto", "capsule_pair"])
def test_host_build_is_the_reference(g64, name):
    g = np.load(GOLDEN)
    batch = workloads.Batch(name, g[name + "/shapes"], g[name + "/vertices"], g[name + "/pairs"])
    ref = g[name + "/signed_distance"]
    # the capsule pair is test_gjk2_distance.cpp:70-154, run there with GJK2(1000, 1e-7)
    got = g64(batch, 1e-7, 1000) if name == "capsule_pair" else g64(batch)
    rs = gjk_status(ref["gjk_status"])
    assert np.array_equal(got["status"], rs)
    sep = (rs == GJK_SEPARATED) & (ref["ok"] == 1)
    assert np.all(got["ok"][sep] == 1)
    assert np.array_equal(got["distance"][sep], ref["distance"][sep])
    assert np.array_equal(got["p_a"][sep], ref["p0"][sep])
    assert np.array_equal(got["p_b"][sep], ref["p1"][sep])
    ov = rs == GJK_INTERSECT
    assert np.all(got["collide"][ov] == 1) and np.all(got["ok"][ov] == 0) and np.all(got["distance"][ov] == -1.0)


def test_host_build_is_the_oracle_on_plain(g64, oracle_lib):
    """All 4096 pairs of the plain workload against the FP64 oracle
    (shapeSignedDistance: the same GJK on separated pairs)."""
    batch = workloads.plain_small()
    got = g64(batch)
    ref = oracle_lib.signed_distance(batch)
    rs = gjk_status(ref["gjk_status"])
    assert np.array_equal(got["status"], rs)
    sep = (rs == GJK_SEPARATED) & (ref["ok"] == 1)
    assert sep.mean() > 0.3
    assert np.array_equal(got["distance"][sep], ref["distance"][sep])


def test_host_build_invalid_and_limits(g64):
    """A pair whose shape index is out of range gets GJK_Failed, ok = 0 and
    distance -1; an iteration limit of 1 leaves pairs undecided or decided
    without a certified distance, never with a wrong flag."""
    batch = workloads.plain_small(256)
    bad = batch.pairs.copy()
    bad["shape_b"][::7] = len(batch.shapes) + 5
    b2 = workloads.Batch("bad", batch.shapes, batch.vertices, bad)
    got = g64(b2)
    sel = np.arange(len(bad)) % 7 == 0
    assert np.all(got["status"][sel] == 4) and np.all(got["ok"][sel] == 0)
    assert np.all(got["distance"][sel] == -1.0)
    full = g64(batch)
    short = g64(batch, 1e-6, 1)
    sep_short = (short["status"] == GJK_SEPARATED) & (short["ok"] == 1)
    # a separation certificate found within one iteration is a true separation
    assert np.all(full["status"][sep_short] == GJK_SEPARATED)
    assert np.all(short["distance"][sep_short] >= full["distance"][sep_short] - 1e-9)
