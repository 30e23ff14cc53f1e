"""The fcl-style C++ API (include/fclg_fcl.hpp): compiles here against the
C ABI; runs its known-answer cases (tests/cpp/fcl_compat_test.cpp) on the GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "fcl_compat_test.cpp")
LIB_DIR = os.path.join(ROOT, "mind-fcl_gb300", "lib")


def _build(tmp_path, link):
    exe = str(tmp_path / "fcl_compat_test")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC]
    if link:
        cmd += ["-L", LIB_DIR, "-lfclg", "-Wl,-rpath," + LIB_DIR, "-o", exe]
    else:
        cmd += ["-fsyntax-only"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_header_compiles(tmp_path):
    _build(tmp_path, link=False)


@pytest.mark.gpu
def test_known_answers_on_gpu(tmp_path):
    import __graft_entry__
    __graft_entry__.build()
    exe = _build(tmp_path, link=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all passed" in r.stdout
