"""Builds lib/libfclg.so (the CUDA kernels + C ABI) for sm_103a with nvcc.

Translation units compile in parallel; objects land in _build/ and the shared
library in lib/ (both git-ignored).  Rebuilds only when a source is newer.
"""
import concurrent.futures
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
# FCLG_BUILD_TAG builds a variant beside the default one (_build_<tag>/,
# lib_<tag>/), FCLG_NVCC_FLAGS adds flags (e.g. -D overrides of the launch
# constants); fclg.api loads a variant through FCLG_LIB.
_TAG = os.environ.get("FCLG_BUILD_TAG", "")
BUILD = os.path.join(PKG, "_build" + ("_" + _TAG if _TAG else ""))
LIB_DIR = os.path.join(PKG, "lib" + ("_" + _TAG if _TAG else ""))
LIB = os.path.join(LIB_DIR, "libfclg.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include"), "-I", CSRC] + os.environ.get("FCLG_NVCC_FLAGS", "").split()


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "fclg.h"))
    return hs


def _obj(src):
    return os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def compile_one(src, verbose_ptxas=False):
    obj = _obj(src)
    cmd = [NVCC, *ARCH, *FLAGS, "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return r.stderr


def build(force=False, verbose_ptxas=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = sources()
    hdrs = headers()
    todo = [s for s in srcs if force or verbose_ptxas or _stale(_obj(s), [s] + hdrs)]
    logs = {}
    if todo:
        with concurrent.futures.ThreadPoolExecutor(max_workers=jobs or min(os.cpu_count() or 8, len(todo))) as ex:
            for s, log in zip(todo, ex.map(lambda s: compile_one(s, verbose_ptxas), todo)):
                logs[s] = log
    objs = [_obj(s) for s in srcs]
    if todo or _stale(LIB, objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return logs


if __name__ == "__main__":
    out = build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    for s, log in out.items():
        if log:
            print("==", os.path.basename(s))
            print(log)
    print(LIB)
