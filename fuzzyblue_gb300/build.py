"""Builds fuzzyblue_gb300/lib/libfuzzyblue_cuda.so (sm_103a) in-tree.

Translation units are compiled in parallel with nvcc, one -gencode each:
  csrc/fb_kernels_plain.cu  PLAIN passes, --fmad=false (no FMA contraction)
  csrc/fb_kernels_mixed.cu  MIXED passes
  csrc/fb_capi.cu           C ABI, build planning, CUDA graphs
  csrc/fb_util.cu           f16 export, tile-shape defaults
  csrc/fb_serve.cu          request loop with HBM admission and a resident LUT cache
  csrc/fb_tune.cu           tile-shape autotuner
  csrc/fb_noalloc.cu        a build that allocates nothing (fixed device scratch)
  csrc/fb_render.cu         headless sky pass and surface lighting on the tables, --fmad=false
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIB_DIR, "libfuzzyblue_cuda.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", os.path.join(ROOT, "include")]
UNITS = {
    "fb_kernels_plain.cu": ["--fmad=false"],
    "fb_kernels_mixed.cu": [],
    "fb_capi.cu": [],
    "fb_util.cu": [],
    "fb_serve.cu": [],
    "fb_tune.cu": [],
    "fb_noalloc.cu": [],
    "fb_render.cu": ["--fmad=false"],
}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(ROOT, "include", "fuzzyblue.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit, flags, force):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD_DIR, unit.replace(".cu", ".o"))
    if not force and not _stale(obj, [src] + _headers()):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (unit, r.stdout, r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj


def build(force=False, verbose=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    units = {u: f for u, f in UNITS.items() if os.path.exists(os.path.join(CSRC, u))}
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], force), units.items()))
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
