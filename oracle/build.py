"""Build recipe for the CPU oracle (test infrastructure only).

  oracle/_build/libfb_oracle.so  the C++ restatement (fb_oracle.cpp), FP32 and FP64
  oracle/_ref/libfbref.so        the reference's own shaders compiled as C++
                                 (ref_glsl/translate.py + glsl_shim.hpp + ref_runner.cpp)

The reference build reads the shader sources from the reference checkout when
it is present and writes the rewritten sources to oracle/_ref/gen/; where the
checkout is absent but the rewritten sources are, it compiles those. Both
outputs are git-ignored. The checkout is FB_REFERENCE_DIR if set, else the
path in oracle/reference_dir.txt, relative to the repository root (a sibling
checkout named `reference`).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libfb_oracle.so")
REF_SO = os.path.join(REF_DIR, "libfbref.so")

COMMON = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle(force=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, "fb_oracle.cpp"), os.path.join(HERE, "fb_oracle.h"),
            os.path.join(ROOT, "include", "fuzzyblue.h")]
    if force or _stale(ORACLE_SO, srcs):
        tmp = ORACLE_SO + ".tmp%d" % os.getpid()
        _run(["g++"] + COMMON + ["-I", os.path.join(ROOT, "include"), srcs[0], "-o", tmp])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_dir():
    """The reference checkout, or None when none is configured."""
    env = os.environ.get("FB_REFERENCE_DIR")
    if env:
        return env
    cfg = os.path.join(HERE, "reference_dir.txt")
    if os.path.exists(cfg):
        with open(cfg) as f:
            rel = f.read().strip()
        if rel:
            return os.path.normpath(os.path.join(ROOT, rel))
    return None


def build_reference(force=False):
    """Returns the path of libfbref.so, or None when neither the reference
    checkout nor previously rewritten sources are available."""
    gen = os.path.join(REF_DIR, "gen")
    ref = reference_dir()
    shaders = os.path.join(ref, "shaders") if ref else None
    sys.path.insert(0, os.path.join(HERE, "ref_glsl"))
    try:
        import translate  # noqa: E402
    finally:
        sys.path.pop(0)
    if shaders and os.path.isdir(shaders):
        translate.main(["--shaders", shaders, "--out", gen])
    if not all(os.path.exists(os.path.join(gen, n)) for n in translate.HEADERS + translate.PASSES + translate.RENDER):
        return None
    runner = os.path.join(HERE, "ref_glsl", "ref_runner.cpp")
    deps = [runner, os.path.join(HERE, "ref_glsl", "glsl_shim.hpp")] + [
        os.path.join(gen, n) for n in translate.HEADERS + translate.PASSES + translate.RENDER]
    if force or _stale(REF_SO, deps):
        tmp = REF_SO + ".tmp%d" % os.getpid()
        _run(["g++"] + COMMON + ["-fsingle-precision-constant", "-w",
                                 "-I", os.path.join(HERE, "ref_glsl"), "-I", gen,
                                 "-I", os.path.join(ROOT, "include"), runner, "-o", tmp])
        os.replace(tmp, REF_SO)
    return REF_SO


def build(force=False):
    o = build_oracle(force)
    r = build_reference(force)
    return o, r


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
