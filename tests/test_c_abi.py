"""The C ABI from a C program (tests/c_abi/build_one.c): include/fuzzyblue.h
compiles as C11 with -pedantic and every call the program makes links against
the library (CPU); on the GPU the program's tables match the Python API's
build of the same atmosphere."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "c_abi", "build_one.c")
LIB_DIR = os.path.join(ROOT, "fuzzyblue_gb300", "lib")


def _compile(out_dir):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    if not os.path.exists(os.path.join(LIB_DIR, "libfuzzyblue_cuda.so")):
        pytest.skip("library not built")
    exe = os.path.join(out_dir, "build_one")
    cmd = [cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", LIB_DIR, "-lfuzzyblue_cuda", "-Wl,-rpath," + LIB_DIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_header_is_c11_and_the_program_links(tmp_path):
    exe = _compile(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_c_program_matches_the_python_api(tmp_path, builder, precision):
    from fuzzyblue_gb300.api import Atmosphere
    from fuzzyblue_gb300.params import Parameters
    exe = _compile(str(tmp_path))
    r = subprocess.run([exe, "3", str(precision)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    sums = [float(x) for x in r.stdout.split("sums")[1].split()]
    pend = Atmosphere.build(builder, Parameters(order=3, precision=precision))
    pend.wait()
    t = pend.atmosphere(0).to_host()
    pend.release()
    ref = [float(np.asarray(t[k][..., :3], np.float64).sum()) for k in ("transmittance", "irradiance", "scattering")]
    # the same build through two front ends gives the same bits; the sums are
    # printed with 10 significant digits and summed in a different order
    for got, want in zip(sums, ref):
        assert got == pytest.approx(want, rel=1e-9, abs=0.0)
