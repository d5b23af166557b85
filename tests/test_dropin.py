"""The igl:: drop-in headers (include/igl_gb300/igl/) compile against the C
ABI, and -- on a GPU -- reproduce the reference's own Catch2 tests
(one_point_cloud at 1e-15, the single-tet sign) through libgwn.so."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "dropin", "dropin_test.cpp")
OUT_DIR = os.path.join(ROOT, "tests", "dropin", "_build")


def compile_dropin(gwn_lib):
    from libigl_gb300 import _native
    os.makedirs(OUT_DIR, exist_ok=True)
    exe = os.path.join(OUT_DIR, "dropin_test")
    libdir = os.path.dirname(_native.LIB_PATH)
    cmd = ["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "tests", "dropin", "eigen_shim"),
           "-I", os.path.join(ROOT, "include", "igl_gb300"), SRC, "-o", exe, "-L", libdir,
           "-lgwn", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True)
    return exe


def test_dropin_headers_compile(gwn_lib):
    assert os.path.exists(compile_dropin(gwn_lib))


def test_dropin_dimension_templates_compile():
    """igl::signed_distance instantiates with fixed-column matrix types (the
    reference's dimension-templates case, 3-D half), and the winding-number
    overloads with float and fixed-column types (compiled, not run)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    obj = os.path.join(OUT_DIR, "dimension_templates.o")
    subprocess.run(["g++", "-c", "-O0", "-std=c++17", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "tests", "dropin", "eigen_shim"),
                    "-I", os.path.join(ROOT, "include", "igl_gb300"),
                    os.path.join(ROOT, "tests", "dropin", "dimension_templates.cpp"),
                    "-o", obj], check=True)
    assert os.path.exists(obj)


@pytest.mark.gpu
def test_dropin_reference_tests_on_gpu(gwn_lib, cuda):
    exe = compile_dropin(gwn_lib)
    r = subprocess.run([exe], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "failures 0" in r.stdout
