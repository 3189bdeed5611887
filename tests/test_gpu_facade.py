"""The C++ façade (include/mprgp/) as a reference user would use it: compiles
tests/cpp/test_facade.cpp -- the reference's MPRGPTest.cpp cases written
against the façade -- links libmprgp_gb300.so and runs it on the GPU."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_facade(lib_built, tmp_path):
    exe = tmp_path / "test_facade"
    libdir = os.path.dirname(lib_built)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_facade.cpp"), "-L", libdir,
                    "-lmprgp_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    res = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "OK (0 failures)" in res.stdout
