"""The optional Eigen adapter (include/mprgp/EigenAdapter.h): Eigen is not
installed here, so the adapter is compiled against a stand-in for the Eigen
names it uses (tests/cpp/fake_eigen) and checked entry for entry (CPU)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_eigen_adapter(tmp_path):
    exe = tmp_path / "test_eigen_adapter"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(HERE, "cpp", "fake_eigen"),
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "cpp", "test_eigen_adapter.cpp"), "-o", str(exe)],
                   check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0 and res.stdout.strip().endswith("ok"), res.stdout + res.stderr
