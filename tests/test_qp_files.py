"""The reference's QP file forms (src/MPRGPSolver/MPRGPUtility.h:157-485) on
fixtures laid out byte for byte from the reference's writers by
tests/golden/qp_files/make_qp_files.py:
  * the fixtures are what the layout rules give for the seeded beam;
  * the C++ façade loads each form and writes it back byte for byte (host
    code only; no GPU);
  * the loaded QP is the beam's QP (exactly in binary, to 12 digits in text).
"""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

import helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
QPDIR = os.path.join(ROOT, "tests", "golden", "qp_files")
sys.path.insert(0, QPDIR)
import make_qp_files as Q  # noqa: E402


@pytest.mark.parametrize("name", sorted(Q.FILES))
def test_fixture_is_the_reference_layout(name):
    qp = Q.beam()
    with open(os.path.join(QPDIR, name), "rb") as f:
        assert f.read() == Q.FILES[name](qp)


def test_fixture_holds_the_beam_qp():
    qp = Q.beam()
    A, B, J, c, x0 = Q.read_jc(os.path.join(QPDIR, "beam_1x2x2.jc.b"))
    Ac, _, _, _ = H.qp_from_beam(qp)
    dense = np.zeros((qp.n, qp.n))
    dense[A[2], A[3]] = A[4]
    assert np.array_equal(dense, Ac.dense())
    assert np.array_equal(B, qp.b) and np.array_equal(x0, qp.x0)
    assert J[0] == qp.nv and np.array_equal(c, np.zeros(qp.nv))
    # the bench's writer of the same layout gives the same bytes
    sys.path.insert(0, ROOT)
    import bench
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "qp.b")
        bench.write_qp_file(qp, path)
        with open(path, "rb") as f1, open(os.path.join(QPDIR, "beam_1x2x2.jc.b"), "rb") as f2:
            assert f1.read() == f2.read()
    At, Bt, P, xt = Q.read_text(os.path.join(QPDIR, "beam_1x2x2.txt"))
    dense_t = np.zeros((qp.n, qp.n))
    dense_t[At[2], At[3]] = At[4]
    assert np.allclose(dense_t, dense, rtol=1e-11, atol=0)
    assert np.allclose(Bt, qp.b, rtol=1e-11, atol=0) and P.shape == (2, 4)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_facade_reads_and_writes_each_form(tmp_path):
    exe = tmp_path / "test_qp_files"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_qp_files.cpp"), "-o", str(exe)],
                   check=True)
    res = subprocess.run([str(exe), QPDIR, str(tmp_path)], capture_output=True, text=True,
                         timeout=120)
    print(res.stdout)
    assert res.returncode == 0 and "OK (0 failures)" in res.stdout, res.stdout + res.stderr
