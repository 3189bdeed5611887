"""The C++ façade (include/mprgp/) as a reference user would use it: compiles
tests/cpp/test_facade.cpp -- the reference's MPRGPTest.cpp cases written
against the façade -- links libmprgp_gb300.so and runs it on the GPU.  It
also solves the reference-layout QP file fixtures (tests/golden/qp_files)
through the file form (MPRGPSolver.h:576-589) and the text form's global
planes; those solutions are checked against the oracle on the same QPs:
||x - x_oracle|| / ||x_oracle|| <= 1e-8 at 1e-10 ||b|| and the same active set."""
import os
import subprocess
import sys

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
QPDIR = os.path.join(ROOT, "tests", "golden", "qp_files")
sys.path.insert(0, QPDIR)
import make_qp_files as Q  # noqa: E402


def _csr(tri):
    n, m, r, c, v = tri
    order = np.lexsort((c, r))
    r, c, v = np.asarray(r)[order], np.asarray(c)[order], np.asarray(v)[order]
    ptr = np.zeros(n + 1, np.int64)
    np.add.at(ptr, r + 1, 1)
    return H.Csr(np.cumsum(ptr), c, v, n, m)


def _check_against_oracle(kind, A, b, J, c, x0, x_gpu):
    tol = 1e-10 * np.linalg.norm(b)
    xo, _, so, _ = H.oracle_solve(kind, A, b, x0, J, c, tol=tol, max_it=10000)
    assert so["code"] == 0
    assert np.linalg.norm(x_gpu - xo) <= 1e-8 * np.linalg.norm(xo)
    assert np.array_equal(H.decide_face_planes(J, c, x_gpu), H.decide_face_planes(J, c, xo))


def test_cpp_facade(lib_built, tmp_path):
    exe = tmp_path / "test_facade"
    libdir = os.path.dirname(lib_built)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_facade.cpp"), "-L", libdir,
                    "-lmprgp_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    res = subprocess.run([str(exe), QPDIR], cwd=tmp_path, capture_output=True, text=True,
                         timeout=300)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "OK (0 failures)" in res.stdout
    # the file-form solutions against the oracle on the same QPs
    A, B, J, c, x0 = Q.read_jc(os.path.join(QPDIR, "beam_1x2x2.jc.b"))
    _check_against_oracle("decoupled", _csr(A), B, _csr(J), c, x0,
                          np.loadtxt(tmp_path / "x_jc.txt"))
    At, Bt, P, xt = Q.read_text(os.path.join(QPDIR, "beam_1x2x2.txt"))
    n = At[0]
    rows = np.arange(len(P) * (n // 3))
    vert = np.repeat(np.arange(n // 3), len(P))
    jr = np.repeat(rows, 3)
    jc = (3 * vert[:, None] + np.arange(3)[None, :]).reshape(-1)
    jv = np.tile(P[:, :3], (n // 3, 1)).reshape(-1)
    Jt = _csr((len(rows), n, jr, jc, jv))
    ct = np.tile(-P[:, 3], n // 3)
    _check_against_oracle("general", _csr(At), Bt, Jt, ct, xt, np.loadtxt(tmp_path / "x_text.txt"))
