"""The bounds-checked debug build (-DMPRGP_CHECKS).

In that build the kernels check every index they read from device arrays --
block columns, the SELL row order, plane offsets -- and report a bad one as
MPRGP_INVALID instead of reading out of bounds.

* CPU: the CUDA sources compile with the checks.
* GPU: the debug library, loaded through MPRGP_LIBRARY in a child process,
  solves the parity QPs -- single solves in both precisions and a served mix
  of cluster-solver and engine instances -- with every result code 0 and the
  same x as the release build (bitwise for the single solves, to 1e-12 for
  the served ones): on valid input no check fires and the checks change no
  arithmetic.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import mprgp_gb300 as M
from mprgp_gb300 import buildlib

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("src", ["engine.cu", "capi.cu", "noalloc.cu"])
def test_sources_compile_with_checks(tmp_path, src):
    cmd = [buildlib.nvcc(), "-c", os.path.join(buildlib.CSRC, src), "-o", str(tmp_path / "x.o"),
           "-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-I",
           os.path.join(buildlib.ROOT, "include"), "-DMPRGP_CHECKS"] + buildlib.ARCH
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


# Solves the cases and prints, per case, the result codes and x's bytes.
CHILD = r"""
import json, sys
import numpy as np
import mprgp_gb300 as M
SEED = 0x5EED
def opts(qp, prec):
    return M.default_options(tol=1e-8 * np.linalg.norm(qp.b), max_it=20000, kind=M.KIND_PLANES,
                             project_x0=1, seed=SEED, precision=prec)
ctx = M.Context(0)
out = {}
singles = [(4, 4, 16, 0), (6, 5, 18, 2), (16, 8, 32, 1)]
for a, b, c, e in singles:
    qp = M.beam(a, b, c, extra_planes_max=e, extra_planes_min=e, plane_mode=2, seed=a + c)
    for prec in (M.PREC_FP64, M.PREC_MIXED):
        x, face, st = ctx.solve_bsr(qp, opts(qp, prec), qp.x0)
        out[f"single-{a}x{b}x{c}-{prec}"] = [int(st.code), x.tobytes().hex()]
dims = [(4, 4, 6), (9, 5, 12), (3, 3, 4), (14, 8, 30), (16, 8, 32)]
qps = [M.beam(*d, extra_planes_max=i % 3, extra_planes_min=i % 3, plane_mode=2, seed=20 + i)
       for i, d in enumerate(dims)]
srv = M.Server(ctx, quantum_phases=64, power_launches=128, max_slots=8, lanes=3)
tickets = {srv.submit(i, q, opts(q, M.PREC_MIXED)): i for i, q in enumerate(qps)}
steps = 0
while tickets:
    srv.step()
    steps += 1
    for t, i in list(tickets.items()):
        state, x, face, st, _ = srv.result(t)
        if state == 2:
            out[f"served-{i}"] = [int(st.code), x.tobytes().hex()]
            del tickets[t]
    assert steps < 200000
srv.close()
print(json.dumps(out))
"""


def _run_child(library):
    env = dict(os.environ)
    if library:
        env["MPRGP_LIBRARY"] = library
    else:
        env.pop("MPRGP_LIBRARY", None)
    r = subprocess.run([sys.executable, "-c", CHILD], capture_output=True, text=True, env=env,
                       cwd=os.path.dirname(HERE), timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.gpu
def test_checked_build_same_bits_as_release():
    checked = buildlib.build(checks=True)
    release = _run_child(None)
    debug = _run_child(checked)
    assert sorted(release) == sorted(debug)
    for k in release:
        assert release[k][0] == 0 and debug[k][0] == 0, (k, release[k][0], debug[k][0])
        if k.startswith("single"):
            assert release[k][1] == debug[k][1], k
        else:  # served: each instance reduces in a fixed order whatever its batch
            xr = np.frombuffer(bytes.fromhex(release[k][1]))
            xd = np.frombuffer(bytes.fromhex(debug[k][1]))
            assert np.linalg.norm(xd - xr) <= 1e-12 * np.linalg.norm(xr), k
    assert len(release) == 11
