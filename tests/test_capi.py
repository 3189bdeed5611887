"""CPU tests of the product library's host side: every function declared in
include/mprgp_gpu.h is exported by libmprgp_gb300.so, the beam generator
builds the documented systems, and calls fail loudly without a GPU.  No GPU
compute is issued here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import helpers as H
import mprgp_gb300 as M

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "mprgp_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mprgp_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib_built):
    lib = C.CDLL(lib_built)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_and_defaults(lib_built):
    L = M.lib()
    assert L.mprgp_status_string(M.NOT_CONVERGED) == b"not converged"
    o = M.default_options()
    assert o.tol == 1e-3 and o.max_it == 1000  # MPRGPSolver.h:546 defaults
    assert o.kind == M.KIND_DECOUPLED


@pytest.mark.parametrize("dims,nv,nnzb", [((4, 4, 16), 425, 4921),
                                          ((32, 32, 128), 140481, 2031169)])
def test_beam_sizes(lib_built, dims, nv, nnzb):
    p = M.BeamParams()
    M.lib().mprgp_beam_default(C.byref(p))
    p.a, p.b, p.c = dims
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    assert M.lib().mprgp_beam_sizes(C.byref(p), C.byref(a), C.byref(b), C.byref(c)) == 0
    assert (a.value, b.value) == (nv, nnzb)


def test_beam_system_properties(lib_built):
    qp = M.beam(3, 2, 4, seed=3)
    A, b, J, c = H.qp_from_beam(qp)
    Ad = A.dense()
    assert np.allclose(Ad, Ad.T, rtol=0, atol=1e-12)
    assert np.linalg.eigvalsh(Ad).min() > 0
    # rigid translations are in K's null space: A t = M t with M lumped
    t = np.tile([1.0, 0.0, 0.0], qp.nv)
    m = Ad[np.arange(0, qp.n, 3), np.arange(0, qp.n, 3)] - 0.0
    At = Ad @ t
    assert np.allclose(At[1::3], 0, atol=1e-10) and np.allclose(At[2::3], 0, atol=1e-10)
    total_mass = At[0::3].sum()
    assert abs(total_mass - 1000.0 * (3 * 2 * 4) * 0.05 ** 3) < 1e-9
    # one floor plane per vertex, y >= 0 (n.x + p >= 0 with p = 0)
    assert len(qp.planes) == qp.nv and np.all(qp.planes[:, 1] == 1.0)
    # x0: rest shape shifted to y = -lift
    assert qp.x0[1::3].min() == pytest.approx(-0.01)


def test_corner_planes(lib_built):
    qp = M.beam(4, 4, 8, extra_planes_max=2, extra_planes_min=2, plane_mode=2)
    k = np.diff(qp.plane_ptr)
    assert k.max() == 3 and k.min() == 1
    walls = qp.planes[(qp.planes[:, 0] == 1.0) | (qp.planes[:, 2] == 1.0)]
    assert len(walls) > 0 and np.allclose(walls[:, 1], 0.0)


def test_conversions_roundtrip(lib_built):
    qp = M.beam(2, 3, 2, extra_planes_max=2, extra_planes_min=2, plane_mode=0, seed=4)
    A, b, J, c = H.qp_from_beam(qp)
    x = np.random.default_rng(0).standard_normal(qp.n)
    # BSR product by hand
    y = np.zeros(qp.n)
    for r in range(qp.nv):
        for q in range(qp.row_ptr[r], qp.row_ptr[r + 1]):
            blk = qp.vals[q].reshape(3, 3)
            y[3 * r:3 * r + 3] += blk @ x[3 * qp.cols[q]:3 * qp.cols[q] + 3]
    assert np.allclose(A.matvec(x), y, rtol=1e-14, atol=1e-14)
    assert np.allclose(J.matvec(x) - c, [pl[:3] @ x[3 * v:3 * v + 3] + pl[3]
                                        for v in range(qp.nv)
                                        for pl in qp.planes[qp.plane_ptr[v]:qp.plane_ptr[v + 1]]])


def test_context_without_gpu_fails_loudly(lib_built):
    n = C.c_int(-1)
    M.lib().mprgp_device_count(C.byref(n))
    if n.value > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(M.MPRGPError) as ei:
        M.Context(0)
    assert ei.value.code == M.NO_DEVICE


def test_beam_mesh_and_numpy_fem_assembly():
    """The exported mesh reproduces the generator's system: a numpy assembly
    of A = M + h^2 K (linear material as FEMEnergy.cpp:657, Lame parameters
    as FEMEnergy.cpp:383-384, lumped mass rho V / 4 as FEMMesh.cpp:501-511)
    and b = M (x0 + h v0) + h^2 M g + h^2 K X from tets and X equals
    mprgp_beam_build's."""
    kw = dict(extra_planes_max=1, extra_planes_min=1, plane_mode=2, seed=17)
    qp = M.beam(2, 3, 4, **kw)
    tets, X, x0, v0 = M.beam_mesh(2, 3, 4, **kw)
    p = qp.params
    nv = qp.nv
    assert tets.shape == (6 * 2 * 3 * 4, 4) and tets.min() >= 0 and tets.max() < nv
    assert np.array_equal(x0, qp.x0)
    E, nu, rho, h = p["young"], p["poisson"], p["rho"], p["dt"]
    lam, mu = nu * E / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    K = np.zeros((3 * nv, 3 * nv))
    mass = np.zeros(nv)
    Xv = X.reshape(-1, 3)
    for t in tets:
        Dm = (Xv[t[1:]] - Xv[t[0]]).T
        V = abs(np.linalg.det(Dm)) / 6.0
        assert V > 0
        inv = np.linalg.inv(Dm)
        gN = np.vstack([-inv.sum(axis=0), inv])
        for a in range(4):
            mass[t[a]] += rho * V / 4
            for b_ in range(4):
                Kab = V * (lam * np.outer(gN[a], gN[b_]) + mu * np.outer(gN[b_], gN[a]) +
                           mu * gN[a].dot(gN[b_]) * np.eye(3))
                K[3 * t[a]:3 * t[a] + 3, 3 * t[b_]:3 * t[b_] + 3] += Kab
    A = np.diag(np.repeat(mass, 3)) + h * h * K
    g = np.tile([0.0, p["gravity"], 0.0], nv)
    m3 = np.repeat(mass, 3)
    b = m3 * (x0 + h * v0) + h * h * m3 * g + h * h * K.dot(X)
    ptr, idx, val = M.bsr_to_csr(nv, qp.row_ptr, qp.cols, qp.vals)
    Ad = np.zeros_like(A)
    for r in range(3 * nv):
        Ad[r, idx[ptr[r]:ptr[r + 1]]] = val[ptr[r]:ptr[r + 1]]
    assert np.abs(Ad - A).max() <= 1e-12 * np.abs(A).max()
    assert np.linalg.norm(b - qp.b) <= 1e-12 * np.linalg.norm(b)
