"""Writes the QP file fixtures in this directory, laid out byte for byte as
the reference's writers lay them out (src/MPRGPSolver/MPRGPUtility.h):

  beam_1x2x2.jc.b       binary (A, B, J, c, x0)           writeQP :407-443
  beam_1x2x2.planes.b   binary per-vertex planes          writeQP :258-292
  beam_1x2x2.txt        text, global planes               writeQP :208-257

Binary sparse matrix (writeSparseMatrix :157-175): size_t rows, cols, nnz,
then nnz Eigen::Triplet<double> records {int row, int col, double value}
(16 bytes) in Eigen's column-major order (column by column, rows
ascending); vectors are raw doubles; the per-vertex plane list is, for each
vertex, a size_t count then count x 4 doubles (n, p).  The text form writes
its numbers with 12 significant digits (setprecision(12), C's %.12g).

The QP is a seeded 1x2x2-cube beam from the oracle's generator: the floor
y >= 0 on every vertex (decoupled, for the (J, c) file the decoupled
file-form solve reads) and, in the text file, the floor and the wall
x >= 0.01 as global planes for every vertex.  Little-endian, 64-bit size_t
(x86_64 and aarch64 alike).

Run from the repository root:  python tests/golden/qp_files/make_qp_files.py
"""
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(TESTS))
sys.path.insert(0, TESTS)

DIMS = (1, 2, 2)
SEED = 21
WALL = (1.0, 0.0, 0.0, -0.01)  # n.x + p >= 0: x >= 0.01


def beam():
    import helpers as H
    return H.oracle_beam(*DIMS, seed=SEED)


def scalar_A(qp):
    """A as scalar triplets (row, col, value) in column-major order."""
    import mprgp_gb300 as M
    ptr, idx, val = M.bsr_to_csr(qp.nv, qp.row_ptr, qp.cols, qp.vals)
    rows = np.repeat(np.arange(qp.n), np.diff(ptr))
    order = np.lexsort((rows, idx))  # by column, then row
    return rows[order], np.asarray(idx)[order], np.asarray(val)[order]


def floor_J(qp):
    """The floor row of every vertex: J = e_y at its 3 columns and c = -p =
    -0.0, as the reference's convert (MPRGPUtility.h:120-154) and its
    collider (LinearConCollider.cpp:71) negate the plane offset p = 0."""
    rows = np.repeat(np.arange(qp.nv), 3)
    cols = (3 * np.arange(qp.nv)[:, None] + np.arange(3)[None, :]).reshape(-1)
    vals = np.tile([0.0, 1.0, 0.0], qp.nv)
    order = np.lexsort((rows, cols))
    return rows[order], cols[order], vals[order], -np.zeros(qp.nv)


def sparse_bytes(nrows, ncols, r, c, v):
    out = struct.pack("<QQQ", nrows, ncols, len(v))
    for a, b, x in zip(r, c, v):
        out += struct.pack("<iid", int(a), int(b), float(x))
    return out


def vec_bytes(v):
    return struct.pack(f"<{len(v)}d", *[float(t) for t in v])


def jc_file(qp):
    r, c, v = scalar_A(qp)
    jr, jc, jv, cc = floor_J(qp)
    return (sparse_bytes(qp.n, qp.n, r, c, v) + vec_bytes(qp.b) +
            sparse_bytes(qp.nv, qp.n, jr, jc, jv) + vec_bytes(cc) + vec_bytes(qp.x0))


def planes_file(qp):
    r, c, v = scalar_A(qp)
    out = sparse_bytes(qp.n, qp.n, r, c, v) + vec_bytes(qp.b)
    for vert in range(qp.nv):
        pl = qp.planes[qp.plane_ptr[vert]:qp.plane_ptr[vert + 1]]
        out += struct.pack("<Q", len(pl))
        for p in pl:
            out += vec_bytes(p)
    return out + vec_bytes(qp.x0)


def g12(x):
    return "%.12g" % x


def text_file(qp):
    r, c, v = scalar_A(qp)
    planes = [(0.0, 1.0, 0.0, 0.0), WALL]
    lines = [f"dimension {qp.n}", f"planes {len(planes)}", "A", f"non_zeros {len(v)}"]
    lines += [f"{a}\t{b}\t{g12(x)}" for a, b, x in zip(r, c, v)]
    lines += ["B", "\t".join(g12(x) for x in qp.b), "P"]
    lines += ["\t".join(g12(x) for x in p) for p in planes]
    lines += ["x0", "\t".join(g12(x) for x in qp.x0)]
    return ("\n".join(lines) + "\n").encode()


FILES = {"beam_1x2x2.jc.b": jc_file, "beam_1x2x2.planes.b": planes_file,
         "beam_1x2x2.txt": text_file}


# ---- readers (the reference's loadQP, for the tests) ----------------------
def _sparse(buf, off):
    nr, nc, nz = struct.unpack_from("<QQQ", buf, off)
    off += 24
    rec = np.frombuffer(buf, dtype=np.dtype([("r", "<i4"), ("c", "<i4"), ("v", "<f8")]),
                        count=nz, offset=off)
    return (nr, nc, rec["r"].copy(), rec["c"].copy(), rec["v"].copy()), off + 16 * nz


def _vec(buf, off, n):
    return np.frombuffer(buf, "<f8", count=n, offset=off).copy(), off + 8 * n


def read_jc(path):
    """(A, B, J, c, x0) with A and J as (rows, cols, r, c, v) triplets."""
    buf = open(path, "rb").read()
    A, off = _sparse(buf, 0)
    B, off = _vec(buf, off, A[0])
    J, off = _sparse(buf, off)
    c, off = _vec(buf, off, J[0])
    x0, off = _vec(buf, off, A[0])
    assert off == len(buf)
    return A, B, J, c, x0


def read_text(path):
    """(A triplets, B, global planes (m, 4), x0) of the text form."""
    tok = open(path).read().split()
    n, m, nnz = int(tok[1]), int(tok[3]), int(tok[6])  # dimension n planes m A non_zeros nnz
    k = 7
    tri = np.array(tok[k:k + 3 * nnz], dtype=object).reshape(nnz, 3)
    k += 3 * nnz
    A = (n, n, tri[:, 0].astype(int), tri[:, 1].astype(int), tri[:, 2].astype(float))
    B = np.array(tok[k + 1:k + 1 + n], float)
    k += 1 + n
    P = np.array(tok[k + 1:k + 1 + 4 * m], float).reshape(m, 4)
    k += 1 + 4 * m
    x0 = np.array(tok[k + 1:k + 1 + n], float)
    assert k + 1 + n == len(tok)
    return A, B, P, x0


def main():
    qp = beam()
    for name, make in FILES.items():
        with open(os.path.join(HERE, name), "wb") as f:
            f.write(make(qp))
        print("wrote", name)


if __name__ == "__main__":
    main()
