// oracle/oracle_capi.cpp -- extern "C" entry points over mprgp_oracle.h.
//
// TEST INFRASTRUCTURE ONLY (see mprgp_oracle.h).  Loaded by tests/ and by
// bench.py's CPU-baseline leg through ctypes; never by the product.
//
// Matrices arrive as CSR (row pointer, column index, value), the natural
// unblocked form of the reference's Eigen::SparseMatrix<double> arguments
// (MPRGPSolver.h:544-625).  Constraints arrive as the reference's (J, c)
// pair, J in CSR, meaning J x >= c.
#include <cstdint>
#include <cstring>

#include "beam_oracle.h"
#include "ica_oracle.h"
#include "mprgp_oracle.h"

using namespace oracle;

namespace {

Csr make_csr(int rows, int cols, const int *ptr, const int *idx, const double *val) {
  Csr M;
  M.rows = rows;
  M.cols = cols;
  M.ptr.assign(ptr, ptr + rows + 1);
  const int nnz = ptr[rows];
  M.idx.assign(idx, idx + nnz);
  M.val.assign(val, val + nnz);
  return M;
}

void write_stats(const SolveStats &s, double *out) {
  if (!out) return;
  out[0] = s.code;
  out[1] = s.iterations;
  out[2] = s.num_cg;
  out[3] = s.num_exp;
  out[4] = s.num_prop;
  out[5] = s.power_iters;
  out[6] = s.residual;
  out[7] = s.alpha_bar;
  out[8] = s.spec_rad;
  out[9] = s.spmv;
}

void copy_face(const std::vector<char> &f, unsigned char *out) {
  if (!out) return;
  for (size_t i = 0; i < f.size(); ++i) out[i] = (unsigned char)f[i];
}

Trace *g_trace = nullptr;  // set by oracle_set_trace (test diagnostics)
bool g_scalar_test = false;  // set by oracle_set_scalar_test

template <typename SOLVER>
int run(SOLVER &solver, Vec &x, double *stats) {
  solver.trace = g_trace;
  solver.scalar_test = g_scalar_test;
  const int code = solver.solve(x);
  write_stats(solver.stats(), stats);
  return code;
}

}  // namespace

extern "C" {

// Projector kinds, matching the reference solve façades:
//   0 MPRGPLowerBound   (MPRGPSolver.h:503-517)  monotone + DiagonalInFace
//   1 MPRGPBoxBound     (MPRGPSolver.h:520-535)  plain MPRGP + DiagonalInFace
//   2 MPRGPDecoupledCon (MPRGPSolver.h:538-590)  monotone + DiagonalDecouple
//   3 MPRGPGeneralCon   (MPRGPSolver.h:593-626)  monotone + DiagonalInFace
// `preconditioned` is the template flag of the Decoupled/General façades.
// `project_x0` = 1 reproduces the solve(A,B,J,c,x) overloads, which project
// x onto the feasible set before solving (MPRGPSolver.h:570-572, 621-623).
// kind + 10 runs the plain MPRGP::solve (MPRGPSolver.h:356-396) with that
// kind's projector and preconditioner instead of MPRGPMonotonic.
// stats (10 doubles): code, iterations, cg, exp, prop, power iters, residual,
// alpha_bar, spectral radius, SpMV count.
static int solve_impl(int kind, int preconditioned, int n, const int *a_ptr, const int *a_idx,
                      const double *a_val, const double *b, int m, const int *j_ptr,
                      const int *j_idx, const double *j_val, const double *c, const double *L,
                      const double *U, double tol, int max_it, uint64_t seed, Vec *evp,
                      int project_x0, double *x, unsigned char *face_out, double *stats) {
  const Csr Am = make_csr(n, n, a_ptr, a_idx, a_val);
  const FixedSparseMatrix FA(Am);
  const Vec B(b, b + n);
  Vec X(x, x + n);
  int code = -100;
  const bool plain = kind >= 10;  // kind + 10: plain MPRGP::solve with that projector
  if (plain) kind -= 10;
  if (plain && kind >= 2) {
    const Csr J = make_csr(m, n, j_ptr, j_idx, j_val);
    const Vec cv(c, c + m);
    if (kind == 2) {
      const Vec JJt = J.rowNorm2();
      DecoupledConProjector proj(J, JJt, cv);
      if (project_x0) { const Vec x0 = X; proj.project(x0, X); }
      DiagonalDecouplePreconSolver<FixedSparseMatrix, false> pre(FA, proj.getFace(), J);
      MPRGP<FixedSparseMatrix, DecoupledConProjector, decltype(pre)> s(FA, B, pre, proj, max_it,
                                                                       tol, evp, seed);
      code = run(s, X, stats);
      copy_face(proj.getFace(), face_out);
    } else {
      GeneralConProjector proj(J, cv);
      if (project_x0) { const Vec x0 = X; proj.project(x0, X); }
      DiagonalInFacePreconSolver<FixedSparseMatrix, false> pre(FA, proj.getFace());
      MPRGP<FixedSparseMatrix, GeneralConProjector, decltype(pre)> s(FA, B, pre, proj, max_it,
                                                                     tol, evp, seed);
      code = run(s, X, stats);
      copy_face(proj.getFace(), face_out);
    }
  } else if (plain && kind == 0) {
    const Vec Lv(L, L + n);
    LowerBoundProjector proj(Lv);
    DiagonalInFacePreconSolver<FixedSparseMatrix> pre(FA, proj.getFace());
    MPRGP<FixedSparseMatrix, LowerBoundProjector, DiagonalInFacePreconSolver<FixedSparseMatrix>>
        s(FA, B, pre, proj, max_it, tol, evp, seed);
    code = run(s, X, stats);
    copy_face(proj.getFace(), face_out);
  } else if (kind == 0 || kind == 1) {
    const Vec Lv(L, L + n);
    const Vec Uv = U ? Vec(U, U + n) : Vec(n, DBL_MAX);
    if (kind == 0) {
      LowerBoundProjector proj(Lv);
      DiagonalInFacePreconSolver<FixedSparseMatrix> pre(FA, proj.getFace());
      MPRGPMonotonic<FixedSparseMatrix, LowerBoundProjector,
                     DiagonalInFacePreconSolver<FixedSparseMatrix>>
          s(FA, B, pre, proj, max_it, tol, evp, seed);
      code = run(s, X, stats);
      copy_face(proj.getFace(), face_out);
    } else {
      BoxBoundProjector proj(Lv, Uv);
      DiagonalInFacePreconSolver<FixedSparseMatrix> pre(FA, proj.getFace());
      MPRGP<FixedSparseMatrix, BoxBoundProjector, DiagonalInFacePreconSolver<FixedSparseMatrix>>
          s(FA, B, pre, proj, max_it, tol, evp, seed);
      code = run(s, X, stats);
      copy_face(proj.getFace(), face_out);
    }
  } else {
    const Csr J = make_csr(m, n, j_ptr, j_idx, j_val);
    const Vec cv(c, c + m);
    if (kind == 2) {
      const Vec JJt = J.rowNorm2();
      DecoupledConProjector proj(J, JJt, cv);
      if (project_x0) {
        const Vec x0 = X;
        proj.project(x0, X);
      }
      if (preconditioned) {
        DiagonalDecouplePreconSolver<FixedSparseMatrix, false> pre(FA, proj.getFace(), J);
        MPRGPMonotonic<FixedSparseMatrix, DecoupledConProjector, decltype(pre)> s(
            FA, B, pre, proj, max_it, tol, evp, seed);
        code = run(s, X, stats);
      } else {
        DiagonalDecouplePreconSolver<FixedSparseMatrix, true> pre(FA, proj.getFace(), J);
        MPRGPMonotonic<FixedSparseMatrix, DecoupledConProjector, decltype(pre)> s(
            FA, B, pre, proj, max_it, tol, evp, seed);
        code = run(s, X, stats);
      }
      copy_face(proj.getFace(), face_out);
    } else if (kind == 3) {
      GeneralConProjector proj(J, cv);
      if (project_x0) {
        const Vec x0 = X;
        proj.project(x0, X);
      }
      if (preconditioned) {
        DiagonalInFacePreconSolver<FixedSparseMatrix, false> pre(FA, proj.getFace());
        MPRGPMonotonic<FixedSparseMatrix, GeneralConProjector, decltype(pre)> s(
            FA, B, pre, proj, max_it, tol, evp, seed);
        code = run(s, X, stats);
      } else {
        DiagonalInFacePreconSolver<FixedSparseMatrix, true> pre(FA, proj.getFace());
        MPRGPMonotonic<FixedSparseMatrix, GeneralConProjector, decltype(pre)> s(
            FA, B, pre, proj, max_it, tol, evp, seed);
        code = run(s, X, stats);
      }
      copy_face(proj.getFace(), face_out);
    }
  }
  std::memcpy(x, X.data(), sizeof(double) * n);
  return code;
}

int oracle_solve(int kind, int preconditioned, int n, const int *a_ptr, const int *a_idx,
                 const double *a_val, const double *b, int m, const int *j_ptr,
                 const int *j_idx, const double *j_val, const double *c, const double *L,
                 const double *U, double tol, int max_it, uint64_t seed, double *ev,
                 int ev_len, int project_x0, double *x, unsigned char *face_out,
                 double *stats) {
  Vec EV;
  Vec *evp = nullptr;
  if (ev) {
    EV.assign(ev, ev + ev_len);
    evp = &EV;
  }
  const int code = solve_impl(kind, preconditioned, n, a_ptr, a_idx, a_val, b, m, j_ptr, j_idx,
                              j_val, c, L, U, tol, max_it, seed, evp, project_x0, x, face_out,
                              stats);
  if (ev && evp) {
    for (int i = 0; i < ev_len && i < (int)EV.size(); ++i) ev[i] = EV[i];
  }
  return code;
}

// The same solve with the power-method warm start of MprgpFemSolver
// (MprgpFemSolver.h:138, .cpp:533 pass &power_ev across frames): ev holds n
// doubles; *ev_valid = 1 on entry starts specRad from ev (else from the
// seeded random vector), and on return *ev_valid = 1 when ev holds a stored
// vector -- the one given, or the iterate specRad stored when it stopped
// early (MPRGPSolver.h:62-74).
int oracle_solve_warm(int kind, int n, const int *a_ptr, const int *a_idx, const double *a_val,
                      const double *b, int m, const int *j_ptr, const int *j_idx,
                      const double *j_val, const double *c, double tol, int max_it,
                      uint64_t seed, double *ev, int *ev_valid, int project_x0, double *x,
                      unsigned char *face_out, double *stats) {
  Vec EV;
  if (*ev_valid) EV.assign(ev, ev + n);
  const int code = solve_impl(kind, 1, n, a_ptr, a_idx, a_val, b, m, j_ptr, j_idx, j_val, c,
                              nullptr, nullptr, tol, max_it, seed, &EV, project_x0, x, face_out,
                              stats);
  *ev_valid = (int)EV.size() == n ? 1 : 0;
  if (*ev_valid) std::memcpy(ev, EV.data(), sizeof(double) * n);
  return code;
}

// Switches the monotone solvers' CG decrease test between the reference's
// comparison of two function values (0, the default) and the scalar form
// the GPU solver evaluates (1).  Applies to the solves that follow.
void oracle_set_scalar_test(int on) { g_scalar_test = on != 0; }

// Projector primitives, one call per operation, for the projector property
// tests (test_case/MPRGPTest.cpp:11-68).  op: 0 project(x)->out,
// 1 DECIDE_FACE(x)->face, 2 PHI(g)->out (face from DECIDE_FACE(x)),
// 3 BETA(g, phi)->out (face from DECIDE_FACE(x)), 4 PHITPHI(x, alpha, phi)->out[0].
// kind: 2 decoupled, 3 general.
int oracle_projector_op(int kind, int op, int n, int m, const int *j_ptr, const int *j_idx,
                        const double *j_val, const double *c, const double *x,
                        const double *g, const double *phi, double alpha, double *out,
                        unsigned char *face_out) {
  const Csr J = make_csr(m, n, j_ptr, j_idx, j_val);
  const Vec cv(c, c + m), X(x, x + n);
  const Vec G = g ? Vec(g, g + n) : Vec(n, 0.0);
  const Vec P = phi ? Vec(phi, phi + n) : Vec(n, 0.0);
  Vec o;
  auto body = [&](auto &proj) {
    switch (op) {
      case 0: proj.project(X, o); break;
      case 1: proj.DECIDE_FACE(X); break;
      case 2: proj.DECIDE_FACE(X); proj.PHI(G, o); break;
      case 3: proj.DECIDE_FACE(X); proj.BETA(G, o, P); break;
      case 4: proj.DECIDE_FACE(X); o.assign(1, proj.PHITPHI(X, alpha, P)); break;
      default: return -5;
    }
    copy_face(proj.getFace(), face_out);
    return 0;
  };
  int rc;
  if (kind == 2) {
    const Vec JJt = J.rowNorm2();
    DecoupledConProjector proj(J, JJt, cv);
    rc = body(proj);
  } else {
    GeneralConProjector proj(J, cv);
    rc = body(proj);
  }
  if (rc == 0 && out)
    for (size_t i = 0; i < o.size(); ++i) out[i] = o[i];
  return rc;
}

// y = A x (FixedSparseMatrix::multiply, MPRGPSolver.h:469-473).
void oracle_spmv(int n, const int *a_ptr, const int *a_idx, const double *a_val,
                 const double *x, double *y) {
  const Csr Am = make_csr(n, n, a_ptr, a_idx, a_val);
  Vec X(x, x + n), Y;
  Am.multiply(X, Y);
  std::memcpy(y, Y.data(), sizeof(double) * n);
}

// specRad (MPRGPSolver.h:42-79) with the seeded start vector.
double oracle_spec_rad(int n, const int *a_ptr, const int *a_idx, const double *a_val,
                       double eps, uint64_t seed, int *iters) {
  const Csr Am = make_csr(n, n, a_ptr, a_idx, a_val);
  const FixedSparseMatrix FA(Am);
  int spmv = 0;
  return MPRGPBase<FixedSparseMatrix, LowerBoundProjector,
                   DiagonalInFacePreconSolver<FixedSparseMatrix>>::specRad(FA, nullptr, eps,
                                                                           seed, iters, &spmv);
}

double oracle_seeded_uniform(uint64_t seed, uint64_t i) { return seeded_uniform(seed, i); }

// Threads of the OpenMP build for SpMV and dot products (1 = serial, as the
// reference).  Returns the count in effect.
int oracle_set_threads(int n) {
#ifdef _OPENMP
  omp_threads() = n > 0 ? n : 1;
#else
  (void)n;
  omp_threads() = 1;
#endif
  return omp_threads();
}

// Enables (cap > 0) or disables the step trace of the next solves.
static Trace g_trace_buf;
void oracle_set_trace(int on) {
  g_trace_buf.clear();
  g_trace = on ? &g_trace_buf : nullptr;
}
int oracle_get_trace(double *out, int cap) {
  const int n = (int)g_trace_buf.size();
  for (int i = 0; i < n && i < cap; ++i)
    for (int k = 0; k < 4; ++k) out[4 * i + k] = g_trace_buf[i][k];
  return n;
}

// ICA (ICASolver.h:287-393) on a BSR matrix and per-vertex planes; see
// ica_oracle.h.  stats (4 doubles): iterations, converged, residual, PGS sweeps.
int oracle_ica_solve(int nv, const int *row_ptr, const int *cols, const double *vals,
                     const double *r, const int *plane_ptr, const double *planes, double *x,
                     double *lambda, int max_it, double tol, int gs_max_it, double gs_tol,
                     double *stats) {
  const IcaStats st = ica_solve(nv, row_ptr, cols, vals, r, plane_ptr, planes, x, lambda, max_it,
                                tol, gs_max_it, gs_tol);
  if (stats) {
    stats[0] = st.iterations;
    stats[1] = st.converged;
    stats[2] = st.residual;
    stats[3] = (double)st.pgs_sweeps;
  }
  return st.converged ? 0 : -1;
}

// The synthetic beam QP (beam_oracle.h).  ip = {a, b, c, planes_max,
// planes_min, mode, facet_layers}; dp = {edge, young, poisson, rho, dt,
// gravity, lift, v0_sigma, active_frac, band, max_tilt}.  Returns a handle
// (NULL for an invalid spec) and the sizes; oracle_beam_take copies the
// arrays out (row_ptr nv+1, cols nnzb, vals 9 nnzb, b and x0 3 nv,
// plane_ptr nv+1, planes 4 m) and frees the handle.
void *oracle_beam_new(const int *ip, const double *dp, uint64_t seed, int *nv, int *nnzb,
                      int *nplanes) {
  BeamSpec s;
  s.a = ip[0]; s.b = ip[1]; s.c = ip[2];
  s.planes_max = ip[3]; s.planes_min = ip[4]; s.mode = ip[5]; s.facet_layers = ip[6];
  s.edge = dp[0]; s.young = dp[1]; s.poisson = dp[2]; s.rho = dp[3]; s.dt = dp[4];
  s.gravity = dp[5]; s.lift = dp[6]; s.v0_sigma = dp[7]; s.active_frac = dp[8];
  s.band = dp[9]; s.max_tilt = dp[10];
  s.seed = seed;
  BeamQPData *q = new BeamQPData;
  if (!build_beam(s, *q)) {
    delete q;
    return nullptr;
  }
  *nv = q->nv;
  *nnzb = (int)q->cols.size();
  *nplanes = (int)(q->planes.size() / 4);
  return q;
}

void oracle_beam_take(void *h, int *row_ptr, int *cols, double *vals, double *b, double *x0,
                      int *plane_ptr, double *planes) {
  BeamQPData *q = static_cast<BeamQPData *>(h);
  std::memcpy(row_ptr, q->row_ptr.data(), sizeof(int) * q->row_ptr.size());
  std::memcpy(cols, q->cols.data(), sizeof(int) * q->cols.size());
  std::memcpy(vals, q->vals.data(), sizeof(double) * q->vals.size());
  std::memcpy(b, q->b.data(), sizeof(double) * q->b.size());
  std::memcpy(x0, q->x0.data(), sizeof(double) * q->x0.size());
  std::memcpy(plane_ptr, q->plane_ptr.data(), sizeof(int) * q->plane_ptr.size());
  std::memcpy(planes, q->planes.data(), sizeof(double) * q->planes.size());
  delete q;
}

}  // extern "C"
