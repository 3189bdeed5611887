// GPU assembly of the implicit-Euler FEM system the MPRGP solve receives.
//
// Restates, for a linear material and lumped mass, what the reference's FEM
// driver builds on the host before every solve (MprgpFemSolver.cpp:315-356
// through FEMSystem::buildSystem, FEMSystem.cpp:167-193):
//   A = M + h^2 K,   b = M (x + h v) + h^2 M g + h^2 K X
// with K the stiffness of MaterialEnergy::evalFLinear (FEMEnergy.cpp:657:
// energy V (mu |eps|^2 + lambda/2 tr(eps)^2), eps = sym(F) - I; Lame
// parameters from E, nu as FEMEnergy.cpp:383-384) and the lumped mass of
// FEMMesh.cpp:501-511 (each vertex of a tet gets rho V / 4).
//
// Layout: the block sparsity pattern (3x3 blocks, one block row per vertex,
// columns sorted) is built once per mesh on the host; per-tet geometry
// (volume and shape-function gradients) lives on the device.  Assembly is a
// gather, one thread per block row over the vertex's incident tets in a
// fixed order: deterministic, no atomics.  The matrix and b go straight
// into an mprgp_problem from device memory.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mprgp_gpu.h"

namespace mprgp {
void set_last_error(const char *what);
}

struct mprgp_fem {
  mprgp_context *ctx = nullptr;
  cudaStream_t stream = nullptr;
  int nv = 0, ntet = 0, nnzb = 0;
  double lam = 0.0, mu = 0.0, rho = 0.0;
  int *tets = nullptr;                   // 4 per tet
  int *row_ptr = nullptr, *cols = nullptr;
  int *vt_ptr = nullptr, *vt = nullptr;  // incident (tet << 2 | local corner) per vertex
  double *geom = nullptr;                // 13 per tet: V, grad N_0..3
  double *X = nullptr;                   // rest shape
  double *mass = nullptr, *KX = nullptr;
  double *vals = nullptr, *b = nullptr;
  double *xin = nullptr, *vin = nullptr;  // staging for host x, v
  int assembled = 0;
};

namespace {

int fail(int code, const char *what) {
  mprgp::set_last_error(what);
  return code;
}
#define FK(call)                                                  \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) return fail(MPRGP_CUDA_ERROR, #call);  \
  } while (0)

// Volume and shape-function gradients of each tet from the rest shape:
// Dm = [X1-X0, X2-X0, X3-X0], grad N_a (a = 1..3) = rows of Dm^-1,
// grad N_0 = -(sum of the others).  A degenerate tet gets V = 0.
__global__ void tet_geom_kernel(int ntet, const int *__restrict__ tets,
                                const double *__restrict__ X, double *geom) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntet) return;
  int v[4];
  for (int a = 0; a < 4; ++a) v[a] = tets[4 * (size_t)t + a];
  double Dm[3][3];
  for (int a = 1; a < 4; ++a)
    for (int d = 0; d < 3; ++d) Dm[d][a - 1] = X[3 * (size_t)v[a] + d] - X[3 * (size_t)v[0] + d];
  const double det = Dm[0][0] * (Dm[1][1] * Dm[2][2] - Dm[1][2] * Dm[2][1]) -
                     Dm[0][1] * (Dm[1][0] * Dm[2][2] - Dm[1][2] * Dm[2][0]) +
                     Dm[0][2] * (Dm[1][0] * Dm[2][1] - Dm[1][1] * Dm[2][0]);
  double *g = geom + 13 * (size_t)t;
  if (det == 0.0) {
    for (int k = 0; k < 13; ++k) g[k] = 0.0;
    return;
  }
  const double id = 1.0 / det;
  double inv[3][3];
  inv[0][0] = (Dm[1][1] * Dm[2][2] - Dm[1][2] * Dm[2][1]) * id;
  inv[0][1] = (Dm[0][2] * Dm[2][1] - Dm[0][1] * Dm[2][2]) * id;
  inv[0][2] = (Dm[0][1] * Dm[1][2] - Dm[0][2] * Dm[1][1]) * id;
  inv[1][0] = (Dm[1][2] * Dm[2][0] - Dm[1][0] * Dm[2][2]) * id;
  inv[1][1] = (Dm[0][0] * Dm[2][2] - Dm[0][2] * Dm[2][0]) * id;
  inv[1][2] = (Dm[0][2] * Dm[1][0] - Dm[0][0] * Dm[1][2]) * id;
  inv[2][0] = (Dm[1][0] * Dm[2][1] - Dm[1][1] * Dm[2][0]) * id;
  inv[2][1] = (Dm[0][1] * Dm[2][0] - Dm[0][0] * Dm[2][1]) * id;
  inv[2][2] = (Dm[0][0] * Dm[1][1] - Dm[0][1] * Dm[1][0]) * id;
  g[0] = fabs(det) / 6.0;
  for (int d = 0; d < 3; ++d) {
    g[1 + 3 * 1 + d] = inv[0][d];
    g[1 + 3 * 2 + d] = inv[1][d];
    g[1 + 3 * 3 + d] = inv[2][d];
    g[1 + 3 * 0 + d] = -(inv[0][d] + inv[1][d] + inv[2][d]);
  }
}

// Position of block (row, col) in the sorted column list of the row.
__device__ __forceinline__ int find_block(const int *__restrict__ cols, int r0, int r1, int col) {
  int lo = r0, hi = r1 - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cols[mid] < col) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// One thread per vertex a: K_ab = V (lam gNa gNb^T + mu gNb gNa^T + mu (gNa . gNb) I)
// summed over the tets around a (in incidence order), scaled by h^2 into the
// block row of A, plus the lumped mass on the diagonal block; K X along the way.
__global__ void assemble_rows_kernel(int nv, const int *__restrict__ tets,
                                     const double *__restrict__ geom,
                                     const int *__restrict__ row_ptr, const int *__restrict__ cols,
                                     const int *__restrict__ vt_ptr, const int *__restrict__ vt,
                                     const double *__restrict__ X, double lam, double mu,
                                     double rho, double h2, double *vals, double *mass,
                                     double *KX) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nv) return;
  const int r0 = row_ptr[a], r1 = row_ptr[a + 1];
  for (int q = r0; q < r1; ++q)
    for (int e = 0; e < 9; ++e) vals[9 * (size_t)q + e] = 0.0;
  double m = 0.0, kx[3] = {0.0, 0.0, 0.0};
  for (int idx = vt_ptr[a]; idx < vt_ptr[a + 1]; ++idx) {
    const int t = vt[idx] >> 2, la = vt[idx] & 3;
    const double *g = geom + 13 * (size_t)t;
    const double V = g[0];
    m += rho * V / 4.0;
    const double gA[3] = {g[1 + 3 * la], g[2 + 3 * la], g[3 + 3 * la]};
    for (int lb = 0; lb < 4; ++lb) {
      const int bv = tets[4 * (size_t)t + lb];
      const double gB[3] = {g[1 + 3 * lb], g[2 + 3 * lb], g[3 + 3 * lb]};
      const double dd = gA[0] * gB[0] + gA[1] * gB[1] + gA[2] * gB[2];
      double *blk = vals + 9 * (size_t)find_block(cols, r0, r1, bv);
      const double xb[3] = {X[3 * (size_t)bv], X[3 * (size_t)bv + 1], X[3 * (size_t)bv + 2]};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const double k = V * (lam * gA[i] * gB[j] + mu * gA[j] * gB[i] + (i == j ? mu * dd : 0.0));
          blk[3 * i + j] += h2 * k;
          kx[i] += k * xb[j];
        }
    }
  }
  double *diag = vals + 9 * (size_t)find_block(cols, r0, r1, a);
  for (int d = 0; d < 3; ++d) diag[4 * d] += m;
  mass[a] = m;
  for (int d = 0; d < 3; ++d) KX[3 * (size_t)a + d] = kx[d];
}

// b = M (x + h v) + h^2 M g + h^2 K X.
__global__ void fem_rhs_kernel(int nv, const double *__restrict__ mass,
                               const double *__restrict__ KX, const double *__restrict__ x,
                               const double *__restrict__ v, double h, double g0, double g1,
                               double g2, double *b) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= 3 * nv) return;
  const int a = q / 3, d = q - 3 * a;
  const double g = d == 0 ? g0 : (d == 1 ? g1 : g2);
  const double h2 = h * h;
  b[q] = mass[a] * (x[q] + h * (v ? v[q] : 0.0)) + h2 * mass[a] * g + h2 * KX[q];
}

template <typename T>
int dmalloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) return MPRGP_OK;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  return e == cudaSuccess ? MPRGP_OK : fail(MPRGP_OOM, "fem: device allocation");
}
template <typename T>
void dfree(T *&p) {
  if (p) cudaFree(p);
  p = nullptr;
}

// x and v as device pointers (copied into staging when they are host memory).
int stage_xv(mprgp_fem *f, const double *x, const double *v, int on_device, const double **dx,
             const double **dv) {
  const size_t n = 3 * (size_t)f->nv;
  if (on_device) {
    *dx = x;
    *dv = v;
    return MPRGP_OK;
  }
  if (!f->xin) {
    int rc = dmalloc(&f->xin, n);
    if (!rc) rc = dmalloc(&f->vin, n);
    if (rc) return rc;
  }
  FK(cudaMemcpyAsync(f->xin, x, n * sizeof(double), cudaMemcpyHostToDevice, f->stream));
  if (v) FK(cudaMemcpyAsync(f->vin, v, n * sizeof(double), cudaMemcpyHostToDevice, f->stream));
  *dx = f->xin;
  *dv = v ? f->vin : nullptr;
  return MPRGP_OK;
}

}  // namespace

extern "C" {

int mprgp_fem_create(mprgp_context *ctx, int nv, int ntet, const int *tets, const double *X,
                     double young, double poisson, double rho, mprgp_fem **out) {
  if (!ctx || !out || nv <= 0 || ntet <= 0 || ntet >= (1 << 29) || !tets || !X ||
      !(young > 0.0) || !(poisson > -1.0 && poisson < 0.5) || !(rho > 0.0))
    return fail(MPRGP_INVALID, "fem_create");
  *out = nullptr;
  // incidence and the block pattern, on the host, once per mesh
  std::vector<int> cnt(nv + 1, 0);
  for (long long i = 0; i < 4LL * ntet; ++i) {
    if (tets[i] < 0 || tets[i] >= nv) return fail(MPRGP_INVALID, "fem_create: tet vertex");
    cnt[tets[i] + 1]++;
  }
  for (int a = 0; a < nv; ++a) cnt[a + 1] += cnt[a];
  std::vector<int> vt(4LL * ntet), fill(cnt.begin(), cnt.end() - 1);
  for (int t = 0; t < ntet; ++t)
    for (int la = 0; la < 4; ++la) vt[fill[tets[4LL * t + la]]++] = (t << 2) | la;
  std::vector<int> row_ptr(nv + 1, 0), cols;
  cols.reserve(16LL * nv);
  std::vector<int> nb;
  for (int a = 0; a < nv; ++a) {
    nb.clear();
    nb.push_back(a);
    for (int idx = cnt[a]; idx < cnt[a + 1]; ++idx) {
      const int t = vt[idx] >> 2;
      for (int lb = 0; lb < 4; ++lb) nb.push_back(tets[4LL * t + lb]);
    }
    std::sort(nb.begin(), nb.end());
    nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
    cols.insert(cols.end(), nb.begin(), nb.end());
    row_ptr[a + 1] = (int)cols.size();
  }
  auto *f = new mprgp_fem();
  f->ctx = ctx;
  f->stream = (cudaStream_t)mprgp_context_stream(ctx);
  f->nv = nv;
  f->ntet = ntet;
  f->nnzb = row_ptr[nv];
  f->lam = poisson * young / ((1.0 + poisson) * (1.0 - 2.0 * poisson));
  f->mu = young / (2.0 * (1.0 + poisson));
  f->rho = rho;
  const size_t n = 3 * (size_t)nv;
  int rc = dmalloc(&f->tets, 4 * (size_t)ntet);
  if (!rc) rc = dmalloc(&f->row_ptr, (size_t)nv + 1);
  if (!rc) rc = dmalloc(&f->cols, (size_t)f->nnzb);
  if (!rc) rc = dmalloc(&f->vt_ptr, (size_t)nv + 1);
  if (!rc) rc = dmalloc(&f->vt, 4 * (size_t)ntet);
  if (!rc) rc = dmalloc(&f->geom, 13 * (size_t)ntet);
  if (!rc) rc = dmalloc(&f->X, n);
  if (!rc) rc = dmalloc(&f->mass, (size_t)nv);
  if (!rc) rc = dmalloc(&f->KX, n);
  if (!rc) rc = dmalloc(&f->vals, 9 * (size_t)f->nnzb);
  if (!rc) rc = dmalloc(&f->b, n);
  if (rc) {
    mprgp_fem_destroy(f);
    return rc;
  }
  cudaStream_t s = f->stream;
  FK(cudaMemcpyAsync(f->tets, tets, sizeof(int) * 4 * (size_t)ntet, cudaMemcpyHostToDevice, s));
  FK(cudaMemcpyAsync(f->row_ptr, row_ptr.data(), sizeof(int) * (nv + 1), cudaMemcpyHostToDevice, s));
  FK(cudaMemcpyAsync(f->cols, cols.data(), sizeof(int) * (size_t)f->nnzb, cudaMemcpyHostToDevice, s));
  FK(cudaMemcpyAsync(f->vt_ptr, cnt.data(), sizeof(int) * (nv + 1), cudaMemcpyHostToDevice, s));
  FK(cudaMemcpyAsync(f->vt, vt.data(), sizeof(int) * 4 * (size_t)ntet, cudaMemcpyHostToDevice, s));
  FK(cudaMemcpyAsync(f->X, X, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  tet_geom_kernel<<<(ntet + 255) / 256, 256, 0, s>>>(ntet, f->tets, f->X, f->geom);
  FK(cudaGetLastError());
  FK(cudaStreamSynchronize(s));  // the host vectors are released next
  *out = f;
  return MPRGP_OK;
}

int mprgp_fem_destroy(mprgp_fem *f) {
  if (!f) return MPRGP_OK;
  if (f->stream) cudaStreamSynchronize(f->stream);
  dfree(f->tets); dfree(f->row_ptr); dfree(f->cols); dfree(f->vt_ptr); dfree(f->vt);
  dfree(f->geom); dfree(f->X); dfree(f->mass); dfree(f->KX); dfree(f->vals); dfree(f->b);
  dfree(f->xin); dfree(f->vin);
  delete f;
  return MPRGP_OK;
}

int mprgp_fem_sizes(mprgp_fem *f, int *nv, int *nnzb) {
  if (!f) return fail(MPRGP_INVALID, "fem_sizes");
  if (nv) *nv = f->nv;
  if (nnzb) *nnzb = f->nnzb;
  return MPRGP_OK;
}

int mprgp_fem_assemble(mprgp_fem *f, double h, const double gravity[3], const double *x,
                       const double *v, int on_device, mprgp_problem *prob, int precisions) {
  if (!f || !(h > 0.0) || !x) return fail(MPRGP_INVALID, "fem_assemble");
  cudaStream_t s = f->stream;
  const double g[3] = {gravity ? gravity[0] : 0.0, gravity ? gravity[1] : 0.0,
                       gravity ? gravity[2] : 0.0};
  assemble_rows_kernel<<<(f->nv + 127) / 128, 128, 0, s>>>(
      f->nv, f->tets, f->geom, f->row_ptr, f->cols, f->vt_ptr, f->vt, f->X, f->lam, f->mu,
      f->rho, h * h, f->vals, f->mass, f->KX);
  FK(cudaGetLastError());
  f->assembled = 1;
  const double *dx, *dv;
  int rc = stage_xv(f, x, v, on_device, &dx, &dv);
  if (rc) return rc;
  const int n3 = 3 * f->nv;
  fem_rhs_kernel<<<(n3 + 255) / 256, 256, 0, s>>>(f->nv, f->mass, f->KX, dx, dv, h, g[0], g[1],
                                                  g[2], f->b);
  FK(cudaGetLastError());
  FK(cudaStreamSynchronize(s));
  if (!prob) return MPRGP_OK;
  rc = mprgp_problem_set_matrix(prob, f->nnzb, f->row_ptr, f->cols, f->vals, precisions, 1);
  if (!rc) rc = mprgp_problem_set_rhs(prob, f->b, 1);
  return rc;
}

int mprgp_fem_rhs(mprgp_fem *f, double h, const double gravity[3], const double *x,
                  const double *v, int on_device, mprgp_problem *prob) {
  if (!f || !(h > 0.0) || !x) return fail(MPRGP_INVALID, "fem_rhs");
  if (!f->assembled) return fail(MPRGP_INVALID, "fem_rhs: assemble first");
  const double g[3] = {gravity ? gravity[0] : 0.0, gravity ? gravity[1] : 0.0,
                       gravity ? gravity[2] : 0.0};
  const double *dx, *dv;
  int rc = stage_xv(f, x, v, on_device, &dx, &dv);
  if (rc) return rc;
  const int n3 = 3 * f->nv;
  fem_rhs_kernel<<<(n3 + 255) / 256, 256, 0, f->stream>>>(f->nv, f->mass, f->KX, dx, dv, h, g[0],
                                                          g[1], g[2], f->b);
  FK(cudaGetLastError());
  FK(cudaStreamSynchronize(f->stream));
  if (!prob) return MPRGP_OK;
  return mprgp_problem_set_rhs(prob, f->b, 1);
}

int mprgp_fem_get(mprgp_fem *f, int *row_ptr, int *cols, double *vals, double *b, double *mass) {
  if (!f || !f->assembled) return fail(MPRGP_INVALID, "fem_get");
  cudaStream_t s = f->stream;
  const size_t n = 3 * (size_t)f->nv;
  if (row_ptr)
    FK(cudaMemcpyAsync(row_ptr, f->row_ptr, sizeof(int) * (f->nv + 1), cudaMemcpyDeviceToHost, s));
  if (cols) FK(cudaMemcpyAsync(cols, f->cols, sizeof(int) * f->nnzb, cudaMemcpyDeviceToHost, s));
  if (vals)
    FK(cudaMemcpyAsync(vals, f->vals, sizeof(double) * 9 * (size_t)f->nnzb,
                       cudaMemcpyDeviceToHost, s));
  if (b) FK(cudaMemcpyAsync(b, f->b, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (mass) FK(cudaMemcpyAsync(mass, f->mass, sizeof(double) * f->nv, cudaMemcpyDeviceToHost, s));
  FK(cudaStreamSynchronize(s));
  return MPRGP_OK;
}

}  // extern "C"
