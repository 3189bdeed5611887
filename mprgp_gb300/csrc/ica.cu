// ICA (Iterative Constraint Anticipation) contact solver on the GPU: the
// reference's comparison baseline for MPRGP, src/MPRGPSolver/ICASolver.h
// (ICASolver :287-463 with ProjectedGaussSeidel :20-150), for
//   A x = r + J^T lambda,  0 <= lambda _|_ J x - p >= 0,
// A in 3x3-block rows (BSR) split as La + Da + Ua by blocks, J given as
// per-vertex planes (n, q): the row n at the vertex's columns with p = -q.
//
// Every iterate is the reference's, computed in a fixed order:
//  * c = p + J Da^-1 (LaUa x - r) and rhs = J^T lambda - Ua x + r are
//    per-vertex passes (thread per vertex);
//  * B = J Da^-1 J^T couples constraints of the same vertex only, so the
//    projected Gauss-Seidel sweep over all rows (GaussSeidel::solve :67-105)
//    is the set of per-vertex sweeps; each sweep ends in a grid reduction of
//    ||lambda - lambda_prev|| for the shared stopping test;
//  * the 3x3-block Gauss-Seidel sweep (:377-388) reads the new x of lower
//    block columns and the old x of upper ones: block rows are grouped in
//    dependency levels (a row's level is one more than the highest level of
//    its lower neighbours), each level's rows are independent and run in
//    parallel, and a grid barrier separates levels -- the same values as the
//    sequential sweep;
//  * ||A x - r - J^T lambda|| ends each iteration.
// One persistent cooperative kernel runs all iterations; grid barriers are
// bounded in time (a wait that runs out sets an error and the kernel
// returns).  Sums run in ascending column / constraint order and this file
// is compiled without fused multiply-adds (-fmad=false), so the results are
// bitwise those of the CPU restatement that performs the same operations.
#include <algorithm>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mprgp_gpu.h"

namespace mprgp {
void set_last_error(const char *what);
int context_lanes_busy(const mprgp_context *c);
}  // namespace mprgp

namespace {

constexpr int kIcaThreads = 256;

struct IcaCtl {
  unsigned int count, gen;
  int err, pad;
};

struct IcaArgs {
  int nv, m, nlevels, max_it, gs_max_it;
  double tol, gs_tol;
  const int *row_ptr, *cols;
  const double *vals;  // 9 per block, row-major
  const double *r;
  const int *plane_ptr;
  const double *planes;  // (n, q) per constraint
  const int *order, *lvl_ptr;  // block rows by level; level starts
  double *x, *lam, *c, *rhs, *inv, *B, *part;
  IcaCtl *ctl;
  double *out;  // iterations, converged, residual, sweeps
  long long wait_ns;
};

__device__ __forceinline__ long long gtimer() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned int atom_add_acq_rel(unsigned int *p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void st_release(unsigned int *p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// Grid barrier with a time bound; false when it (or another CTA's) ran out.
__device__ bool ica_barrier(IcaCtl *ctl, long long wait_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (gridDim.x == 1) return true;
  if (threadIdx.x == 0) {
    volatile int *verr = &ctl->err;
    const unsigned int g = ld_acquire(&ctl->gen);
    const unsigned int arrived = atom_add_acq_rel(&ctl->count, 1u);
    int ok = 1;
    if (arrived == gridDim.x - 1) {
      ctl->count = 0u;
      st_release(&ctl->gen, g + 1);
    } else {
      const long long t0 = gtimer();
      while (ld_acquire(&ctl->gen) == g) {
        if (*verr) {
          ok = 0;
          break;
        }
        if (gtimer() - t0 > wait_ns) {
          atomicCAS(&ctl->err, 0, 1);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    s_ok = ok && *verr == 0;
  }
  __syncthreads();
  return s_ok;
}

// Sum of one double per thread over the grid, the same on every CTA: block
// sums in a fixed tree, written to part[par][block], then one warp adds the
// block sums in a fixed order.  `ok` turns false if the barrier gave up.
__device__ double grid_sum(double v, double *part, int par, IcaCtl *ctl, long long wait_ns,
                           bool &ok) {
  __shared__ double sh[kIcaThreads / 32];
  __shared__ double s_tot;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kIcaThreads / 32; ++w) t += sh[w];
    part[par * gridDim.x + blockIdx.x] = t;
  }
  ok = ica_barrier(ctl, wait_ns);
  if (!ok) return 0.0;
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) t += part[par * gridDim.x + b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) s_tot = t;
  }
  __syncthreads();
  return s_tot;
}

__device__ __forceinline__ void mul3(const double *M, const double *v, double *y) {
#pragma unroll
  for (int k = 0; k < 3; ++k) y[k] = (M[3 * k] * v[0] + M[3 * k + 1] * v[1]) + M[3 * k + 2] * v[2];
}

// 3x3 inverse: adjugate over the determinant expanded along row 0.
__device__ void inverse3(const double *m, double *inv) {
  const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7],
               i = m[8];
  const double c00 = e * i - f * h, c01 = f * g - d * i, c02 = d * h - e * g;
  const double det = (a * c00 + b * c01) + c * c02;
  const double s = 1.0 / det;
  inv[0] = c00 * s;
  inv[1] = (c * h - b * i) * s;
  inv[2] = (b * f - c * e) * s;
  inv[3] = c01 * s;
  inv[4] = (a * i - c * g) * s;
  inv[5] = (c * d - a * f) * s;
  inv[6] = c02 * s;
  inv[7] = (b * g - a * h) * s;
  inv[8] = (a * e - b * d) * s;
}

// (J^T lambda) at vertex v.
__device__ __forceinline__ void jt_lambda(const IcaArgs &a, int v, double jl[3]) {
  jl[0] = jl[1] = jl[2] = 0.0;
  for (int q = a.plane_ptr[v]; q < a.plane_ptr[v + 1]; ++q) {
    const double *pl = a.planes + 4 * (size_t)q;
    const double l = a.lam[q];
#pragma unroll
    for (int k = 0; k < 3; ++k) jl[k] = jl[k] + l * pl[k];
  }
}

// Row sums of block row v over the blocks whose column passes `take`.
template <typename Take>
__device__ __forceinline__ void row_sum(const IcaArgs &a, int v, const double *x, Take take,
                                        double acc[3]) {
  acc[0] = acc[1] = acc[2] = 0.0;
  for (int k = a.row_ptr[v]; k < a.row_ptr[v + 1]; ++k) {
    const int u = a.cols[k];
    if (!take(u)) continue;
    const double *blk = a.vals + 9 * (size_t)k;
    const double *xc = x + 3 * (size_t)u;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int b = 0; b < 3; ++b) acc[r] = acc[r] + blk[3 * r + b] * xc[b];
  }
}

__global__ void __launch_bounds__(kIcaThreads) ica_kernel(IcaArgs a) {
  __shared__ double s_blk[kIcaThreads / 32][32][12];  // per warp: 32 blocks + their x
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gthreads = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int gwarp = gtid >> 5, gwarps = gthreads >> 5;
  // reset (:296-350): Da^-1 per block row; B = J Da^-1 J^T per vertex.
  for (int v = gtid; v < a.nv; v += gthreads) {
    double *inv = a.inv + 9 * (size_t)v;
    for (int k = a.row_ptr[v]; k < a.row_ptr[v + 1]; ++k)
      if (a.cols[k] == v) inverse3(a.vals + 9 * (size_t)k, inv);
    const int q0 = a.plane_ptr[v], nq = a.plane_ptr[v + 1] - q0;
    for (int j = 0; j < nq; ++j) {
      double t[3];
      mul3(inv, a.planes + 4 * (size_t)(q0 + j), t);
      for (int i = 0; i < nq; ++i) {
        const double *ni = a.planes + 4 * (size_t)(q0 + i);
        a.B[9 * (size_t)v + 3 * i + j] = (ni[0] * t[0] + ni[1] * t[1]) + ni[2] * t[2];
      }
    }
    for (int q = q0; q < q0 + nq; ++q) a.lam[q] = 0.0;
  }
  int par = 0, it = 0, conv = 0;
  long long sweeps = 0;
  double res = 0.0;
  bool ok = true;
  for (; it < a.max_it; ++it) {
    // c = p + J Da^-1 (LaUa x - r)                                    (:371)
    for (int v = gtid; v < a.nv; v += gthreads) {
      double u[3], w[3];
      row_sum(a, v, a.x, [v](int col) { return col != v; }, u);
#pragma unroll
      for (int k = 0; k < 3; ++k) u[k] = u[k] - a.r[3 * v + k];
      mul3(a.inv + 9 * (size_t)v, u, w);
      for (int q = a.plane_ptr[v]; q < a.plane_ptr[v + 1]; ++q) {
        const double *pl = a.planes + 4 * (size_t)q;
        a.c[q] = -pl[3] + ((pl[0] * w[0] + pl[1] * w[1]) + pl[2] * w[2]);
      }
    }
    // projected Gauss-Seidel on B, warm-started from the last lambda (:372)
    for (int s = 0; s < a.gs_max_it; ++s) {
      double ss = 0.0;
      for (int v = gtid; v < a.nv; v += gthreads) {
        const int q0 = a.plane_ptr[v], nq = a.plane_ptr[v + 1] - q0;
        const double *B = a.B + 9 * (size_t)v;
        double old[3] = {0.0, 0.0, 0.0}, l[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < nq; ++i) old[i] = a.lam[q0 + i];
        for (int i = 0; i < nq; ++i) {
          double ub = 0.0;
          for (int j = i + 1; j < nq; ++j) ub = ub + B[3 * i + j] * old[j];
          double rr = a.c[q0 + i] - ub;
          for (int j = 0; j < i; ++j) rr -= l[j] * B[3 * i + j];
          const double li = rr * (1.0 / B[3 * i + i]);
          l[i] = li > 0 ? li : 0;
        }
        for (int i = 0; i < nq; ++i) {
          a.lam[q0 + i] = l[i];
          const double d = l[i] - old[i];
          ss = ss + d * d;
        }
      }
      const double tot = grid_sum(ss, a.part, par, a.ctl, a.wait_ns, ok);
      par ^= 1;
      ++sweeps;
      if (!ok) return;
      if (sqrt(tot) <= a.gs_tol) break;
    }
    // rhs = J^T lambda - Ua x + r (old x)                              (:374)
    for (int v = gtid; v < a.nv; v += gthreads) {
      double jl[3], ua[3];
      jt_lambda(a, v, jl);
      row_sum(a, v, a.x, [v](int col) { return col > v; }, ua);
#pragma unroll
      for (int k = 0; k < 3; ++k) a.rhs[3 * v + k] = (jl[k] - ua[k]) + a.r[3 * v + k];
    }
    if (!ica_barrier(a.ctl, a.wait_ns)) return;
    // 3x3-block Gauss-Seidel sweep (:377-388), level by level, one warp per
    // block row: the lanes fetch the row's lower blocks and their x together
    // (one round of loads); lane k (k < 3) then subtracts them from scalar
    // row k in column order, and lane k forms component k of the new x.
    for (int lv = 0; lv < a.nlevels; ++lv) {
      for (int t = a.lvl_ptr[lv] + gwarp; t < a.lvl_ptr[lv + 1]; t += gwarps) {
        const int v = a.order[t];
        const int k0 = a.row_ptr[v], k1 = a.row_ptr[v + 1];
        double acc = lane < 3 ? a.rhs[3 * v + lane] : 0.0;
        for (int base = k0; base < k1; base += 32) {
          const int j = base + lane;
          const int u = j < k1 ? a.cols[j] : v;
          const bool low = u < v;
          if (low) {
            const double *blk = a.vals + 9 * (size_t)j;
            const double *xc = a.x + 3 * (size_t)u;
#pragma unroll
            for (int e = 0; e < 9; ++e) s_blk[wid][lane][e] = blk[e];
#pragma unroll
            for (int b = 0; b < 3; ++b) s_blk[wid][lane][9 + b] = xc[b];
          }
          const unsigned int lower = __ballot_sync(0xffffffffu, low);
          __syncwarp();
          if (lane < 3) {
            const int cnt = min(32, k1 - base);
            for (int q = 0; q < cnt; ++q) {
              if (!((lower >> q) & 1u)) continue;
              const double *s = s_blk[wid][q];
#pragma unroll
              for (int b = 0; b < 3; ++b) acc -= s[3 * lane + b] * s[9 + b];
            }
          }
          __syncwarp();
        }
        const double r0 = __shfl_sync(0xffffffffu, acc, 0), r1 = __shfl_sync(0xffffffffu, acc, 1),
                     r2 = __shfl_sync(0xffffffffu, acc, 2);
        if (lane < 3) {
          const double *M = a.inv + 9 * (size_t)v + 3 * lane;
          a.x[3 * (size_t)v + lane] = (M[0] * r0 + M[1] * r1) + M[2] * r2;
        }
      }
      if (!ica_barrier(a.ctl, a.wait_ns)) return;
    }
    // residual = ||A x - r - J^T lambda||                              (:390)
    double ss = 0.0;
    for (int v = gtid; v < a.nv; v += gthreads) {
      double jl[3], ax[3];
      jt_lambda(a, v, jl);
      row_sum(a, v, a.x, [](int) { return true; }, ax);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double t = (ax[k] - a.r[3 * v + k]) - jl[k];
        ss = ss + t * t;
      }
    }
    const double tot = grid_sum(ss, a.part, par, a.ctl, a.wait_ns, ok);
    par ^= 1;
    if (!ok) return;
    res = sqrt(tot);
    if (res <= a.tol) {
      conv = 1;
      break;
    }
  }
  if (gtid == 0) {
    a.out[0] = (double)it;
    a.out[1] = (double)conv;
    a.out[2] = res;
    a.out[3] = (double)sweeps;
  }
}

int fail(int code, const char *what) {
  mprgp::set_last_error(what);
  return code;
}

}  // namespace

extern "C" {

int mprgp_ica_solve(mprgp_context *ctx, int nv, int nnzb, const int *row_ptr, const int *cols,
                    const double *vals, const double *r, const int *plane_ptr,
                    const double *planes, double *x, double *lambda, int max_it, double tol,
                    int gs_max_it, double gs_tol, mprgp_ica_stats *stats) {
  if (!ctx || nv <= 0 || nnzb <= 0 || !row_ptr || !cols || !vals || !r || !plane_ptr || !x ||
      max_it < 0 || gs_max_it < 0 || !(tol >= 0.0) || !(gs_tol >= 0.0))
    return fail(MPRGP_INVALID, "ica_solve: arguments");
  if (mprgp::context_lanes_busy(ctx))
    return fail(MPRGP_BUSY, "ica_solve: the context has asynchronous server runs in flight");
  const int m = plane_ptr[nv];
  if (m < 0 || (m > 0 && (!planes || !lambda))) return fail(MPRGP_INVALID, "ica_solve: planes");
  if (row_ptr[0] != 0 || row_ptr[nv] != nnzb) return fail(MPRGP_INVALID, "ica_solve: row_ptr");
  // Dependency levels of the block sweep and the checks the kernel relies
  // on: a diagonal block in every row, columns in range, <= 3 planes a vertex.
  std::vector<int> level(nv, 0), cnt(1, 0);
  int nlevels = 0;
  for (int v = 0; v < nv; ++v) {
    if (plane_ptr[v + 1] < plane_ptr[v] || plane_ptr[v + 1] - plane_ptr[v] > 3)
      return fail(MPRGP_INVALID, "ica_solve: 0..3 planes per vertex");
    if (row_ptr[v + 1] < row_ptr[v]) return fail(MPRGP_INVALID, "ica_solve: row_ptr");
    bool diag = false;
    int lv = 0;
    for (int k = row_ptr[v]; k < row_ptr[v + 1]; ++k) {
      const int u = cols[k];
      if (u < 0 || u >= nv) return fail(MPRGP_INVALID, "ica_solve: column out of range");
      if (u == v) diag = true;
      if (u < v) lv = std::max(lv, level[u] + 1);
    }
    if (!diag) return fail(MPRGP_INVALID, "ica_solve: missing diagonal block");
    level[v] = lv;
    nlevels = std::max(nlevels, lv + 1);
  }
  std::vector<int> lvl_ptr(nlevels + 1, 0), order(nv);
  for (int v = 0; v < nv; ++v) lvl_ptr[level[v] + 1]++;
  for (int l = 0; l < nlevels; ++l) lvl_ptr[l + 1] += lvl_ptr[l];
  {
    std::vector<int> fill(lvl_ptr.begin(), lvl_ptr.end() - 1);
    for (int v = 0; v < nv; ++v) order[fill[level[v]]++] = v;
  }
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ica_kernel, kIcaThreads, 0) !=
          cudaSuccess || per_sm < 1)
    return fail(MPRGP_CUDA_ERROR, "ica_solve: occupancy");
  const int grid = std::max(1, std::min(nsm, (nv + kIcaThreads - 1) / kIcaThreads));
  cudaStream_t s = (cudaStream_t)mprgp_context_stream(ctx);
  const size_t n = 3 * (size_t)nv, mm = std::max(m, 1);
  // one device block for everything, carved in 256-byte steps
  size_t off = 0;
  auto take = [&off](size_t bytes) {
    const size_t at = off;
    off = (off + bytes + 255) & ~size_t(255);
    return at;
  };
  const size_t o_rp = take(sizeof(int) * (nv + 1)), o_cols = take(sizeof(int) * nnzb),
               o_vals = take(sizeof(double) * 9 * (size_t)nnzb), o_r = take(sizeof(double) * n),
               o_pp = take(sizeof(int) * (nv + 1)), o_pl = take(sizeof(double) * 4 * mm),
               o_ord = take(sizeof(int) * nv), o_lp = take(sizeof(int) * (nlevels + 1)),
               o_x = take(sizeof(double) * n), o_lam = take(sizeof(double) * mm),
               o_c = take(sizeof(double) * mm), o_rhs = take(sizeof(double) * n),
               o_inv = take(sizeof(double) * 9 * (size_t)nv),
               o_B = take(sizeof(double) * 9 * (size_t)nv),
               o_part = take(sizeof(double) * 2 * grid), o_ctl = take(sizeof(IcaCtl)),
               o_out = take(sizeof(double) * 4);
  unsigned char *d = nullptr;
  if (cudaMallocAsync((void **)&d, off, s) != cudaSuccess)
    return fail(MPRGP_OOM, "ica_solve: device memory");
  int rc = MPRGP_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double out[4] = {0, 0, 0, 0};
  float ms = 0.f;
  auto up = [&](size_t o, const void *h, size_t bytes) {
    return cudaMemcpyAsync(d + o, h, bytes, cudaMemcpyHostToDevice, s);
  };
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = up(o_rp, row_ptr, sizeof(int) * (nv + 1));
  if (e == cudaSuccess) e = up(o_cols, cols, sizeof(int) * nnzb);
  if (e == cudaSuccess) e = up(o_vals, vals, sizeof(double) * 9 * (size_t)nnzb);
  if (e == cudaSuccess) e = up(o_r, r, sizeof(double) * n);
  if (e == cudaSuccess) e = up(o_pp, plane_ptr, sizeof(int) * (nv + 1));
  if (e == cudaSuccess && m > 0) e = up(o_pl, planes, sizeof(double) * 4 * (size_t)m);
  if (e == cudaSuccess) e = up(o_ord, order.data(), sizeof(int) * nv);
  if (e == cudaSuccess) e = up(o_lp, lvl_ptr.data(), sizeof(int) * (nlevels + 1));
  if (e == cudaSuccess) e = up(o_x, x, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMemsetAsync(d + o_ctl, 0, sizeof(IcaCtl), s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    IcaArgs a;
    a.nv = nv;
    a.m = m;
    a.nlevels = nlevels;
    a.max_it = max_it;
    a.gs_max_it = gs_max_it;
    a.tol = tol;
    a.gs_tol = gs_tol;
    a.row_ptr = (const int *)(d + o_rp);
    a.cols = (const int *)(d + o_cols);
    a.vals = (const double *)(d + o_vals);
    a.r = (const double *)(d + o_r);
    a.plane_ptr = (const int *)(d + o_pp);
    a.planes = (const double *)(d + o_pl);
    a.order = (const int *)(d + o_ord);
    a.lvl_ptr = (const int *)(d + o_lp);
    a.x = (double *)(d + o_x);
    a.lam = (double *)(d + o_lam);
    a.c = (double *)(d + o_c);
    a.rhs = (double *)(d + o_rhs);
    a.inv = (double *)(d + o_inv);
    a.B = (double *)(d + o_B);
    a.part = (double *)(d + o_part);
    a.ctl = (IcaCtl *)(d + o_ctl);
    a.out = (double *)(d + o_out);
    a.wait_ns = 5000000000LL;  // 5 s per barrier wait
    void *params[] = {&a};
    e = cudaEventRecord(e0, s);
    if (e == cudaSuccess)
      e = cudaLaunchCooperativeKernel((const void *)ica_kernel, dim3(grid), dim3(kIcaThreads),
                                      params, 0, s);
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
  }
  IcaCtl ctl{};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&ctl, d + o_ctl, sizeof(IcaCtl), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d + o_out, sizeof(out), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(x, d + o_x, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && m > 0)
    e = cudaMemcpyAsync(lambda, d + o_lam, sizeof(double) * m, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e != cudaSuccess) rc = fail(MPRGP_CUDA_ERROR, "ica_solve: CUDA call failed");
  else if (ctl.err) rc = fail(MPRGP_TIMEOUT, "ica_solve: device wait limit reached");
  cudaFreeAsync(d, s);
  cudaStreamSynchronize(s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc) return rc;
  if (stats) {
    stats->iterations = (int)out[0];
    stats->converged = (int)out[1];
    stats->residual = out[2];
    stats->pgs_sweeps = (long long)out[3];
    stats->levels = nlevels;
    stats->device_ms = ms;
  }
  return out[1] != 0.0 ? MPRGP_OK : MPRGP_NOT_CONVERGED;
}

}  // extern "C"
