// Plane-constraint generation on the GPU: the proximity query of the
// reference's LinearConCollider::handle(body, plane, delta)
// (LinearConCollider.cpp:140-161) for a batch of planes.
//
// For every vertex v with position x_v and every plane (n, p) (|n| = 1, the
// half-space n.x + p >= 0), in plane order: the plane becomes a constraint of
// v when n.x_v + p - delta <= 0, unless v already holds a plane within 1e-4
// of it in (n, p) (GeomConCache::addConPlane, LinearConCollider.cpp:43-56);
// with `decoupled`, only the first such plane of a vertex becomes a
// constraint (the one-per-vertex rule, LinearConCollider.cpp:153-158).
// The result -- per-vertex plane lists in CSR form, the reference's (n, p)
// layout -- is written into a problem's constraints from device memory.
//
// The distance test and the duplicate test are evaluated with explicit
// round-to-nearest operations (no fused multiply-adds), in the order
// written, so the selection is the same as a plain FP64 evaluation of the
// same expressions on the host.
#include <algorithm>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mprgp_gpu.h"

namespace mprgp {
void set_last_error(const char *what);
}

namespace {

constexpr int kMaxPerVertex = 3;  // the solver's limit on planes per vertex
constexpr int kScanBlock = 1024;

int fail(int code, const char *what) {
  mprgp::set_last_error(what);
  return code;
}
#define PK(call)                                                  \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) return fail(MPRGP_CUDA_ERROR, #call);  \
  } while (0)

// n.x + p - delta, left to right, no contraction.
__device__ __forceinline__ double signed_gap(const double *pl, const double *x, double delta) {
  double s = __dmul_rn(pl[0], x[0]);
  s = __dadd_rn(s, __dmul_rn(pl[1], x[1]));
  s = __dadd_rn(s, __dmul_rn(pl[2], x[2]));
  s = __dadd_rn(s, pl[3]);
  return __dsub_rn(s, delta);
}

// |a - b| <= 1e-4 over the four components, no contraction.
__device__ __forceinline__ bool same_plane(const double *a, const double *b) {
  double s = 0.0;
  for (int k = 0; k < 4; ++k) {
    const double d = __dsub_rn(a[k], b[k]);
    s = __dadd_rn(s, __dmul_rn(d, d));
  }
  return __dsqrt_rn(s) <= 1e-4;
}

// Per vertex: the selected planes (indices into `planes`), their count, and
// an overflow flag when more than kMaxPerVertex would be selected.
__global__ void select_planes_kernel(int nv, const double *__restrict__ x, int np,
                                     const double *__restrict__ planes, double delta,
                                     int decoupled, int *count, int *sel, int *overflow) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const double xv[3] = {x[3 * (size_t)v], x[3 * (size_t)v + 1], x[3 * (size_t)v + 2]};
  int k = 0;
  int mine[kMaxPerVertex];
  for (int q = 0; q < np; ++q) {
    const double *pl = planes + 4 * (size_t)q;
    if (!(signed_gap(pl, xv, delta) <= 0.0)) continue;
    bool dup = false;
    for (int j = 0; j < k; ++j) dup |= same_plane(planes + 4 * (size_t)mine[j], pl);
    if (dup) continue;
    if (k == kMaxPerVertex) {
      atomicExch(overflow, v + 1);
      break;
    }
    mine[k++] = q;
    if (decoupled) break;
  }
  count[v] = k;
  for (int j = 0; j < k; ++j) sel[kMaxPerVertex * (size_t)v + j] = mine[j];
}

// Exclusive scan of `count` into ptr[0..n] in three passes: block scans with
// block totals, a scan of the totals, and the block offsets added back.
__global__ void scan_blocks_kernel(int n, const int *__restrict__ in, int *out, int *totals) {
  __shared__ int s[kScanBlock];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  s[threadIdx.x] = i < n ? in[i] : 0;
  __syncthreads();
  for (int off = 1; off < kScanBlock; off <<= 1) {
    const int t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i + 1] = s[threadIdx.x];  // inclusive, shifted by one
  if (threadIdx.x == kScanBlock - 1) totals[blockIdx.x] = s[threadIdx.x];
}

__global__ void scan_totals_kernel(int nb, int *totals) {  // one thread: nb is small
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int run = 0;
  for (int b = 0; b < nb; ++b) {
    const int t = totals[b];
    totals[b] = run;
    run += t;
  }
}

__global__ void scan_add_kernel(int n, const int *__restrict__ totals, int *out) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i == 0) out[0] = 0;
  if (i < n) out[i + 1] += totals[blockIdx.x];
}

__global__ void write_planes_kernel(int nv, const int *__restrict__ ptr,
                                    const int *__restrict__ sel, const double *__restrict__ planes,
                                    double *out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int b = ptr[v], k = ptr[v + 1] - b;
  for (int j = 0; j < k; ++j) {
    const double *pl = planes + 4 * (size_t)sel[kMaxPerVertex * (size_t)v + j];
    for (int c = 0; c < 4; ++c) out[4 * (size_t)(b + j) + c] = pl[c];
  }
}

}  // namespace

extern "C" {

int mprgp_planes_collide(mprgp_context *ctx, mprgp_problem *prob, const double *x, int on_device,
                         int nplanes, const double *planes, double delta, int decoupled,
                         int *num_constraints) {
  if (!ctx || !prob || nplanes < 0 || (nplanes > 0 && !planes))
    return fail(MPRGP_INVALID, "planes_collide");
  int nv = 0;
  {
    int rc = mprgp_problem_num_vertices(prob, &nv);
    if (rc) return rc;
  }
  cudaStream_t s = (cudaStream_t)mprgp_context_stream(ctx);
  const size_t n = 3 * (size_t)nv;
  const int nb = (nv + kScanBlock - 1) / kScanBlock;
  // Working arrays of this call (freed before it returns).
  double *d_x = nullptr, *d_planes = nullptr, *d_out = nullptr;
  int *d_count = nullptr, *d_sel = nullptr, *d_ptr = nullptr, *d_tot = nullptr, *d_over = nullptr;
  int rc = MPRGP_OK;
  auto cleanup = [&]() {
    cudaStreamSynchronize(s);
    cudaFree(d_x); cudaFree(d_planes); cudaFree(d_out); cudaFree(d_count); cudaFree(d_sel);
    cudaFree(d_ptr); cudaFree(d_tot); cudaFree(d_over);
  };
#define PC(call)                                   \
  do {                                             \
    cudaError_t _e = (call);                       \
    if (_e != cudaSuccess) {                       \
      cleanup();                                   \
      return fail(MPRGP_CUDA_ERROR, #call);        \
    }                                              \
  } while (0)
  const double *xs = x;
  if (!x) {  // the problem's current x
    PC(cudaMalloc((void **)&d_x, n * sizeof(double)));
    rc = mprgp_problem_get_x(prob, d_x, 1);
    if (rc) {
      cleanup();
      return rc;
    }
    xs = d_x;
  } else if (!on_device) {
    PC(cudaMalloc((void **)&d_x, n * sizeof(double)));
    PC(cudaMemcpyAsync(d_x, x, n * sizeof(double), cudaMemcpyHostToDevice, s));
    xs = d_x;
  }
  PC(cudaMalloc((void **)&d_planes, 4 * (size_t)std::max(nplanes, 1) * sizeof(double)));
  if (nplanes > 0)
    PC(cudaMemcpyAsync(d_planes, planes, 4 * (size_t)nplanes * sizeof(double),
                       cudaMemcpyHostToDevice, s));
  PC(cudaMalloc((void **)&d_count, (size_t)nv * sizeof(int)));
  PC(cudaMalloc((void **)&d_sel, (size_t)kMaxPerVertex * nv * sizeof(int)));
  PC(cudaMalloc((void **)&d_ptr, ((size_t)nv + 1) * sizeof(int)));
  PC(cudaMalloc((void **)&d_tot, (size_t)nb * sizeof(int)));
  PC(cudaMalloc((void **)&d_over, sizeof(int)));
  PC(cudaMemsetAsync(d_over, 0, sizeof(int), s));
  select_planes_kernel<<<(nv + 255) / 256, 256, 0, s>>>(nv, xs, nplanes, d_planes, delta,
                                                        decoupled ? 1 : 0, d_count, d_sel, d_over);
  PC(cudaGetLastError());
  scan_blocks_kernel<<<nb, kScanBlock, 0, s>>>(nv, d_count, d_ptr, d_tot);
  PC(cudaGetLastError());
  scan_totals_kernel<<<1, 1, 0, s>>>(nb, d_tot);
  PC(cudaGetLastError());
  scan_add_kernel<<<nb, kScanBlock, 0, s>>>(nv, d_tot, d_ptr);
  PC(cudaGetLastError());
  int over = 0, m = 0;
  PC(cudaMemcpyAsync(&over, d_over, sizeof(int), cudaMemcpyDeviceToHost, s));
  PC(cudaMemcpyAsync(&m, d_ptr + nv, sizeof(int), cudaMemcpyDeviceToHost, s));
  PC(cudaStreamSynchronize(s));
  if (over) {
    cleanup();
    return fail(MPRGP_INVALID, "planes_collide: a vertex needs more than 3 planes");
  }
  PC(cudaMalloc((void **)&d_out, 4 * (size_t)std::max(m, 1) * sizeof(double)));
  write_planes_kernel<<<(nv + 255) / 256, 256, 0, s>>>(nv, d_ptr, d_sel, d_planes, d_out);
  PC(cudaGetLastError());
  PC(cudaStreamSynchronize(s));
  rc = mprgp_problem_set_planes(prob, d_ptr, d_out, 1);
  cleanup();
  if (!rc && num_constraints) *num_constraints = m;
  return rc;
#undef PC
}

}  // extern "C"
