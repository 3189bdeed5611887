// Host side of the C ABI (include/mprgp_gpu.h): device memory for each QP
// instance, uploads, and launches of the persistent engine.
//
// Every failure is reported as a status code; nothing falls back to a CPU
// path.  A problem keeps A (SELL-32, FP64 and/or FP32), b, the constraints,
// x, the face and the power-method vector resident between solves.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mprgp_gpu.h"
#include "engine.h"
#include "nvtx_ranges.h"

namespace mprgp {
cudaError_t launch_engine(const EngineArgs &args, int grid, cudaStream_t stream);
cudaError_t build_power_graph(int grid, int variant, const EngineArgs *d_args, PowCtl *d_pc,
                              cudaGraph_t *graph, cudaGraphExec_t *exec);
cudaError_t power_max_blocks_per_sm(int variant, int *n);
cudaError_t launch_power_persistent(const EngineArgs &args, PowCtl *d_pc, int limit, int grid,
                                    cudaStream_t stream);
cudaError_t power_persistent_max_blocks_per_sm(int *n);
cudaError_t launch_cluster(const ClusterArgs &args, int csize, cudaStream_t stream);
cudaError_t cluster_max_active(int csize, int *n);
cudaError_t launch_power_direct(int grid, int variant, int launches, const EngineArgs *d_args,
                                PowCtl *d_pc, cudaStream_t stream);
cudaError_t engine_max_blocks_per_sm(int *n, int stage_bytes);
void launch_bsr_to_sell(int nv, const int *row_ptr, const int *cols, const double *vals,
                        const int *slice_off, const int *rowmap, int *out_cols, short *out_cols16,
                        int *c16ok, double *out64, float *out32, double *dinv, int *bad,
                        cudaStream_t st);
void launch_planes_setup(int nv, const int *plane_ptr, const double *in, double *out, double *nn,
                         double *indn, const double *dinv, unsigned char *unit, cudaStream_t st);
void launch_planes_axis(int m, const double *in, unsigned char *axis, cudaStream_t st);
void launch_state_scatter(const InstDesc *desc, int n, InstState *states, InstState *const *home,
                          const int *fresh, cudaStream_t st);
void launch_state_gather(const InstDesc *desc, int n, InstState *states, InstState *const *home,
                         cudaStream_t st);
void launch_spmv(const SellMatrix &A, int nv, bool fp32, const double *x, double *y,
                 cudaStream_t st);
}  // namespace mprgp

using namespace mprgp;

// Device and pinned-host resources of one engine lane, and the run in flight
// on it.  Lane 0 runs on the context stream (the synchronous calls); the
// server's asynchronous form runs the small instances on lane 1, the large
// ones' MPRGP phases on lane 2 and (in its three-lane form) their power
// method on lane 3, each on a stream of its own, so no lane's run waits for
// another's.
struct LaneRun {
  bool active = false;
  int n = 0, n_large = 0, quantum = 0, cluster_quantum = 0, power_launches = 0;
  bool power = false, power_graph = false, power_persistent = false, egraph = false;
  int power_variant = 0;  // the power loop's kernel variant (3: the power-step loop)
  int egraph_stream = 0;  // > 0: the engine loop ran as this many stream launches
  int class_n[kClusterClasses] = {0, 0, 0, 0, 0};
  std::vector<mprgp_problem *> probs;
  std::vector<mprgp_options> opts;
  std::vector<int> pos;
};

struct HostIO {  // pinned: the run's control blocks in and out
  Ctl ctl_in, ctl_out;
  PowCtl pc_in[2], pc_out[2];  // power loop, engine loop
  EngineArgs args;
};

struct Lane {
  bool ready = false, own_stream = false;
  cudaStream_t stream = nullptr;
  Ctl *ctl = nullptr;
  EngineArgs *d_args = nullptr;
  PowCtl *d_pc = nullptr, *d_pc2 = nullptr;  // power loop, engine loop
  cudaStream_t side[kClusterClasses] = {};   // one per cluster size (run concurrently)
  cudaEvent_t fork_ev = nullptr, join_ev[kClusterClasses] = {};
  cudaEvent_t fence = nullptr;               // context-stream work the run depends on
  nvtxRangeId_t nvtx = 0;                    // the run in flight on the host timeline
  cudaEvent_t e0 = nullptr, e1 = nullptr, e_pow = nullptr, e_end = nullptr;
  // loop graphs of the phase kernel, keyed grid * 4 + variant (they hold
  // this lane's d_args / d_pc / d_pc2)
  std::map<int, std::pair<cudaGraph_t, cudaGraphExec_t>> graphs;
  // per-run arrays in desc order (grown on demand); d_st holds the run's
  // instance states, home their problems' own state blocks
  int cap = 0, icap = 0;
  InstDesc *d_desc = nullptr, *h_desc = nullptr;
  int *d_prefix = nullptr, *h_prefix = nullptr;
  InstState *d_st = nullptr, *h_st_in = nullptr, *h_st_out = nullptr;
  InstState **d_home = nullptr, **h_home = nullptr;
  int *d_fresh = nullptr, *h_fresh = nullptr;
  int *d_item_inst = nullptr, *h_item_inst = nullptr;  // items of the large instances
  HostIO *io = nullptr;
  LaneRun run;
};
constexpr int kLanes = 7;  // 0: synchronous calls; 1..6: the server's asynchronous lanes

// Pinned staging for the small arrays the host builds and uploads (SELL slice
// offsets and row order, plane offsets).  A cudaMemcpyAsync from pageable
// memory returns only after the stream's earlier work, which may wait for SM
// room behind other lanes' runs; one from pinned memory returns at once.  A
// ring: a region is written again only after the event recorded behind its
// copy has completed.
struct HostRing {
  static constexpr size_t kBytes = 16u << 20;
  char *base = nullptr;
  size_t head = 0;
  bool failed = false;  // no pinned memory: uploads stay pageable
  struct Use {
    size_t a, b;
    cudaEvent_t ev;
  };
  std::deque<Use> uses;               // in ring order
  std::vector<cudaEvent_t> spare;     // completed events for reuse
};

struct mprgp_context {
  int device = 0;
  // Uploads and setup kernels; the highest priority the device offers, so
  // that the few CTAs of a setup kernel are placed before the pending CTAs of
  // a lane's long runs (the lanes' runs wait for this stream's work).
  cudaStream_t stream = nullptr;
  // Device-to-host reads that must not wait for the context stream: results
  // of a lane run that has ended, and offsets read from caller device arrays.
  cudaStream_t io = nullptr;
  int nsm = 0, bps = 0, bps_stage = 0;
  int stage = 0;         // stage FP32 A in shared memory (1) or not (0)
  int power_kernel = 1;  // power method by the dedicated kernel (1) or the engine (0)
  int power_graph = 1;   // power-kernel loop as a CUDA-graph WHILE node (1) or stream launches (0)
  int power_variant = 0; // power kernel with 40 registers (0, 6 CTAs/SM) or 64 (1, 4 CTAs/SM)
  int bps_power_v[4] = {0, 0, 0, 0};  // per power-kernel variant (2: all phases, 3: power steps)
  int power_step = 1;    // power loop as the power-step loop (1, the default; deferred
                         // finalize) or the phase kernel with a finalize per launch (0)
  int power_persistent = 0;  // power loop as one persistent cooperative launch when the run
                            // is synchronous and its items fit (1)
  int bps_power_pp = 0;      // resident CTAs per SM of that kernel
  int engine_graph = 0;  // large instances' phases as a graph loop of the phase kernel (1)
                         // or the persistent cooperative engine (0)
  int cluster = 16;      // largest cluster of the small-instance solver (0 = off)
  int cluster_items = 1; // items per CTA allowed in the largest cluster (1..kClusterItems)
  int cluster_ok[kClusterClasses] = {0, 0, 0, 0, 0};  // cluster sizes 1, 2, 4, 8, 16 usable
  int ctas_per_sm = 0;   // persistent CTAs per SM (0 = all resident)
  size_t l2_bytes = 0;   // the device's L2 size
  cudaMemPool_t pool = nullptr;      // every device array of the context's problems
  mprgp_problem *scratch = nullptr;
  int bps_power = 0;
  Lane lane[kLanes];
  HostRing ring;
  long long launches = 0;  // kernels launched (each power-loop iteration counts)
  double solver_ms = 0.0;  // device time of engine runs, summed over runs (lanes overlap)
  double power_ms = 0.0;   // device time of the power loop alone
};

struct mprgp_problem {
  mprgp_context *ctx = nullptr;
  int nv = 0, nnzb = 0, m = 0, nslices = 0, slots = 0;
  int cons = 0;  // 0 none, 1 planes, 2 bounds (lower), 3 bounds (box)
  int has64 = 0, has32 = 0;
  int xc = 0, ev_valid = 0, planes_dirty = 0;
  int *slice_off = nullptr, *cols = nullptr;
  short *cols16 = nullptr;  // the columns as 16-bit offsets from the row's vertex
  int *c16ok = nullptr;     // set by the conversion: every offset fitted in 16 bits
  double *v64 = nullptr;
  float *v32 = nullptr;
  double *dinv = nullptr, *b = nullptr;
  int *plane_ptr = nullptr;
  double *planes_raw = nullptr, *planes = nullptr, *pl_nn = nullptr, *pl_indn = nullptr;
  unsigned char *pl_unit = nullptr;  // per vertex: its planes are orthonormal
  unsigned char *pl_axis = nullptr;  // per plane row: its normal's unit axis (3: none)
  double *L = nullptr, *U = nullptr;
  unsigned char *face = nullptr;
  int face_len = 0;
  double *vec = nullptr, *ev = nullptr, *part = nullptr;
  float *vec32 = nullptr;
  unsigned int *cnt = nullptr;
  int *bad = nullptr;           // set on the device when A had a column outside 0..nv-1
  int bad_host = -1;            // its value once read back (-1: not read since set_matrix)
  InstState *st = nullptr;
  double *trace = nullptr;
  int trace_cap = 0, trace_n = 0;
  // device staging for host BSR uploads (grow-only)
  int *stage_ptr = nullptr, *stage_cols = nullptr;
  double *stage_vals = nullptr;
  size_t stage_nnzb = 0;
  std::vector<int> h_plane_ptr;
  std::vector<int> h_len;     // blocks per row of A
  int *rowmap = nullptr;      // SELL row -> vertex (nullptr: identity)
  unsigned long long layout = 0;
  int want64 = 0, want32 = 0;
  int phase_host = 0;  // the instance's phase at the end of its last engine run
  // Result of the last power method that started from the seeded random
  // vector.  That power method is a deterministic function of (A, seed,
  // precision form), so a later solve with the same three and the same start
  // reuses it and gets a bitwise identical alpha_bar (a timestep re-solve of
  // a resident scene keeps A and the seed).
  struct {
    int valid = 0, prec = 0, power_iters = 0;
    unsigned long long seed = 0, gen = 0;
    double spec_rad = 0.0;
  } pcache;
  // Result of the last power method that started from the stored vector ev
  // and left ev unchanged (it ran to its iteration limit; specRad writes ev
  // only when it stops early, MPRGPSolver.h:62-74): a deterministic function
  // of (A, ev, precision form), reused while the three stay the same -- a
  // resident scene's follow-up timesteps warm-start from ev.
  struct {
    int valid = 0, prec = 0, power_iters = 0;
    unsigned long long gen = 0, ev_gen = 0;
    double spec_rad = 0.0;
  } pcache_ev;
  int pcache_on = 1;
  unsigned long long matrix_gen = 0;  // bumped by every set_matrix
  unsigned long long ev_gen = 0;      // bumped whenever ev may have been rewritten
  int run_random = 0, run_cached = 0;  // how the current solve's power method starts
  int run_ev = 0;                      // ... from ev (ev_gen at its start: run_ev_gen)
  unsigned long long run_ev_gen = 0;
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *what) {
  g_last_error = what;
  return code;
}
int cuda_fail(cudaError_t e, const char *what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return MPRGP_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return MPRGP_NO_DEVICE;
  return MPRGP_CUDA_ERROR;
}
#define CK(call)                                       \
  do {                                                 \
    cudaError_t _e = (call);                           \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

// Device memory comes from the context's stream-ordered pool: allocations
// and frees are ordered on the context stream and freed blocks stay reserved
// for the next problem, so admitting and evicting problems in a serving loop
// neither calls cudaMalloc nor synchronises the device (cudaFree would).
template <typename T>
int dalloc(mprgp_context *c, T **p, size_t count) {
  *p = nullptr;
  if (count == 0) return MPRGP_OK;
  CK(cudaMallocFromPoolAsync((void **)p, count * sizeof(T), c->pool, c->stream));
  return MPRGP_OK;
}
template <typename T>
void dfree(mprgp_context *c, T *&p) {
  if (p) cudaFreeAsync((void *)p, c->stream);
  p = nullptr;
}

int nitems_of(int nv) { return (nv + kThreads - 1) / kThreads; }

// Host -> device copy of a host-built array on stream s through the pinned
// ring (pageable, and so ordered behind the stream's earlier work, only when
// the array is larger than half the ring or pinned memory was refused).
int upload(mprgp_context *c, void *dst, const void *src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return MPRGP_OK;
  HostRing &R = c->ring;
  if (!R.base && !R.failed) {
    if (cudaMallocHost((void **)&R.base, HostRing::kBytes) != cudaSuccess) {
      cudaGetLastError();
      R.base = nullptr;
      R.failed = true;
    }
  }
  if (!R.base || bytes > HostRing::kBytes / 2) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    return MPRGP_OK;
  }
  const size_t sz = (bytes + 255) & ~(size_t)255;
  if (R.head + sz > HostRing::kBytes) R.head = 0;
  const size_t a = R.head, b = a + sz;
  // wait for earlier copies out of [a, b); retire every completed one
  for (auto &u : R.uses)
    if (u.a < b && a < u.b) CK(cudaEventSynchronize(u.ev));
  while (!R.uses.empty() && cudaEventQuery(R.uses.front().ev) == cudaSuccess) {
    R.spare.push_back(R.uses.front().ev);
    R.uses.pop_front();
  }
  std::memcpy(R.base + a, src, bytes);
  CK(cudaMemcpyAsync(dst, R.base + a, bytes, cudaMemcpyHostToDevice, s));
  cudaEvent_t ev;
  if (!R.spare.empty()) {
    ev = R.spare.back();
    R.spare.pop_back();
  } else {
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  CK(cudaEventRecord(ev, s));
  R.uses.push_back({a, b, ev});
  R.head = b;
  return MPRGP_OK;
}

void free_problem_arrays(mprgp_problem *p) {
  dfree(p->ctx, p->slice_off); dfree(p->ctx, p->cols); dfree(p->ctx, p->cols16); dfree(p->ctx, p->c16ok); dfree(p->ctx, p->v64); dfree(p->ctx, p->v32);
  dfree(p->ctx, p->dinv); dfree(p->ctx, p->b); dfree(p->ctx, p->plane_ptr); dfree(p->ctx, p->planes_raw);
  dfree(p->ctx, p->planes); dfree(p->ctx, p->pl_nn); dfree(p->ctx, p->pl_indn); dfree(p->ctx, p->pl_unit); dfree(p->ctx, p->pl_axis); dfree(p->ctx, p->L); dfree(p->ctx, p->U);
  dfree(p->ctx, p->face); dfree(p->ctx, p->vec); dfree(p->ctx, p->vec32); dfree(p->ctx, p->ev); dfree(p->ctx, p->part); dfree(p->ctx, p->cnt); dfree(p->ctx, p->bad); dfree(p->ctx, p->st);
  dfree(p->ctx, p->trace); dfree(p->ctx, p->stage_ptr); dfree(p->ctx, p->stage_cols); dfree(p->ctx, p->stage_vals);
  dfree(p->ctx, p->rowmap);
}

// The SELL row order of a problem: vertices with several constraint planes
// are gathered into whole warps (slices of 32 rows), and those slices are
// spread evenly over the matrix, so that the multi-plane projection runs in
// few, uniform warps whose extra work is shared by all SMs; the other
// vertices keep their order.  Identity when no vertex has several planes.
// The key identifies the order.
unsigned long long layout_key(const mprgp_problem *p) {
  unsigned long long h = 1469598103934665603ull;
  if (p->cons != 1 || p->h_plane_ptr.empty()) return h;
  for (int v = 0; v < p->nv; ++v)
    if (p->h_plane_ptr[v + 1] - p->h_plane_ptr[v] >= 2) {
      h ^= (unsigned long long)v + 0x9E3779B97F4A7C15ull;
      h *= 1099511628211ull;
    }
  return h;
}

// (Re)builds the SELL copy of A from the device BSR in the order above.
int build_layout(mprgp_problem *p, unsigned long long key) {
  mprgp_context *c = p->ctx;
  cudaStream_t s = c->stream;
  const int nv = p->nv;
  std::vector<int> order;  // slot -> vertex
  if (p->cons == 1 && !p->h_plane_ptr.empty()) {
    std::vector<int> multi, single;
    for (int v = 0; v < nv; ++v) {
      if (p->h_plane_ptr[v + 1] - p->h_plane_ptr[v] >= 2) multi.push_back(v);
      else single.push_back(v);
    }
    if (!multi.empty()) {
      const long long nsl = p->nslices;
      const long long heavy = ((long long)multi.size() + kSlice - 1) / kSlice;
      std::vector<char> is_heavy(nsl, 0);
      for (long long h = 0; h < heavy; ++h)
        is_heavy[std::min(nsl - 1, (2 * h + 1) * nsl / (2 * heavy))] = 1;
      order.reserve(nv);
      size_t im = 0, is = 0;
      for (long long sl = 0; sl < nsl; ++sl) {
        const int cap = (int)std::min<long long>(kSlice, nv - sl * kSlice);
        for (int t = 0; t < cap; ++t) {
          const bool want_multi = is_heavy[sl] ? im < multi.size() : is >= single.size();
          order.push_back(want_multi ? multi[im++] : single[is++]);
        }
      }
    }
  }
  const bool ident = order.empty();
  std::vector<int> off(p->nslices + 1, 0);
  for (int sl = 0; sl < p->nslices; ++sl) {
    int w = 0;
    for (int q = sl * kSlice; q < std::min(nv, (sl + 1) * kSlice); ++q)
      w = std::max(w, p->h_len[ident ? q : order[q]]);
    off[sl + 1] = off[sl] + w;
  }
  const int slots = off[p->nslices];
  if (slots != p->slots || p->want64 != p->has64 || p->want32 != p->has32) {
    dfree(c, p->cols);
    dfree(c, p->cols16);
    dfree(c, p->v64);
    dfree(c, p->v32);
    int rc = dalloc(c, &p->cols, (size_t)slots * kSlice);
    if (!rc) rc = dalloc(c, &p->cols16, (size_t)slots * kSlice);
    if (!rc && p->want64) rc = dalloc(c, &p->v64, (size_t)slots * kSlice * 9);
    if (!rc && p->want32) rc = dalloc(c, &p->v32, (size_t)slots * kSlice * 9);
    if (rc) return rc;
    p->slots = slots;
    p->has64 = p->want64;
    p->has32 = p->want32;
  }
  int rc0 = upload(c, p->slice_off, off.data(), sizeof(int) * (p->nslices + 1), s);
  if (rc0) return rc0;
  if (ident) {
    dfree(c, p->rowmap);
  } else {
    if (!p->rowmap) {
      int rc = dalloc(c, &p->rowmap, nv);
      if (rc) return rc;
    }
    rc0 = upload(c, p->rowmap, order.data(), sizeof(int) * nv, s);
    if (rc0) return rc0;
  }
  CK(cudaMemsetAsync(p->c16ok, 1, sizeof(int), s));  // nonzero until an offset does not fit
  c->launches++;
  launch_bsr_to_sell(nv, p->stage_ptr, p->stage_cols, p->stage_vals, p->slice_off, p->rowmap,
                     p->cols, p->cols16, p->c16ok, p->v64, p->v32, p->dinv, p->bad, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "bsr_to_sell");
  p->layout = key;
  return MPRGP_OK;
}

int resolve_options(const mprgp_problem *p, const mprgp_options *o, int *kind, int *alg,
                    int *pre) {
  *kind = o->kind;
  if (*kind < MPRGP_KIND_LOWER || *kind > MPRGP_KIND_PLANES)
    return fail(MPRGP_INVALID, "unknown kind");
  if ((*kind >= MPRGP_KIND_DECOUPLED && p->cons != 1) ||
      (*kind == MPRGP_KIND_LOWER && p->cons < 2) || (*kind == MPRGP_KIND_BOX && p->cons != 3))
    return fail(MPRGP_INVALID, "constraints not set for this kind");
  // Façade defaults (MPRGPSolver.h:503-626): BoxBound uses plain MPRGP, the
  // others MPRGPMonotonic; DecoupledCon uses DiagonalDecouplePreconSolver,
  // the others DiagonalInFacePreconSolver.
  *alg = o->algorithm == MPRGP_ALG_DEFAULT
             ? (*kind == MPRGP_KIND_BOX ? ALG_PLAIN : ALG_MONOTONE)
             : (o->algorithm == MPRGP_ALG_PLAIN ? ALG_PLAIN : ALG_MONOTONE);
  if (o->algorithm < 0 || o->algorithm > MPRGP_ALG_PLAIN) return fail(MPRGP_INVALID, "algorithm");
  switch (o->precond) {
    case MPRGP_PRECOND_DEFAULT:
      *pre = *kind == MPRGP_KIND_DECOUPLED ? PRE_DECOUPLE : PRE_INFACE;
      break;
    case MPRGP_PRECOND_NONE: *pre = PRE_NONE; break;
    case MPRGP_PRECOND_INFACE: *pre = PRE_INFACE; break;
    case MPRGP_PRECOND_DECOUPLE:
      if (*kind != MPRGP_KIND_DECOUPLED && *kind != MPRGP_KIND_PLANES)
        return fail(MPRGP_INVALID, "DECOUPLE preconditioner needs plane constraints");
      *pre = PRE_DECOUPLE;
      break;
    default: return fail(MPRGP_INVALID, "precond");
  }
  if (o->precision == MPRGP_PREC_MIXED && (!p->has32 || !p->has64))
    return fail(MPRGP_INVALID, "mixed precision needs both FP64 and FP32 copies of A");
  if (o->precision == MPRGP_PREC_FP64 && !p->has64)
    return fail(MPRGP_INVALID, "FP64 solve needs the FP64 copy of A");
  if (o->precision != MPRGP_PREC_FP64 && o->precision != MPRGP_PREC_MIXED)
    return fail(MPRGP_INVALID, "precision");
  if (!(o->tol >= 0.0) || o->max_it < 0) return fail(MPRGP_INVALID, "tol/max_it");
  return MPRGP_OK;
}

// Prepares the desc and initial state of one instance.
int prepare(mprgp_problem *p, const mprgp_options *o, int item_begin, InstDesc *d,
            InstState *s) {
  int kind, alg, pre;
  int rc = resolve_options(p, o, &kind, &alg, &pre);
  if (rc) return rc;
  if (!p->b) return fail(MPRGP_INVALID, "rhs not set");
  if (!p->cols) return fail(MPRGP_INVALID, "matrix not set");
  cudaStream_t st = p->ctx->stream;
  if (p->cons == 1 && p->planes_dirty) {
    p->ctx->launches++;
    launch_planes_setup(p->nv, p->plane_ptr, p->planes_raw, p->planes, p->pl_nn, p->pl_indn,
                        p->dinv, p->pl_unit, st);
    CK(cudaGetLastError());
    if (p->m > 0) {
      p->ctx->launches++;
      launch_planes_axis(p->m, p->planes_raw, p->pl_axis, st);
      CK(cudaGetLastError());
    }
    p->planes_dirty = 0;
  }
  std::memset(d, 0, sizeof(*d));
  d->A.nslices = p->nslices;
  d->A.slice_off = p->slice_off;
  d->A.cols = p->cols;
  d->A.cols16 = p->cols16;
  d->A.c16ok = p->c16ok;
  d->A.v64 = p->v64;
  d->A.v32 = p->v32;
  d->A.rowmap = p->rowmap;
#ifdef MPRGP_CHECKS
  d->A.nv = p->nv;
  d->A.bad = p->bad;
#endif
  d->nv = p->nv;
  d->nitems = nitems_of(p->nv);
  d->item_begin = item_begin;
  d->m = p->m;
  d->kind = kind;
  d->alg = alg;
  d->pre = pre;
  d->prec = (alg == ALG_MONOTONE) ? o->precision : PREC_FP64;
  d->max_it = o->max_it;
  d->tol = o->tol < 1e-30 ? 1e-30 : o->tol;  // setParameters (MPRGPSolver.h:34-39)
  d->seed = o->seed;
  d->b = p->b;
  d->dinv = p->dinv;
  d->plane_ptr = p->plane_ptr;
  d->planes = p->planes;
  d->pl_nn = p->pl_nn;
  d->pl_indn = p->pl_indn;
  d->pl_unit = p->pl_unit;
  d->pl_axis = (p->cons == 1 && p->m > 0) ? p->pl_axis : nullptr;
  d->L = p->L;
  d->U = p->U;
  d->face = p->face;
  const size_t n = 3 * (size_t)p->nv;
  for (int i = 0; i < kNumBuf; ++i) d->buf[i] = p->vec + (size_t)i * n;
  for (int i = 0; i < kNumBuf32; ++i) d->buf32[i] = p->vec32 + (size_t)i * n;
  d->ev = p->ev;
  d->part = p->part;
  d->cnt = p->cnt;
  d->bad = p->bad;
  d->st = p->st;
  d->trace = p->trace;
  d->trace_cap = p->trace_cap;
  std::memset(s, 0, sizeof(*s));
  s->xc = p->xc;
  s->code = -1;
  s->ev_valid = (o->use_ev && p->ev_valid) ? 1 : 0;
  d->project_x0 = o->project_x0 ? 1 : 0;
  if (s->ev_valid) {
    s->phase = PH_POW;
    s->pow_src = -1;
    s->pow_scale = 1.0;
  } else {
    s->phase = PH_POW_RAND;
  }
  // Power phases use buffers that are otherwise idle until PH_INIT.
  return MPRGP_OK;
}

void fill_stats(const InstState &s, double ms, mprgp_stats *out) {
  if (!out) return;
  out->code = s.code;
  out->iterations = s.iters_out;
  out->num_cg = s.num_cg;
  out->num_exp = s.num_exp;
  out->num_prop = s.num_prop;
  out->power_iters = s.power_iters;
  out->active = s.active;
  out->ev_updated = s.ev_upd;
  out->residual = s.residual;
  out->alpha_bar = s.alpha_bar;
  out->spec_rad = s.spec_rad;
  out->spmv_fp64 = s.spmv64;
  out->spmv_fp32 = s.spmv32;
  out->phases = s.phases;
  out->device_ms = ms;
  out->power_passes = s.pow_spmv;
}

// Cluster-size class (log2 of the cluster size) of an instance of `items`
// items on the cluster solver, or -1 for the persistent engine.
int cluster_class(const mprgp_context *c, int items) {
  int largest = -1;
  for (int q = 0; q < kClusterClasses; ++q) {
    const int cs = 1 << q;
    if (cs > c->cluster) break;
    if (!c->cluster_ok[q]) continue;
    if (items <= cs) return q;  // one item per CTA
    largest = q;
  }
  if (largest >= 0 && items <= (1 << largest) * c->cluster_items) return largest;
  return -1;
}

// Grid of the power kernel over `items` items: every resident CTA, or the
// items rounded up to a multiple of 32 when that is fewer (few distinct sizes,
// so few cached graph instantiations).
int power_grid(mprgp_context *c, int items, int variant) {
  const int cap = std::max(1, c->nsm * c->bps_power_v[variant]);
  return std::min(cap, (items + 31) / 32 * 32);
}

// The instantiated loop graph of a lane for `grid` CTAs of a phase-kernel
// variant (0, 1: the power loop with the lane's d_pc; 2: the all-phase loop
// with its d_pc2).
int power_graph(Lane &L, int grid, int variant, cudaGraphExec_t *exec) {
  const int key = grid * 4 + variant;
  auto it = L.graphs.find(key);
  if (it == L.graphs.end()) {
    cudaGraph_t g;
    cudaGraphExec_t e;
    CK(build_power_graph(grid, variant, L.d_args, variant == 2 ? L.d_pc2 : L.d_pc, &g, &e));
    it = L.graphs.emplace(key, std::make_pair(g, e)).first;
  }
  *exec = it->second.second;
  return MPRGP_OK;
}

// Creates a lane's streams, events and control blocks on first use.
int lane_init(mprgp_context *c, int k) {
  Lane &L = c->lane[k];
  if (L.ready) return MPRGP_OK;
  if (k == 0) {
    L.stream = c->stream;
  } else {
    CK(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
    L.own_stream = true;
  }
  for (int q = 0; q < kClusterClasses; ++q) {
    CK(cudaStreamCreateWithFlags(&L.side[q], cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&L.join_ev[q], cudaEventDisableTiming));
  }
  CK(cudaEventCreateWithFlags(&L.fork_ev, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&L.fence, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&L.e_end, cudaEventDisableTiming));
  CK(cudaEventCreate(&L.e0));
  CK(cudaEventCreate(&L.e1));
  CK(cudaEventCreate(&L.e_pow));
  CK(cudaMallocHost((void **)&L.io, sizeof(HostIO)));
  std::memset(L.io, 0, sizeof(HostIO));
  int rc = dalloc(c, &L.ctl, 1);
  if (!rc) rc = dalloc(c, &L.d_args, 1);
  if (!rc) rc = dalloc(c, &L.d_pc, 1);
  if (!rc) rc = dalloc(c, &L.d_pc2, 1);
  if (rc) return rc;
  CK(cudaMemsetAsync(L.ctl, 0, sizeof(Ctl), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  L.ready = true;
  return MPRGP_OK;
}

void lane_free(mprgp_context *c, Lane &L) {
  if (!L.ready) return;
  if (L.stream) cudaStreamSynchronize(L.stream);
  for (int q = 0; q < kClusterClasses; ++q)
    if (L.side[q]) cudaStreamSynchronize(L.side[q]);
  dfree(c, L.ctl);
  dfree(c, L.d_args);
  dfree(c, L.d_pc);
  dfree(c, L.d_pc2);
  dfree(c, L.d_desc);
  dfree(c, L.d_prefix);
  dfree(c, L.d_st);
  dfree(c, L.d_fresh);
  dfree(c, L.d_home);
  dfree(c, L.d_item_inst);
  cudaStreamSynchronize(c->stream);
  cudaFreeHost(L.h_desc);
  cudaFreeHost(L.h_prefix);
  cudaFreeHost(L.h_st_in);
  cudaFreeHost(L.h_st_out);
  cudaFreeHost(L.h_fresh);
  cudaFreeHost(L.h_home);
  cudaFreeHost(L.h_item_inst);
  cudaFreeHost(L.io);
  for (auto &kv : L.graphs) {
    cudaGraphExecDestroy(kv.second.second);
    cudaGraphDestroy(kv.second.first);
  }
  L.graphs.clear();
  for (int q = 0; q < kClusterClasses; ++q) {
    if (L.side[q]) cudaStreamDestroy(L.side[q]);
    if (L.join_ev[q]) cudaEventDestroy(L.join_ev[q]);
  }
  cudaEventDestroy(L.fork_ev);
  cudaEventDestroy(L.fence);
  cudaEventDestroy(L.e_end);
  cudaEventDestroy(L.e0);
  cudaEventDestroy(L.e1);
  cudaEventDestroy(L.e_pow);
  if (L.own_stream) cudaStreamDestroy(L.stream);
  L = Lane();
}

// Grows a lane's per-run arrays to `n` instances and `items` items of large
// instances (the lane is idle).
int lane_reserve(mprgp_context *c, Lane &L, int n, int items) {
  if (items > L.icap) {
    const int icap = std::max(1024, std::max(items, 2 * L.icap));
    dfree(c, L.d_item_inst);
    cudaFreeHost(L.h_item_inst);
    L.h_item_inst = nullptr;
    L.icap = 0;
    int rc = dalloc(c, &L.d_item_inst, icap);
    if (rc) return rc;
    CK(cudaMallocHost((void **)&L.h_item_inst, sizeof(int) * icap));
    L.icap = icap;
  }
  if (n <= L.cap) return MPRGP_OK;
  const int cap = std::max(64, std::max(n, 2 * L.cap));
  dfree(c, L.d_desc);
  dfree(c, L.d_prefix);
  dfree(c, L.d_st);
  dfree(c, L.d_fresh);
  dfree(c, L.d_home);
  cudaFreeHost(L.h_desc);
  cudaFreeHost(L.h_prefix);
  cudaFreeHost(L.h_st_in);
  cudaFreeHost(L.h_st_out);
  cudaFreeHost(L.h_fresh);
  cudaFreeHost(L.h_home);
  L.h_desc = nullptr;
  L.h_prefix = L.h_fresh = nullptr;
  L.h_st_in = L.h_st_out = nullptr;
  L.h_home = nullptr;
  L.cap = 0;
  int rc = dalloc(c, &L.d_desc, cap);
  if (!rc) rc = dalloc(c, &L.d_prefix, cap + 1);
  // the run's states, then the power-step loop's two copies
  if (!rc) rc = dalloc(c, &L.d_st, 3 * (size_t)cap);
  if (!rc) rc = dalloc(c, &L.d_fresh, cap);
  if (!rc) rc = dalloc(c, &L.d_home, cap);
  if (rc) return rc;
  CK(cudaMallocHost((void **)&L.h_desc, sizeof(InstDesc) * cap));
  CK(cudaMallocHost((void **)&L.h_prefix, sizeof(int) * (cap + 1)));
  CK(cudaMallocHost((void **)&L.h_st_in, sizeof(InstState) * cap));
  CK(cudaMallocHost((void **)&L.h_st_out, sizeof(InstState) * cap));
  CK(cudaMallocHost((void **)&L.h_fresh, sizeof(int) * cap));
  CK(cudaMallocHost((void **)&L.h_home, sizeof(InstState *) * cap));
  L.cap = cap;
  return MPRGP_OK;
}

bool other_lanes_active(const mprgp_context *c, int k) {
  for (int j = 0; j < kLanes; ++j)
    if (j != k && c->lane[j].run.active) return true;
  return false;
}

}  // namespace

namespace mprgp {

// Device bytes a new allocation of the context can use now: the device's
// free memory plus what the context's pool holds reserved but unused (the
// pool keeps freed blocks for reuse instead of returning them).
int context_room(mprgp_context *c, size_t *room) {
  size_t fr = 0, tot = 0;
  cudaError_t e = cudaMemGetInfo(&fr, &tot);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemGetInfo");
  unsigned long long reserved = 0, used = 0;  // the pool attributes are 64-bit
  e = cudaMemPoolGetAttribute(c->pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
  if (e == cudaSuccess) e = cudaMemPoolGetAttribute(c->pool, cudaMemPoolAttrUsedMemCurrent, &used);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemPoolGetAttribute");
  *room = fr + (size_t)(reserved > used ? reserved - used : 0);
  return MPRGP_OK;
}

// Whether any asynchronous lane of the context has a run in flight.
int context_lanes_busy(const mprgp_context *c) {
  return other_lanes_active(c, 0) ? 1 : 0;
}

// Lane (1: small, 2: large) that the server's asynchronous form gives an
// instance of `nv` vertices: small ones are those of the cluster solver.
int engine_lane_of(const mprgp_context *c, int nv) {
  return cluster_class(c, nitems_of(nv)) >= 0 ? 1 : 2;
}

// Whether a solve of `p` started now with options `o` begins with the power
// method (it does unless the exact power-method cache applies).
int engine_needs_power(const mprgp_problem *p, const mprgp_options *o) {
  int kind, alg, pre;
  if (resolve_options(p, o, &kind, &alg, &pre)) return 1;
  const int prec = (alg == ALG_MONOTONE) ? o->precision : PREC_FP64;
  if (o->use_ev && p->ev_valid) {  // warm-started power method
    const bool cached = p->pcache_on && p->pcache_ev.valid && p->pcache_ev.prec == prec &&
                        p->pcache_ev.gen == p->matrix_gen && p->pcache_ev.ev_gen == p->ev_gen;
    return cached ? 0 : 1;
  }
  const bool cached = p->pcache_on && p->pcache.valid && p->pcache.seed == o->seed &&
                      p->pcache.prec == prec && p->pcache.gen == p->matrix_gen;
  return cached ? 0 : 1;
}

// Whether `p` was left in a power-method phase by its last engine run.
int engine_in_power(const mprgp_problem *p) {
  const int ph = p->phase_host;
  return ph == PH_POW_RAND || ph == PH_POW || ph == PH_POW_LAST;
}

// Starts one engine run over `n` problems on lane `k` and returns without
// waiting for it.  Instances with fresh[i] != 0 start a solve (their initial
// state is uploaded); the others resume from the state left in device memory
// by the previous run.  The run advances the large instances by at most
// `quantum` macro-phases (0: until all are done; < 0: none, the run is the
// power loop alone) after up to `power_launches` launches of the power
// kernel, and the small ones (cluster solver) by at most `cluster_quantum`
// phases (0: until done).  The problems must stay untouched until
// engine_end.
int engine_begin(mprgp_context *c, int k, int n, mprgp_problem *const *probs,
                 const mprgp_options *opts, const int *fresh, int quantum, int power_launches,
                 int cluster_quantum) {
  if (k < 0 || k >= kLanes || n <= 0) return fail(MPRGP_INVALID, "engine_begin");
  int rc = lane_init(c, k);
  if (rc) return rc;
  Lane &L = c->lane[k];
  if (L.run.active) return fail(MPRGP_INVALID, "engine lane busy");
  // Small instances run on the cluster solver, one cluster each, grouped by
  // cluster size (the smallest usable size that gives every CTA its items);
  // the others on the power loop and the engine.  The desc array holds the
  // large instances first, then each cluster-size class.
  LaneRun &R = L.run;
  R.probs.assign(probs, probs + n);
  R.opts.assign(opts, opts + n);
  R.pos.assign(n, 0);
  std::vector<int> cls(n);
  int n_large = 0, large_items = 0;
  for (int q = 0; q < kClusterClasses; ++q) R.class_n[q] = 0;
  for (int i = 0; i < n; ++i) {
    mprgp_problem *p = probs[i];
    if (!p || p->ctx != c) return fail(MPRGP_INVALID, "problem/context mismatch");
    cls[i] = cluster_class(c, nitems_of(p->nv));
    if (cls[i] < 0) {
      R.pos[i] = n_large++;
      large_items += nitems_of(p->nv);
    } else {
      R.class_n[cls[i]]++;
    }
  }
  rc = lane_reserve(c, L, n, large_items);
  if (rc) return rc;
  int class_off[kClusterClasses];
  {
    int f = n_large;
    for (int q = 0; q < kClusterClasses; ++q) {
      class_off[q] = f;
      f += R.class_n[q];
    }
    int fill[kClusterClasses];
    for (int q = 0; q < kClusterClasses; ++q) fill[q] = class_off[q];
    for (int i = 0; i < n; ++i)
      if (cls[i] >= 0) R.pos[i] = fill[cls[i]]++;
  }
  InstDesc *desc = L.h_desc;
  InstState *st = L.h_st_in;  // desc order
  int *prefix = L.h_prefix;
  prefix[0] = 0;
  for (int i = 0; i < n; ++i)
    if (R.pos[i] < n_large) prefix[R.pos[i] + 1] = nitems_of(probs[i]->nv);
  for (int j = 0; j < n_large; ++j) prefix[j + 1] += prefix[j];
  double wait_s = 0.0;
  long long phase_bound = 0;
  for (int i = 0; i < n; ++i) {
    mprgp_problem *p = probs[i];
    const int j = R.pos[i];
    rc = prepare(p, &opts[i], j < n_large ? prefix[j] : 0, &desc[j], &st[j]);
    if (rc) return rc;
    desc[j].st = L.d_st + j;  // the run's state array
    L.h_home[j] = p->st;
    L.h_fresh[j] = fresh[i] ? 1 : 0;
    wait_s = std::max(wait_s, opts[i].wait_limit_s);
    // Each MPRGP iteration takes at most 4 phases (CG: spmv, candidate,
    // optional delta^T A delta and residual replacement; expansion 3;
    // proportioning 2); the power method at most 1003.
    phase_bound = std::max(phase_bound, 1100LL + 8LL * ((long long)opts[i].max_it + 2));
  }
  if (wait_s <= 0.0) wait_s = 5.0;
  {
    // The large instances' matrix bytes per pass (FP32 values in the mixed
    // form): beyond three quarters of L2 the run streams them evict-first.
    // So do a server's large-instance lanes (k >= 2) whatever their size:
    // they share L2 with the small-instance lane, whose short phases reuse
    // their matrices far more often (serving stream: 1316-1325 solves/s with
    // the size rule alone, 1348-1352 with this one).
    size_t mbytes = 0;
    for (int i = 0; i < n; ++i)
      if (R.pos[i] < n_large)
        mbytes += (size_t)probs[i]->slots * kSlice *
                  (9 * (desc[R.pos[i]].prec == PREC_MIXED ? 4 : 8) + (probs[i]->cols16 ? 2 : 4));
    const int stream_l2 = (k >= 2 || mbytes > c->l2_bytes / 4 * 3) ? 1 : 0;
    for (int j = 0; j < n_large; ++j) desc[j].A.stream_l2 = stream_l2;
  }
  for (int i = 0; i < n; ++i) {
    if (!fresh[i]) continue;
    mprgp_problem *p = probs[i];
    InstState &S = st[R.pos[i]];
    const InstDesc &D = desc[R.pos[i]];
    p->phase_host = S.phase;
    p->run_random = S.phase == PH_POW_RAND;
    p->run_ev = S.phase == PH_POW && S.pow_src < 0;
    p->run_ev_gen = p->ev_gen;
    p->run_cached = 0;
    const bool hit_random = p->run_random && p->pcache_on && p->pcache.valid &&
                            p->pcache.seed == opts[i].seed && p->pcache.prec == D.prec &&
                            p->pcache.gen == p->matrix_gen;
    const bool hit_ev = p->run_ev && p->pcache_on && p->pcache_ev.valid &&
                        p->pcache_ev.prec == D.prec && p->pcache_ev.gen == p->matrix_gen &&
                        p->pcache_ev.ev_gen == p->ev_gen;
    if (hit_random || hit_ev) {
      // the state advance_power leaves when the power method ends
      S.spec_rad = hit_ev ? p->pcache_ev.spec_rad : p->pcache.spec_rad;
      S.power_iters = hit_ev ? p->pcache_ev.power_iters : p->pcache.power_iters;
      S.alpha_bar = 2.0 / S.spec_rad;
      // random start: the vector it would store is the one already stored;
      // start from ev: the cached run stored none
      S.ev_upd = 0;
      S.phase = D.project_x0 ? PH_PROJ0 : PH_INIT;
      p->run_cached = 1;
      p->phase_host = S.phase;
    }
  }
  unsigned int in_power = 0;  // large instances in a power phase
  for (int i = 0; i < n; ++i) {
    const int ph = probs[i]->phase_host;
    if (R.pos[i] < n_large)
      in_power += (ph == PH_POW_RAND || ph == PH_POW || ph == PH_POW_LAST) ? 1u : 0u;
  }
  cudaStream_t s = L.stream;
  if (s != c->stream) {  // the problems' uploads and setup kernels come first
    CK(cudaEventRecord(L.fence, c->stream));
    CK(cudaStreamWaitEvent(s, L.fence, 0));
  }
  CK(cudaMemcpyAsync(L.d_desc, desc, sizeof(InstDesc) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(L.d_prefix, prefix, sizeof(int) * (n_large + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(L.d_st, st, sizeof(InstState) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(L.d_fresh, L.h_fresh, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(L.d_home, L.h_home, sizeof(InstState *) * n, cudaMemcpyHostToDevice, s));
  for (int j = 0; j < n_large; ++j)
    for (int t = prefix[j]; t < prefix[j + 1]; ++t) L.h_item_inst[t] = j;
  if (large_items > 0)
    CK(cudaMemcpyAsync(L.d_item_inst, L.h_item_inst, sizeof(int) * large_items,
                       cudaMemcpyHostToDevice, s));
  launch_state_scatter(L.d_desc, n, L.d_st, L.d_home, L.d_fresh, s);
  CK(cudaGetLastError());
  HostIO &io = *L.io;
  std::memset(&io.ctl_in, 0, sizeof(Ctl));
  io.ctl_in.active = n_large;
  io.ctl_in.snap[0] = io.ctl_in.snap[1] = n_large;
  CK(cudaMemcpyAsync(L.ctl, &io.ctl_in, sizeof(Ctl), cudaMemcpyHostToDevice, s));
  EngineArgs &args = io.args;
  std::memset(&args, 0, sizeof(args));
  args.desc = L.d_desc;
  args.item_prefix = L.d_prefix;
  args.item_inst = L.d_item_inst;
  args.states = L.d_st;
  args.ninst = n_large;
  args.total_items = prefix[n_large];
  long long maxp = phase_bound;
  if (quantum > 0) maxp = std::min<long long>(maxp, quantum);
  args.max_phases = (int)std::min<long long>(maxp, INT_MAX);
  args.wait_ns = (long long)(wait_s * 1e9);
  args.total_ns = (long long)(std::max(60.0, 20.0 * wait_s) * 1e9);
  const bool stage = c->stage && c->bps_stage > 0;
  args.stage_bytes = stage ? kStageBytes : 0;
  args.ctl = L.ctl;
  args.pst[0] = L.d_st + L.cap;
  args.pst[1] = L.d_st + 2 * (size_t)L.cap;
  int per_sm = stage ? c->bps_stage : c->bps;
  if (c->ctas_per_sm > 0) per_sm = std::min(per_sm, c->ctas_per_sm);
  // Equally many items per CTA: a phase ends with its busiest CTA, so the
  // grid is the fewest CTAs that give each the same count (c3's 1,360 items:
  // 454 CTAs of 3, not 608 of 2 or 3).
  const int e_cap = std::max(1, c->nsm * per_sm);
  const int e_per = std::max(1, (prefix[n_large] + e_cap - 1) / e_cap);
  const int grid = std::max(1, (prefix[n_large] + e_per - 1) / e_per);

  // The power method first (at most 1003 phases: the seeded start, 1001
  // iterations, the last difference), as a device-driven loop of launches of
  // the power kernel while any instance is in a power phase; then the engine.
  R.power = c->power_kernel && in_power > 0 && power_launches > 0;
  cudaGraphExec_t pexec = nullptr;
  R.power_variant = c->power_step ? 3 : c->power_variant;
  const int pgrid = power_grid(c, prefix[n_large], R.power_variant);
  // ... or as one persistent cooperative launch: only on lane 0 with no other
  // lane in flight (its CTAs must all be resident) and when every CTA holds
  // at most kPowOwn items
  const int pp_cap = c->nsm * c->bps_power_pp;
  R.power_persistent = R.power && c->power_persistent && k == 0 && !other_lanes_active(c, k) &&
                       pp_cap > 0 && prefix[n_large] <= pp_cap * kPowOwn;
  // equally many items per CTA (the phase waits for the busiest CTA)
  const int pp_per = pp_cap > 0 ? (prefix[n_large] + pp_cap - 1) / pp_cap : 1;
  const int pp_grid = std::max(1, (prefix[n_large] + pp_per - 1) / std::max(1, pp_per));
  if (R.power) {
    if (c->power_graph && !R.power_persistent) {
      rc = power_graph(L, pgrid, R.power_variant, &pexec);
      if (rc) return rc;
    }
    io.pc_in[0] = {in_power, 0u, 0u, 0u, (unsigned int)power_launches, 0u};
    CK(cudaMemcpyAsync(L.d_pc, &io.pc_in[0], sizeof(PowCtl), cudaMemcpyHostToDevice, s));
  }
  R.power_graph = pexec != nullptr;
  // The large instances' remaining phases: the persistent cooperative engine,
  // or the same phases as a graph loop of the all-phase kernel -- always the
  // latter while another lane has a run in flight, since a cooperative launch
  // needs every one of its CTAs resident at once.
  R.egraph = n_large > 0 && quantum >= 0 &&
             (c->engine_graph || k != 0 || other_lanes_active(c, k));
  cudaGraphExec_t eexec = nullptr;
  const int egrid = power_grid(c, prefix[n_large], 2);
  // Stream form of that loop (with the power loop's stream form, for
  // profilers that cannot see kernels inside conditional graphs): one launch
  // per phase of the quantum, those after the last working one return at once.
  R.egraph_stream = (R.egraph && !c->power_graph && quantum > 0) ? args.max_phases : 0;
  if (R.egraph && !R.egraph_stream) {
    rc = power_graph(L, egrid, 2, &eexec);
    if (rc) return rc;
  }
  if (R.egraph) {
    io.pc_in[1] = {(unsigned int)n_large, 0u, 0u, 0u, (unsigned int)args.max_phases, 0u};
    CK(cudaMemcpyAsync(L.d_pc2, &io.pc_in[1], sizeof(PowCtl), cudaMemcpyHostToDevice, s));
  }
  if (R.power || R.egraph)
    CK(cudaMemcpyAsync(L.d_args, &args, sizeof(EngineArgs), cudaMemcpyHostToDevice, s));
  CK(cudaEventRecord(L.e0, s));
  // The cluster-size classes run on side streams, concurrently with each
  // other and with the power loop; the engine starts once they are done.
  if (n - n_large > 0) CK(cudaEventRecord(L.fork_ev, s));
  for (int q = 0; q < kClusterClasses; ++q) {
    if (!R.class_n[q]) continue;
    ClusterArgs cargs;
    cargs.desc = L.d_desc + class_off[q];
    cargs.ninst = R.class_n[q];
    cargs.max_phases = (int)std::min<long long>(
        cluster_quantum > 0 ? std::min<long long>(phase_bound, cluster_quantum) : phase_bound,
        INT_MAX);
    CK(cudaStreamWaitEvent(L.side[q], L.fork_ev, 0));
    CK(launch_cluster(cargs, 1 << q, L.side[q]));
    CK(cudaEventRecord(L.join_ev[q], L.side[q]));
  }
  if (R.power && R.power_persistent)
    CK(launch_power_persistent(args, L.d_pc, power_launches, pp_grid, s));
  else if (R.power && pexec) CK(cudaGraphLaunch(pexec, s));
  else if (R.power)
    CK(launch_power_direct(pgrid, R.power_variant, power_launches, L.d_args, L.d_pc, s));
  CK(cudaEventRecord(L.e_pow, s));  // the lane stream's power loop ends here
  for (int q = 0; q < kClusterClasses; ++q)
    if (R.class_n[q]) CK(cudaStreamWaitEvent(s, L.join_ev[q], 0));
  if (R.egraph && R.egraph_stream)
    CK(launch_power_direct(egrid, 2, R.egraph_stream, L.d_args, L.d_pc2, s));
  else if (R.egraph) CK(cudaGraphLaunch(eexec, s));
  else if (n_large > 0 && quantum >= 0) CK(launch_engine(args, grid, s));
  CK(cudaEventRecord(L.e1, s));
  if (R.power) CK(cudaMemcpyAsync(&io.pc_out[0], L.d_pc, sizeof(PowCtl), cudaMemcpyDeviceToHost, s));
  if (R.egraph) CK(cudaMemcpyAsync(&io.pc_out[1], L.d_pc2, sizeof(PowCtl), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&io.ctl_out, L.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
  launch_state_gather(L.d_desc, n, L.d_st, L.d_home, s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(L.h_st_out, L.d_st, sizeof(InstState) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(L.e_end, s));
  R.n = n;
  R.n_large = n_large;
  R.quantum = quantum;
  R.cluster_quantum = cluster_quantum;
  R.power_launches = power_launches;
  R.active = true;
  static const char *kRunNames[kLanes] = {"mprgp run", "mprgp lane small", "mprgp lane large",
                                          "mprgp lane power", "mprgp lane power",
                                          "mprgp lane power", "mprgp lane power"};
  L.nvtx = nvtx_start(kRunNames[k]);
  return MPRGP_OK;
}

// Copies a problem's solution (3 nv doubles) and face codes into host
// memory after an engine run that used it has ended (engine_end), on the
// read stream: unlike mprgp_problem_get_x, it does not wait for uploads and
// setup kernels queued on the context stream for other problems meanwhile.
int problem_read_result(mprgp_problem *p, double *x, unsigned char *face) {
  mprgp_context *c = p->ctx;
  const size_t n = 3 * (size_t)p->nv;
  CK(cudaMemcpyAsync(x, p->vec + (size_t)(B_X0 + p->xc) * n, sizeof(double) * n,
                     cudaMemcpyDeviceToHost, c->io));
  if (face && p->face_len > 0)
    CK(cudaMemcpyAsync(face, p->face, p->face_len, cudaMemcpyDeviceToHost, c->io));
  CK(cudaStreamSynchronize(c->io));
  return MPRGP_OK;
}

// Whether lane k's run has finished (1), is still in flight (0), or the lane
// has no run (-1).
int engine_ready(mprgp_context *c, int k) {
  if (k < 0 || k >= kLanes || !c->lane[k].run.active) return -1;
  const cudaError_t e = cudaEventQuery(c->lane[k].e_end);
  if (e == cudaErrorNotReady) return 0;
  return 1;  // finished, or failed: engine_end reports which
}

// Waits for lane k's run and takes its results: done[i] reports instances
// that finished (or failed); stats are filled for every instance.
int engine_end(mprgp_context *c, int k, mprgp_stats *stats, int *done) {
  if (k < 0 || k >= kLanes || !c->lane[k].run.active) return fail(MPRGP_INVALID, "engine_end");
  Lane &L = c->lane[k];
  LaneRun &R = L.run;
  R.active = false;
  nvtx_end(L.nvtx);
  L.nvtx = 0;
  const int n = R.n, n_large = R.n_large;
  CK(cudaEventSynchronize(L.e_end));
  const HostIO &io = *L.io;
  float ms = 0.f, pms = 0.f;
  CK(cudaEventElapsedTime(&ms, L.e0, L.e1));
  if (R.power) CK(cudaEventElapsedTime(&pms, L.e0, L.e_pow));
  c->power_ms += pms;
  // every body of a loop graph issues kPowerUnroll launches, the stream form
  // all `power_launches` (those after the last working one return at once)
  // (the power-step loop adds its settle kernel to every body)
  const long long body = kPowerUnroll + (R.power_variant == 3 ? 1 : 0);
  if (R.power && R.power_persistent)
    c->launches += 1;
  else if (R.power && R.power_graph)
    c->launches += body * ((io.pc_out[0].launches + kPowerUnroll - 1) / kPowerUnroll);
  else if (R.power && R.power_variant == 3)
    c->launches += body * ((R.power_launches + kPowerUnroll - 1) / kPowerUnroll);
  else if (R.power)
    c->launches += R.power_launches;
  for (int q = 0; q < kClusterClasses; ++q) c->launches += R.class_n[q] ? 1 : 0;
  if (R.egraph && R.egraph_stream)
    c->launches += R.egraph_stream;
  else if (R.egraph)
    c->launches += (long long)kPowerUnroll * ((io.pc_out[1].launches + kPowerUnroll - 1) / kPowerUnroll);
  else
    c->launches += (n_large > 0 && R.quantum >= 0) ? 1 : 0;
  c->launches += 2;  // state scatter and gather
  c->solver_ms += ms;
  const Ctl &ctl1 = io.ctl_out;
  int worst = MPRGP_OK;
  for (int i = 0; i < n; ++i) {
    mprgp_problem *p = R.probs[i];
    InstState x = L.h_st_out[R.pos[i]];
    p->phase_host = x.phase;
    const bool finished = x.phase == PH_DONE;
    const bool large = R.pos[i] < n_large;
    // an engine error concerns the engine's instances; an instance left
    // unfinished by a run that had no phase limit hit the hard phase bound
    const bool err = large && ctl1.err;
    const bool unbounded = (large ? R.quantum : R.cluster_quantum) == 0;
    if (err) x.code = ctl1.err;
    else if (!finished && unbounded) x.code = MPRGP_TIMEOUT;
    p->xc = x.xc;
    p->trace_n = x.trace_n;
    if (x.ev_upd) p->ev_gen++;  // PH_INIT has stored, or will store, a new ev
    if (finished && x.ev_upd && x.code > MPRGP_BREAKDOWN) p->ev_valid = 1;
    if (finished && !err && p->run_ev && !p->run_cached && !x.ev_upd &&
        p->ev_gen == p->run_ev_gen) {
      auto &pc = p->pcache_ev;
      pc.valid = 1;
      pc.prec = L.h_desc[R.pos[i]].prec;
      pc.gen = p->matrix_gen;
      pc.ev_gen = p->ev_gen;
      pc.spec_rad = x.spec_rad;
      pc.power_iters = x.power_iters;
    }
    if (finished && !err && p->run_random && !p->run_cached) {
      auto &pc = p->pcache;
      pc.valid = 1;
      pc.seed = R.opts[i].seed;
      pc.prec = L.h_desc[R.pos[i]].prec;
      pc.gen = p->matrix_gen;
      pc.spec_rad = x.spec_rad;
      pc.power_iters = x.power_iters;
    }
    fill_stats(x, ms, stats ? &stats[i] : nullptr);
    if (done) done[i] = finished || err || (!finished && unbounded);
    if ((finished || err || unbounded) && x.code < worst) worst = x.code;
  }
  if (ctl1.err) return fail(ctl1.err, "device wait limit reached");
  return worst < MPRGP_NOT_CONVERGED ? worst : MPRGP_OK;
}

// One engine run on lane 0 (the context stream), waited for.
int engine_run(mprgp_context *c, int n, mprgp_problem *const *probs, const mprgp_options *opts,
               const int *fresh, int quantum, int power_launches, int cluster_quantum,
               mprgp_stats *stats, int *done) {
  int rc = engine_begin(c, 0, n, probs, opts, fresh, quantum, power_launches, cluster_quantum);
  if (rc) {
    c->lane[0].run.active = false;
    return rc;
  }
  return engine_end(c, 0, stats, done);
}

}  // namespace mprgp

namespace {

// Launches the engine over `n` prepared instances until all are done.
int run_engine(mprgp_context *c, int n, mprgp_problem *const *probs, const mprgp_options *opts,
               mprgp_stats *stats) {
  NvtxScope range("mprgp solve");
  std::vector<int> fresh(n, 1);
  return mprgp::engine_run(c, n, probs, opts, fresh.data(), 0, 1003, 0, stats, nullptr);
}

}  // namespace

namespace mprgp {
// Lets other translation units of the library report through mprgp_last_error().
void set_last_error(const char *what) { g_last_error = what; }
}  // namespace mprgp

extern "C" {

int mprgp_version(void) { return 10000; }

const char *mprgp_status_string(int s) {
  switch (s) {
    case MPRGP_OK: return "ok";
    case MPRGP_NOT_CONVERGED: return "not converged";
    case MPRGP_BREAKDOWN: return "breakdown";
    case MPRGP_OOM: return "out of device memory";
    case MPRGP_TIMEOUT: return "device wait limit reached";
    case MPRGP_INVALID: return "invalid argument";
    case MPRGP_CUDA_ERROR: return "CUDA error";
    case MPRGP_NO_DEVICE: return "no CUDA device";
    case MPRGP_BUSY: return "busy";
    default: return "unknown status";
  }
}

const char *mprgp_last_error(void) { return g_last_error.c_str(); }

void mprgp_default_options(mprgp_options *o) {
  std::memset(o, 0, sizeof(*o));
  o->tol = 1e-3;  // MPRGPDecoupledCon::solve defaults (MPRGPSolver.h:546)
  o->max_it = 1000;
  o->kind = MPRGP_KIND_DECOUPLED;
  o->algorithm = MPRGP_ALG_DEFAULT;
  o->precond = MPRGP_PRECOND_DEFAULT;
  o->precision = MPRGP_PREC_FP64;
  o->project_x0 = 0;
  o->use_ev = 0;
  o->seed = 0x5eedULL;
  o->wait_limit_s = 5.0;
}

int mprgp_device_count(int *count) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (count) *count = (e == cudaSuccess) ? n : 0;
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
  return MPRGP_OK;
}

int mprgp_context_create(int device, mprgp_context **out) {
  if (!out) return fail(MPRGP_INVALID, "out");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(MPRGP_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= n) return fail(MPRGP_INVALID, "device");
  CK(cudaSetDevice(device));
  int coop = 0;
  CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
  if (!coop) return fail(MPRGP_NO_DEVICE, "device lacks cooperative launch");
  auto *c = new mprgp_context();
  c->device = device;
  CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device));
  {
    int l2 = 0;
    CK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device));
    c->l2_bytes = (size_t)l2;
  }
  CK(engine_max_blocks_per_sm(&c->bps, 0));
  CK(engine_max_blocks_per_sm(&c->bps_stage, kStageBytes));
  if (c->bps < 1) {
    delete c;
    return fail(MPRGP_NO_DEVICE, "engine kernel cannot be resident");
  }
  {
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, greatest));
  }
  CK(cudaStreamCreateWithFlags(&c->io, cudaStreamNonBlocking));
  cudaMemPoolProps props;
  std::memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  CK(cudaMemPoolCreate(&c->pool, &props));
  unsigned long long keep = ~0ULL;  // never trim: freed blocks serve the next problem
  CK(cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  CK(power_max_blocks_per_sm(0, &c->bps_power_v[0]));
  CK(power_max_blocks_per_sm(1, &c->bps_power_v[1]));
  CK(power_max_blocks_per_sm(2, &c->bps_power_v[2]));
  CK(power_max_blocks_per_sm(3, &c->bps_power_v[3]));
  CK(power_persistent_max_blocks_per_sm(&c->bps_power_pp));
  c->bps_power = c->bps_power_v[0];
  {
    int largest = 0;
    for (int q = 0; q < kClusterClasses; ++q) {
      int nc = 0;
      c->cluster_ok[q] = cluster_max_active(1 << q, &nc) == cudaSuccess && nc >= 1;
      cudaGetLastError();
      if (c->cluster_ok[q]) largest = 1 << q;
    }
    c->cluster = std::min(c->cluster, largest);
  }
  int rc = lane_init(c, 0);
  if (rc) return rc;
  *out = c;
  return MPRGP_OK;
}

int mprgp_context_destroy(mprgp_context *c) {
  if (!c) return MPRGP_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->scratch) mprgp_problem_destroy(c->scratch);
  for (int k = kLanes - 1; k >= 0; --k) lane_free(c, c->lane[k]);
  cudaStreamSynchronize(c->stream);
  for (auto &u : c->ring.uses) cudaEventDestroy(u.ev);
  for (auto ev : c->ring.spare) cudaEventDestroy(ev);
  if (c->ring.base) cudaFreeHost(c->ring.base);
  cudaStreamDestroy(c->stream);
  if (c->io) cudaStreamDestroy(c->io);
  if (c->pool) cudaMemPoolDestroy(c->pool);
  delete c;
  return MPRGP_OK;
}

void *mprgp_context_stream(mprgp_context *c) { return c ? (void *)c->stream : nullptr; }

int mprgp_context_sync(mprgp_context *c) {
  if (!c) return fail(MPRGP_INVALID, "ctx");
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 1; k < kLanes; ++k)
    if (c->lane[k].ready) CK(cudaStreamSynchronize(c->lane[k].stream));
  return MPRGP_OK;
}

int mprgp_context_set_tuning(mprgp_context *c, int stage, int ctas_per_sm) {
  if (!c || stage < 0 || stage > 127 || ctas_per_sm < 0) return fail(MPRGP_INVALID, "set_tuning");
  c->power_kernel = (stage & 2) ? 0 : 1;
  c->power_graph = (stage & 4) ? 0 : 1;
  c->power_variant = (stage & 8) ? 1 : 0;
  c->engine_graph = (stage & 16) ? 1 : 0;
  c->power_persistent = (stage & 32) ? 1 : 0;
  c->power_step = (stage & 64) ? 0 : 1;
  c->bps_power = c->bps_power_v[c->power_variant];
  stage &= 1;
  c->stage = stage;
  c->ctas_per_sm = ctas_per_sm;
  return MPRGP_OK;
}

int mprgp_context_counters(mprgp_context *c, long long *launches, double *solver_ms,
                           double *power_ms) {
  if (!c) return fail(MPRGP_INVALID, "context_counters");
  if (launches) *launches = c->launches;
  if (solver_ms) *solver_ms = c->solver_ms;
  if (power_ms) *power_ms = c->power_ms;
  return MPRGP_OK;
}

int mprgp_context_set_cluster(mprgp_context *c, int cluster) {
  if (!c || cluster < 0 || cluster > kClusterMax || (cluster & (cluster - 1)))
    return fail(MPRGP_INVALID, "set_cluster: 0 or a power of two up to 16");
  if (cluster > 0) {
    int q = 0;
    while ((1 << q) < cluster) ++q;
    if (!c->cluster_ok[q]) return fail(MPRGP_INVALID, "set_cluster: size not available");
  }
  c->cluster = cluster;
  return MPRGP_OK;
}

int mprgp_context_set_cluster_items(mprgp_context *c, int items) {
  if (!c || items < 1 || items > kClusterItems)
    return fail(MPRGP_INVALID, "set_cluster_items: 1..4");
  c->cluster_items = items;
  return MPRGP_OK;
}

int mprgp_context_info(mprgp_context *c, int *nsm, int *blocks_per_sm) {
  if (!c) return fail(MPRGP_INVALID, "ctx");
  if (nsm) *nsm = c->nsm;
  if (blocks_per_sm) *blocks_per_sm = c->bps;
  return MPRGP_OK;
}

int mprgp_context_room(mprgp_context *c, size_t *bytes) {
  if (!c || !bytes) return fail(MPRGP_INVALID, "context_room");
  return mprgp::context_room(c, bytes);
}

size_t mprgp_problem_bytes(int nv, int nnzb, int nplanes, int precisions) {
  const size_t nsl = (size_t)(nv + kSlice - 1) / kSlice;
  // SELL slots of 32 rows: the blocks plus a padding allowance of 8 slots a slice
  const size_t slots = ((size_t)nnzb + kSlice - 1) / kSlice + nsl * 8;
  size_t by = (nsl + 1) * 4 + slots * kSlice * (4 + 2);  // 32- and 16-bit columns
  if (precisions & 1) by += slots * kSlice * 9 * 8;
  if (precisions & 2) by += slots * kSlice * 9 * 4;
  const size_t n = 3 * (size_t)nv;
  by += n * 8 * (kNumBuf + 3) + n * 4 * kNumBuf32;  // vectors, dinv, b, ev, FP32 shadows
  by += (size_t)nplanes * (8 * 4 * 2 + 8 * 2 + 2) + (size_t)(nv + 1) * 4 + n * 16 + n;
  by += (size_t)nitems_of(nv) * kPart * 8 * 2 + sizeof(InstState) + 64;
  by += (size_t)nnzb * (9 * 8 + 4) + (size_t)(nv + 1) * 4 + (size_t)nv * 4;  // BSR copy, rowmap
  return by;
}

int mprgp_problem_create(mprgp_context *c, int nv, mprgp_problem **out) {
  if (!c || !out || nv <= 0) return fail(MPRGP_INVALID, "problem_create");
  *out = nullptr;
  CK(cudaSetDevice(c->device));
  auto *p = new mprgp_problem();
  p->ctx = c;
  p->nv = nv;
  p->nslices = (nv + kSlice - 1) / kSlice;
  const size_t n = 3 * (size_t)nv;
  int rc = 0;
  if ((rc = dalloc(p->ctx, &p->vec, n * kNumBuf)) || (rc = dalloc(p->ctx, &p->vec32, n * kNumBuf32)) ||
      (rc = dalloc(p->ctx, &p->ev, n)) ||
      (rc = dalloc(p->ctx, &p->b, n)) || (rc = dalloc(p->ctx, &p->dinv, n)) ||
      (rc = dalloc(p->ctx, &p->part, (size_t)nitems_of(nv) * kPart * 2)) || (rc = dalloc(p->ctx, &p->cnt, 1)) || (rc = dalloc(p->ctx, &p->bad, 1)) || (rc = dalloc(p->ctx, &p->c16ok, 1)) ||
      (rc = dalloc(p->ctx, &p->st, 1)) || (rc = dalloc(p->ctx, &p->slice_off, p->nslices + 1))) {
    free_problem_arrays(p);
    delete p;
    return rc;
  }
  cudaMemsetAsync(p->vec, 0, n * kNumBuf * sizeof(double), c->stream);
  *out = p;
  return MPRGP_OK;
}

int mprgp_problem_destroy(mprgp_problem *p) {
  if (!p) return MPRGP_OK;
  cudaSetDevice(p->ctx->device);
  free_problem_arrays(p);  // stream-ordered after the problem's last use
  delete p;
  return MPRGP_OK;
}

int mprgp_problem_set_matrix(mprgp_problem *p, int nnzb, const int *row_ptr, const int *cols,
                             const double *vals, int precisions, int on_device) {
  if (!p || nnzb <= 0 || !row_ptr || !cols || !vals || (precisions & 3) == 0)
    return fail(MPRGP_INVALID, "set_matrix");
  mprgp_context *c = p->ctx;
  cudaStream_t s = c->stream;
  const int nv = p->nv;
  std::vector<int> h_ptr(nv + 1);
  if (on_device) {
    CK(cudaMemcpyAsync(h_ptr.data(), row_ptr, sizeof(int) * (nv + 1), cudaMemcpyDeviceToHost, c->io));
    CK(cudaStreamSynchronize(c->io));
  } else {
    std::memcpy(h_ptr.data(), row_ptr, sizeof(int) * (nv + 1));
  }
  if (h_ptr[0] != 0 || h_ptr[nv] != nnzb) return fail(MPRGP_INVALID, "row_ptr ends");
  for (int r = 0; r < nv; ++r)
    if (h_ptr[r + 1] < h_ptr[r]) return fail(MPRGP_INVALID, "row_ptr not monotone");
  // Block columns are checked on the device as A is converted: a solve of an
  // A that had one outside 0..nv-1 returns MPRGP_INVALID (the conversion
  // keeps every index in range, so nothing reads out of bounds).
  // The BSR stays on the device (the SELL layout is rebuilt from it when the
  // constraint planes change which vertices have several planes).
  if (!p->stage_ptr) {
    int rc = dalloc(p->ctx, &p->stage_ptr, nv + 1);
    if (rc) return rc;
  }
  if ((size_t)nnzb > p->stage_nnzb) {
    dfree(p->ctx, p->stage_cols);
    dfree(p->ctx, p->stage_vals);
    int rc = dalloc(p->ctx, &p->stage_cols, nnzb);
    if (!rc) rc = dalloc(p->ctx, &p->stage_vals, (size_t)nnzb * 9);
    if (rc) return rc;
    p->stage_nnzb = nnzb;
  }
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  CK(cudaMemcpyAsync(p->stage_ptr, row_ptr, sizeof(int) * (nv + 1), kind, s));
  CK(cudaMemcpyAsync(p->stage_cols, cols, sizeof(int) * nnzb, kind, s));
  CK(cudaMemsetAsync(p->bad, 0, sizeof(int), s));
  p->bad_host = -1;
  CK(cudaMemcpyAsync(p->stage_vals, vals, sizeof(double) * 9 * nnzb, kind, s));
  p->h_len.resize(nv);
  for (int r = 0; r < nv; ++r) p->h_len[r] = h_ptr[r + 1] - h_ptr[r];
  p->nnzb = nnzb;
  p->want64 = precisions & 1;
  p->want32 = (precisions >> 1) & 1;
  const int rc = build_layout(p, layout_key(p));
  if (rc) return rc;
  p->planes_dirty = 1;  // 1/diag(J D^-1 J^T) depends on D
  p->matrix_gen++;      // a new A: the cached power methods no longer apply
  p->pcache.valid = p->pcache_ev.valid = 0;
  return MPRGP_OK;
}

int mprgp_problem_set_rhs(mprgp_problem *p, const double *b, int on_device) {
  if (!p || !b) return fail(MPRGP_INVALID, "set_rhs");
  CK(cudaMemcpyAsync(p->b, b, sizeof(double) * 3 * (size_t)p->nv,
                     on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                     p->ctx->stream));
  return MPRGP_OK;
}

int mprgp_problem_set_planes(mprgp_problem *p, const int *plane_ptr, const double *planes,
                             int on_device) {
  if (!p || !plane_ptr) return fail(MPRGP_INVALID, "set_planes");
  const int nv = p->nv;
  std::vector<int> h(nv + 1);
  if (on_device) {
    CK(cudaMemcpyAsync(h.data(), plane_ptr, sizeof(int) * (nv + 1), cudaMemcpyDeviceToHost,
                       p->ctx->io));
    CK(cudaStreamSynchronize(p->ctx->io));
  } else {
    std::memcpy(h.data(), plane_ptr, sizeof(int) * (nv + 1));
  }
  if (h[0] != 0) return fail(MPRGP_INVALID, "plane_ptr[0] != 0");
  for (int v = 0; v < nv; ++v) {
    const int k = h[v + 1] - h[v];
    if (k < 0 || k > kMaxPlanes) return fail(MPRGP_INVALID, "0..3 planes per vertex");
  }
  const int m = h[nv];
  if (m > 0 && !planes) return fail(MPRGP_INVALID, "planes");
  cudaStream_t s = p->ctx->stream;
  if (m != p->m || p->cons != 1) {
    dfree(p->ctx, p->plane_ptr); dfree(p->ctx, p->planes_raw); dfree(p->ctx, p->planes); dfree(p->ctx, p->pl_nn);
    dfree(p->ctx, p->pl_indn); dfree(p->ctx, p->pl_axis); dfree(p->ctx, p->face);
    int rc = dalloc(p->ctx, &p->plane_ptr, nv + 1);
    if (!rc) rc = dalloc(p->ctx, &p->planes_raw, 4 * (size_t)std::max(m, 1));
    if (!rc) rc = dalloc(p->ctx, &p->planes, 4 * (size_t)std::max(m, 1));
    if (!rc) rc = dalloc(p->ctx, &p->pl_nn, (size_t)std::max(m, 1));
    if (!rc) rc = dalloc(p->ctx, &p->pl_indn, (size_t)std::max(m, 1));
    if (!rc && !p->pl_unit) rc = dalloc(p->ctx, &p->pl_unit, (size_t)nv);
    if (!rc) rc = dalloc(p->ctx, &p->pl_axis, (size_t)std::max(m, 1));
    if (!rc) rc = dalloc(p->ctx, &p->face, (size_t)std::max(m, 1));
    if (rc) return rc;
  }
  {
    const int rc = upload(p->ctx, p->plane_ptr, h.data(), sizeof(int) * (nv + 1), s);
    if (rc) return rc;
  }
  if (m > 0)
    CK(cudaMemcpyAsync(p->planes_raw, planes, sizeof(double) * 4 * (size_t)m,
                       on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(p->face, 0, std::max(m, 1), s));
  p->m = m;
  p->face_len = m;
  p->cons = 1;
  p->planes_dirty = 1;
  p->h_plane_ptr.swap(h);
  if (p->cols && p->stage_vals) {
    const unsigned long long key = layout_key(p);
    if (key != p->layout) return build_layout(p, key);
  }
  return MPRGP_OK;
}

int mprgp_problem_set_bounds(mprgp_problem *p, const double *L, const double *U) {
  if (!p || !L) return fail(MPRGP_INVALID, "set_bounds");
  const size_t n = 3 * (size_t)p->nv;
  cudaStream_t s = p->ctx->stream;
  if (p->cons < 2) {
    dfree(p->ctx, p->face);
    int rc = dalloc(p->ctx, &p->L, n);
    if (!rc) rc = dalloc(p->ctx, &p->U, n);
    if (!rc) rc = dalloc(p->ctx, &p->face, n);
    if (rc) return rc;
  }
  CK(cudaMemcpyAsync(p->L, L, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  if (U) CK(cudaMemcpyAsync(p->U, U, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(p->face, 0, n, s));
  CK(cudaStreamSynchronize(s));
  p->cons = U ? 3 : 2;
  p->face_len = (int)n;
  p->m = (int)n;
  return MPRGP_OK;
}

int mprgp_problem_set_x(mprgp_problem *p, const double *x, int on_device) {
  if (!p || !x) return fail(MPRGP_INVALID, "set_x");
  const size_t n = 3 * (size_t)p->nv;
  CK(cudaMemcpyAsync(p->vec + (size_t)(B_X0 + p->xc) * n, x, sizeof(double) * n,
                     on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                     p->ctx->stream));
  return MPRGP_OK;
}

int mprgp_problem_get_x(mprgp_problem *p, double *x, int on_device) {
  if (!p || !x) return fail(MPRGP_INVALID, "get_x");
  const size_t n = 3 * (size_t)p->nv;
  CK(cudaMemcpyAsync(x, p->vec + (size_t)(B_X0 + p->xc) * n, sizeof(double) * n,
                     on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                     p->ctx->stream));
  if (!on_device) CK(cudaStreamSynchronize(p->ctx->stream));
  return MPRGP_OK;
}

int mprgp_problem_num_vertices(mprgp_problem *p, int *nv) {
  if (!p || !nv) return fail(MPRGP_INVALID, "num_vertices");
  *nv = p->nv;
  return MPRGP_OK;
}

int mprgp_problem_get_planes(mprgp_problem *p, int *plane_ptr, double *planes) {
  if (!p || p->cons != 1) return fail(MPRGP_INVALID, "get_planes: no planes set");
  if (plane_ptr) std::copy(p->h_plane_ptr.begin(), p->h_plane_ptr.end(), plane_ptr);
  if (planes && p->m > 0) {
    CK(cudaMemcpyAsync(planes, p->planes_raw, sizeof(double) * 4 * (size_t)p->m,
                       cudaMemcpyDeviceToHost, p->ctx->stream));
    CK(cudaStreamSynchronize(p->ctx->stream));
  }
  return MPRGP_OK;
}

int mprgp_problem_num_constraints(mprgp_problem *p, int *m) {
  if (!p || !m) return fail(MPRGP_INVALID, "num_constraints");
  *m = p->face_len;
  return MPRGP_OK;
}

int mprgp_problem_get_face(mprgp_problem *p, unsigned char *face) {
  if (!p || !face) return fail(MPRGP_INVALID, "get_face");
  if (p->face_len == 0) return MPRGP_OK;
  CK(cudaMemcpyAsync(face, p->face, p->face_len, cudaMemcpyDeviceToHost, p->ctx->stream));
  CK(cudaStreamSynchronize(p->ctx->stream));
  return MPRGP_OK;
}

int mprgp_problem_set_power_cache(mprgp_problem *p, int enable) {
  if (!p) return fail(MPRGP_INVALID, "set_power_cache");
  p->pcache_on = enable ? 1 : 0;
  if (!enable) p->pcache.valid = p->pcache_ev.valid = 0;
  return MPRGP_OK;
}

int mprgp_problem_set_ev(mprgp_problem *p, const double *ev) {
  if (!p) return fail(MPRGP_INVALID, "set_ev");
  p->ev_gen++;
  if (!ev) { p->ev_valid = 0; return MPRGP_OK; }
  CK(cudaMemcpyAsync(p->ev, ev, sizeof(double) * 3 * (size_t)p->nv, cudaMemcpyHostToDevice,
                     p->ctx->stream));
  p->ev_valid = 1;
  return MPRGP_OK;
}

int mprgp_problem_get_ev(mprgp_problem *p, double *ev, int *valid) {
  if (!p) return fail(MPRGP_INVALID, "get_ev");
  if (valid) *valid = p->ev_valid;
  if (ev && p->ev_valid) {
    CK(cudaMemcpyAsync(ev, p->ev, sizeof(double) * 3 * (size_t)p->nv, cudaMemcpyDeviceToHost,
                       p->ctx->stream));
    CK(cudaStreamSynchronize(p->ctx->stream));
  }
  return MPRGP_OK;
}

int mprgp_problem_set_trace(mprgp_problem *p, int capacity) {
  if (!p || capacity < 0) return fail(MPRGP_INVALID, "set_trace");
  dfree(p->ctx, p->trace);
  p->trace_cap = 0;
  p->trace_n = 0;
  if (capacity == 0) return MPRGP_OK;
  int rc = dalloc(p->ctx, &p->trace, 4 * (size_t)capacity);
  if (rc) return rc;
  p->trace_cap = capacity;
  return MPRGP_OK;
}

int mprgp_problem_get_trace(mprgp_problem *p, double *out, int capacity, int *count) {
  if (!p) return fail(MPRGP_INVALID, "get_trace");
  const int n = std::min(p->trace_n, p->trace_cap);
  if (count) *count = n;
  if (out && n > 0) {
    CK(cudaMemcpyAsync(out, p->trace, sizeof(double) * 4 * std::min(n, capacity),
                       cudaMemcpyDeviceToHost, p->ctx->stream));
    CK(cudaStreamSynchronize(p->ctx->stream));
  }
  return MPRGP_OK;
}

int mprgp_problem_solve(mprgp_problem *p, const mprgp_options *opt, mprgp_stats *stats) {
  if (!p || !opt) return fail(MPRGP_INVALID, "solve");
  CK(cudaSetDevice(p->ctx->device));
  mprgp_problem *arr[1] = {p};
  const int rc = run_engine(p->ctx, 1, arr, opt, stats);
  if (rc == MPRGP_OK && stats) return stats->code;
  return rc;
}

int mprgp_problem_spmv(mprgp_problem *p, const double *x_dev, double *y_dev, int precision) {
  if (!p || !x_dev || !y_dev || !p->cols) return fail(MPRGP_INVALID, "spmv");
  const bool f32 = precision == MPRGP_PREC_MIXED;
  if ((f32 && !p->has32) || (!f32 && !p->has64)) return fail(MPRGP_INVALID, "spmv precision");
  if (p->bad_host < 0) {  // the device check of A's columns, read once per matrix
    int b = 0;
    CK(cudaMemcpyAsync(&b, p->bad, sizeof(int), cudaMemcpyDeviceToHost, p->ctx->stream));
    CK(cudaStreamSynchronize(p->ctx->stream));
    p->bad_host = b;
  }
  if (p->bad_host) return fail(MPRGP_INVALID, "spmv: A has a column outside 0..nv-1");
  SellMatrix A;
  A.stream_l2 = 0;
  A.nslices = p->nslices;
  A.slice_off = p->slice_off;
  A.cols = p->cols;
  A.cols16 = p->cols16;
  A.c16ok = p->c16ok;
  A.rowmap = p->rowmap;
  A.v64 = p->v64;
  A.v32 = p->v32;
#ifdef MPRGP_CHECKS
  A.nv = p->nv;
  A.bad = p->bad;
#endif
  p->ctx->launches++;
  launch_spmv(A, p->nv, f32, x_dev, y_dev, p->ctx->stream);
  CK(cudaGetLastError());
  return MPRGP_OK;
}

int mprgp_solve_batch(mprgp_context *c, int count, mprgp_problem *const *probs,
                      const mprgp_options *opts, mprgp_stats *stats) {
  if (!c || count <= 0 || !probs || !opts) return fail(MPRGP_INVALID, "solve_batch");
  CK(cudaSetDevice(c->device));
  return run_engine(c, count, probs, opts, stats);
}

int mprgp_solve_bsr(mprgp_context *c, int nv, int nnzb, const int *row_ptr, const int *cols,
                    const double *vals, const double *b, const int *plane_ptr,
                    const double *planes, const double *L, const double *U,
                    const mprgp_options *opt, double *x, unsigned char *face, double *ev,
                    mprgp_stats *stats) {
  if (!c || !opt || !x || !b) return fail(MPRGP_INVALID, "solve_bsr");
  CK(cudaSetDevice(c->device));
  if (c->scratch && c->scratch->nv != nv) {
    mprgp_problem_destroy(c->scratch);
    c->scratch = nullptr;
  }
  if (!c->scratch) {
    int rc = mprgp_problem_create(c, nv, &c->scratch);
    if (rc) return rc;
  }
  mprgp_problem *p = c->scratch;
  const int prec = opt->precision == MPRGP_PREC_MIXED ? 3 : 1;
  // the constraints before the matrix: the SELL layout (which depends on
  // the planes) is then built once, for the constraints of this call
  int rc = opt->kind >= MPRGP_KIND_DECOUPLED
               ? mprgp_problem_set_planes(p, plane_ptr, planes, 0)
               : mprgp_problem_set_bounds(p, L, opt->kind == MPRGP_KIND_BOX ? U : nullptr);
  if (!rc) rc = mprgp_problem_set_matrix(p, nnzb, row_ptr, cols, vals, prec, 0);
  if (!rc) rc = mprgp_problem_set_rhs(p, b, 0);
  p->xc = 0;
  if (!rc) rc = mprgp_problem_set_x(p, x, 0);
  p->ev_valid = 0;
  if (!rc && ev && opt->use_ev) rc = mprgp_problem_set_ev(p, ev);
  if (rc) return rc;
  mprgp_stats local;
  mprgp_problem *arr[1] = {p};
  rc = run_engine(c, 1, arr, opt, &local);
  if (rc < MPRGP_NOT_CONVERGED) {
    if (stats) *stats = local;
    return rc;
  }
  rc = mprgp_problem_get_x(p, x, 0);
  if (!rc && face) rc = mprgp_problem_get_face(p, face);
  if (!rc && ev && local.ev_updated) rc = mprgp_problem_get_ev(p, ev, nullptr);
  if (stats) *stats = local;
  if (rc) return rc;
  return local.code;
}

}  // extern "C"
