// mprgp_solve_noalloc: a plane-constrained MPRGP solve that allocates nothing.
//
// Some callers cannot call cudaMalloc while they solve: a real-time control
// loop that must not enter the allocator (an allocation can synchronize the
// device and take unbounded time), a plug-in living inside a host program
// that owns and budgets all device memory itself, or a host that shares the
// GPU under a fixed memory quota.  This entry point takes every input and output as a
// device pointer the caller already owns and runs the same persistent engine
// as mprgp_problem_solve, with all of its working memory (the SELL copy of
// A, the solver vectors, the per-item partial sums, the state and the grid
// barrier) carved out of one file-scope device array, g_noalloc_scratch.
//
// Limits and rules, stated for users:
//   * The array is kNoAllocScratchBytes (64 MiB) and every GPU that loads
//     this library holds it until the process exits.  A problem whose working
//     set does not fit is rejected with MPRGP_INVALID before any device work
//     (roughly 37k vertices / 110k unknowns for FP64, fewer in mixed form).
//   * The first call on a device does a one-time set-up on that device: it
//     looks up the array's device address (cudaGetSymbolAddress) and the
//     resident size of the engine grid.  Make that first call before any
//     stream capture.  The address is kept for the life of the process, so
//     resetting the device (cudaDeviceReset) after the first call is not
//     supported.
//   * On an error (MPRGP_TIMEOUT, MPRGP_BREAKDOWN, ...) x and face are left
//     as the caller passed them, as mprgp_solve_bsr does.
//   * Every call shares the one array and leaves its contents behind; the
//     call clears what must start at zero.  Calls whose GPU work overlaps --
//     on different streams, or from different host threads -- race on the
//     array and give wrong answers.  Serialize them.
//   * It calls no cudaMalloc, cudaFree or any other allocating routine.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mprgp_gpu.h"
#include "engine.h"

namespace mprgp {
cudaError_t launch_engine(const EngineArgs &args, int grid, cudaStream_t stream);
cudaError_t engine_max_blocks_per_sm(int *n, int stage_bytes);
void launch_bsr_to_sell(int nv, const int *row_ptr, const int *cols, const double *vals,
                        const int *slice_off, const int *rowmap, int *out_cols, short *out_cols16,
                        int *c16ok, double *out64, float *out32, double *dinv, int *bad,
                        cudaStream_t st);
void launch_planes_setup(int nv, const int *plane_ptr, const double *in, double *out, double *nn,
                         double *indn, const double *dinv, unsigned char *unit, cudaStream_t st);
void set_last_error(const char *what);
}  // namespace mprgp

using namespace mprgp;

namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
constexpr int kMaxDevices = 64;

// The scratch of every mprgp_solve_noalloc call.  In host code this name is
// only a stand-in: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct DeviceSetup {
  bool ready = false;
  unsigned char *base = nullptr;  // device address of g_noalloc_scratch
  int nsm = 0, bps = 0;
};
DeviceSetup g_dev[kMaxDevices];
std::mutex g_dev_mutex;

int err(int code, const std::string &what) {
  set_last_error(what.c_str());
  return code;
}
int cuda_err(cudaError_t e, const char *what) {
  return err(e == cudaErrorNoDevice ? MPRGP_NO_DEVICE : MPRGP_CUDA_ERROR,
             std::string(what) + ": " + cudaGetErrorString(e));
}
#define NCK(call)                                     \
  do {                                                \
    cudaError_t _e = (call);                          \
    if (_e != cudaSuccess) return cuda_err(_e, #call); \
  } while (0)

// One-time set-up per device, with that device current.
int setup_device(DeviceSetup **out) {
  int dev = 0;
  NCK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return err(MPRGP_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lock(g_dev_mutex);
  DeviceSetup &d = g_dev[dev];
  if (!d.ready) {
    void *ptr = nullptr;
    NCK(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    int coop = 0;
    NCK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return err(MPRGP_NO_DEVICE, "device lacks cooperative launch");
    NCK(cudaDeviceGetAttribute(&d.nsm, cudaDevAttrMultiProcessorCount, dev));
    NCK(engine_max_blocks_per_sm(&d.bps, 0));
    if (d.bps < 1) return err(MPRGP_NO_DEVICE, "engine kernel cannot be resident");
    d.base = static_cast<unsigned char *>(ptr);
    d.ready = true;
  }
  *out = &d;
  return MPRGP_OK;
}

// Bump allocator over the scratch array (offsets only; nothing is allocated).
struct Carve {
  size_t off = 0;
  template <typename T>
  size_t take(size_t count) {
    off = (off + 255) & ~size_t(255);
    const size_t at = off;
    off += count * sizeof(T);
    return at;
  }
};

}  // namespace

extern "C" int mprgp_solve_noalloc(void *stream, int nv, int nnzb, const int *row_ptr,
                                   const int *cols, const double *vals, const double *b,
                                   const int *plane_ptr, const double *planes,
                                   const mprgp_options *opt, double *x, unsigned char *face,
                                   mprgp_stats *stats) {
  if (!opt || nv <= 0 || nnzb <= 0 || !row_ptr || !cols || !vals || !b || !plane_ptr || !x)
    return err(MPRGP_INVALID, "solve_noalloc: missing argument");
  if (opt->kind != MPRGP_KIND_DECOUPLED && opt->kind != MPRGP_KIND_PLANES)
    return err(MPRGP_INVALID, "solve_noalloc: plane kinds (DECOUPLED, PLANES) only");
  if (opt->algorithm == MPRGP_ALG_PLAIN)
    return err(MPRGP_INVALID, "solve_noalloc: monotone algorithm only");
  if (opt->use_ev) return err(MPRGP_INVALID, "solve_noalloc: no stored power vector");
  if (!(opt->tol >= 0.0) || opt->max_it < 0) return err(MPRGP_INVALID, "solve_noalloc: tol/max_it");
  const bool mixed = opt->precision == MPRGP_PREC_MIXED;
  if (!mixed && opt->precision != MPRGP_PREC_FP64)
    return err(MPRGP_INVALID, "solve_noalloc: precision");
  int pre;
  switch (opt->precond) {
    case MPRGP_PRECOND_DEFAULT:
      pre = opt->kind == MPRGP_KIND_DECOUPLED ? PRE_DECOUPLE : PRE_INFACE;
      break;
    case MPRGP_PRECOND_NONE: pre = PRE_NONE; break;
    case MPRGP_PRECOND_INFACE: pre = PRE_INFACE; break;
    case MPRGP_PRECOND_DECOUPLE: pre = PRE_DECOUPLE; break;
    default: return err(MPRGP_INVALID, "solve_noalloc: precond");
  }
  const int nslices = (nv + kSlice - 1) / kSlice;
  const size_t n = 3 * (size_t)nv;
  // Lower bound on the working set, before any device work.
  {
    Carve c;
    c.take<int>((size_t)nnzb);
    c.take<double>((size_t)nnzb * 9);
    c.take<double>(n * (kNumBuf + 2));
    if (c.off > kNoAllocScratchBytes)
      return err(MPRGP_INVALID, "solve_noalloc: problem needs more than the 64 MiB scratch array");
  }
  DeviceSetup *dev = nullptr;
  int rc = setup_device(&dev);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  // Host copies of the two small index arrays: SELL slice widths, checks.
  std::vector<int> h_ptr(nv + 1), h_pp(nv + 1);
  NCK(cudaMemcpyAsync(h_ptr.data(), row_ptr, sizeof(int) * (nv + 1), cudaMemcpyDeviceToHost, s));
  NCK(cudaMemcpyAsync(h_pp.data(), plane_ptr, sizeof(int) * (nv + 1), cudaMemcpyDeviceToHost, s));
  NCK(cudaStreamSynchronize(s));
  if (h_ptr[0] != 0 || h_ptr[nv] != nnzb) return err(MPRGP_INVALID, "solve_noalloc: row_ptr");
  if (h_pp[0] != 0) return err(MPRGP_INVALID, "solve_noalloc: plane_ptr");
  for (int v = 0; v < nv; ++v) {
    if (h_ptr[v + 1] < h_ptr[v]) return err(MPRGP_INVALID, "solve_noalloc: row_ptr not monotone");
    const int k = h_pp[v + 1] - h_pp[v];
    if (k < 0 || k > kMaxPlanes) return err(MPRGP_INVALID, "solve_noalloc: 0..3 planes per vertex");
  }
  const int m = h_pp[nv];
  if (m > 0 && !planes) return err(MPRGP_INVALID, "solve_noalloc: planes");
  std::vector<int> off(nslices + 1, 0);
  for (int sl = 0; sl < nslices; ++sl) {
    int w = 0;
    for (int r = sl * kSlice; r < std::min(nv, (sl + 1) * kSlice); ++r)
      w = std::max(w, h_ptr[r + 1] - h_ptr[r]);
    off[sl + 1] = off[sl] + w;
  }
  const size_t slots = (size_t)off[nslices];
  const int nitems = (nv + kThreads - 1) / kThreads;

  // Layout of the working set inside the scratch array.
  Carve c;
  const size_t o_ctl = c.take<Ctl>(1), o_desc = c.take<InstDesc>(1), o_pref = c.take<int>(2);
  const size_t o_st = c.take<InstState>(1), o_cnt = c.take<unsigned int>(1);
  const size_t o_bad = c.take<int>(1);
  const size_t o_soff = c.take<int>(nslices + 1), o_cols = c.take<int>(slots * kSlice);
  const size_t o_v64 = c.take<double>(slots * kSlice * 9);
  const size_t o_v32 = mixed ? c.take<float>(slots * kSlice * 9) : 0;
  const size_t o_dinv = c.take<double>(n), o_pl = c.take<double>(4 * (size_t)std::max(m, 1));
  const size_t o_nn = c.take<double>(std::max(m, 1)), o_indn = c.take<double>(std::max(m, 1));
  const size_t o_face = c.take<unsigned char>(std::max(m, 1));
  const size_t o_vec = c.take<double>(n * kNumBuf), o_ev = c.take<double>(n);
  const size_t o_vec32 = mixed ? c.take<float>(n * kNumBuf32) : 0;
  const size_t o_part = c.take<double>((size_t)nitems * kPart);
  if (c.off > kNoAllocScratchBytes) {
    return err(MPRGP_INVALID, "solve_noalloc: problem needs " + std::to_string(c.off >> 20) +
                                  " MiB of scratch; the array holds 64 MiB");
  }
  unsigned char *base = dev->base;
  Ctl *ctl = reinterpret_cast<Ctl *>(base + o_ctl);
  InstDesc *d_desc = reinterpret_cast<InstDesc *>(base + o_desc);
  int *d_pref = reinterpret_cast<int *>(base + o_pref);
  InstState *d_st = reinterpret_cast<InstState *>(base + o_st);
  unsigned int *d_cnt = reinterpret_cast<unsigned int *>(base + o_cnt);
  int *d_soff = reinterpret_cast<int *>(base + o_soff);
  int *d_cols = reinterpret_cast<int *>(base + o_cols);
  double *d_v64 = reinterpret_cast<double *>(base + o_v64);
  float *d_v32 = mixed ? reinterpret_cast<float *>(base + o_v32) : nullptr;
  double *d_dinv = reinterpret_cast<double *>(base + o_dinv);
  double *d_pl = reinterpret_cast<double *>(base + o_pl);
  double *d_nn = reinterpret_cast<double *>(base + o_nn);
  double *d_indn = reinterpret_cast<double *>(base + o_indn);
  unsigned char *d_face = base + o_face;
  double *d_vec = reinterpret_cast<double *>(base + o_vec);

  // A -> SELL-32 (+ D^-1), planes -> (n, c) rows, x -> X0; zero what counts.
  NCK(cudaMemcpyAsync(d_soff, off.data(), sizeof(int) * (nslices + 1), cudaMemcpyHostToDevice, s));
  int *d_bad = reinterpret_cast<int *>(base + o_bad);
  NCK(cudaMemsetAsync(d_bad, 0, sizeof(int), s));
  launch_bsr_to_sell(nv, row_ptr, cols, vals, d_soff, nullptr, d_cols, nullptr, nullptr, d_v64, d_v32, d_dinv, d_bad,
                     s);
  NCK(cudaGetLastError());
  {  // the conversion checks the block columns; no solve on an invalid A
    int bad = 0;
    NCK(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    NCK(cudaStreamSynchronize(s));
    if (bad) return err(MPRGP_INVALID, "solve_noalloc: A has a column outside 0..nv-1");
  }
  if (m > 0) {
    launch_planes_setup(nv, plane_ptr, planes, d_pl, d_nn, d_indn, d_dinv, nullptr, s);
    NCK(cudaGetLastError());
  }
  NCK(cudaMemsetAsync(d_face, 0, std::max(m, 1), s));
  NCK(cudaMemcpyAsync(d_vec + (size_t)B_X0 * n, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));

  InstDesc D;
  std::memset(&D, 0, sizeof(D));
  D.A.nslices = nslices;
  D.A.slice_off = d_soff;
  D.A.cols = d_cols;
  D.A.v64 = d_v64;
  D.A.v32 = d_v32;
  D.A.rowmap = nullptr;
#ifdef MPRGP_CHECKS
  D.A.nv = nv;
  D.A.bad = d_bad;
#endif
  D.nv = nv;
  D.nitems = nitems;
  D.item_begin = 0;
  D.m = m;
  D.kind = opt->kind == MPRGP_KIND_DECOUPLED ? KIND_DECOUPLED : KIND_PLANES;
  D.alg = ALG_MONOTONE;
  D.pre = pre;
  D.prec = mixed ? PREC_MIXED : PREC_FP64;
  D.max_it = opt->max_it;
  D.tol = opt->tol < 1e-30 ? 1e-30 : opt->tol;
  D.seed = opt->seed;
  D.b = b;
  D.dinv = d_dinv;
  D.plane_ptr = plane_ptr;
  D.planes = d_pl;
  D.pl_nn = d_nn;
  D.pl_indn = d_indn;
  D.pl_unit = nullptr;  // the general per-vertex QPs throughout
  D.face = d_face;
  for (int i = 0; i < kNumBuf; ++i) D.buf[i] = d_vec + (size_t)i * n;
  for (int i = 0; i < kNumBuf32; ++i)
    D.buf32[i] = mixed ? reinterpret_cast<float *>(base + o_vec32) + (size_t)i * n : nullptr;
  D.ev = reinterpret_cast<double *>(base + o_ev);
  D.part = reinterpret_cast<double *>(base + o_part);
  D.cnt = d_cnt;
  D.st = d_st;
  InstState S;
  std::memset(&S, 0, sizeof(S));
  S.code = -1;
  S.phase = PH_POW_RAND;
  D.project_x0 = opt->project_x0 ? 1 : 0;
  const int pref[2] = {0, nitems};
  Ctl c0;
  std::memset(&c0, 0, sizeof(c0));
  c0.active = 1;
  c0.snap[0] = c0.snap[1] = 1;
  NCK(cudaMemcpyAsync(d_desc, &D, sizeof(D), cudaMemcpyHostToDevice, s));
  NCK(cudaMemcpyAsync(d_st, &S, sizeof(S), cudaMemcpyHostToDevice, s));
  NCK(cudaMemcpyAsync(d_pref, pref, sizeof(pref), cudaMemcpyHostToDevice, s));
  NCK(cudaMemcpyAsync(ctl, &c0, sizeof(c0), cudaMemcpyHostToDevice, s));
  NCK(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned int), s));

  const double wait_s = opt->wait_limit_s > 0.0 ? opt->wait_limit_s : 5.0;
  EngineArgs args;
  args.desc = d_desc;
  args.item_prefix = d_pref;
  args.item_inst = nullptr;  // one instance
  args.states = nullptr;
  args.ninst = 1;
  args.total_items = nitems;
  args.max_phases = (int)std::min<long long>(1100LL + 8LL * ((long long)opt->max_it + 2), INT_MAX);
  args.wait_ns = (long long)(wait_s * 1e9);
  args.total_ns = (long long)(std::max(60.0, 20.0 * wait_s) * 1e9);
  args.stage_bytes = 0;
  args.ctl = ctl;
  const int grid = std::max(1, std::min(nitems, dev->nsm * dev->bps));
  const auto t0 = std::chrono::steady_clock::now();
  NCK(launch_engine(args, grid, s));
  InstState out;
  Ctl c1;
  NCK(cudaMemcpyAsync(&out, d_st, sizeof(out), cudaMemcpyDeviceToHost, s));
  NCK(cudaMemcpyAsync(&c1, ctl, sizeof(c1), cudaMemcpyDeviceToHost, s));
  NCK(cudaStreamSynchronize(s));
  const double ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (c1.err) out.code = c1.err;
  else if (out.phase != PH_DONE) out.code = MPRGP_TIMEOUT;
#ifdef MPRGP_CHECKS
  {  // an index check failed during the solve
    int bad = 0;
    NCK(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    NCK(cudaStreamSynchronize(s));
    if (bad) out.code = MPRGP_INVALID;
  }
#endif
  if (out.code >= MPRGP_NOT_CONVERGED) {  // results only for a finished solve
    NCK(cudaMemcpyAsync(x, d_vec + (size_t)(B_X0 + out.xc) * n, sizeof(double) * n,
                        cudaMemcpyDeviceToDevice, s));
    if (face && m > 0) NCK(cudaMemcpyAsync(face, d_face, m, cudaMemcpyDeviceToDevice, s));
    NCK(cudaStreamSynchronize(s));
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->code = out.code;
    stats->iterations = out.iters_out;
    stats->num_cg = out.num_cg;
    stats->num_exp = out.num_exp;
    stats->num_prop = out.num_prop;
    stats->power_iters = out.power_iters;
    stats->active = out.active;
    stats->ev_updated = out.ev_upd;
    stats->residual = out.residual;
    stats->alpha_bar = out.alpha_bar;
    stats->spec_rad = out.spec_rad;
    stats->spmv_fp64 = out.spmv64;
    stats->spmv_fp32 = out.spmv32;
    stats->phases = out.phases;
    stats->device_ms = ms;
    stats->power_passes = out.pow_spmv;
  }
  if (c1.err) return err(c1.err, "solve_noalloc: device wait limit reached");
  return out.code;
}
