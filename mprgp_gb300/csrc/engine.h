// Shared host/device layout of the persistent MPRGP engine.
//
// One engine launch advances any number of QP instances ("instances") in
// lockstep macro-phases.  A macro-phase walks a work list of items -- 256
// consecutive vertex rows of one instance -- across the whole grid, then one
// bounded grid barrier separates it from the next.  Each instance carries its
// own state machine (InstState), which restates the control flow of the
// reference's MPRGPMonotonic::solve / MPRGP::solve (MPRGPSolver.h:356-454).
// The CTA that completes the last item of an instance in a phase reduces that
// instance's per-item partial sums (fixed order: deterministic) and advances
// its state; the other CTAs read the new state after the barrier.
#pragma once
#include <cstdint>

namespace mprgp {

constexpr int kThreads = 256;       // threads per CTA = vertex rows per item
constexpr int kSlice = 32;          // SELL slice height (one warp)
constexpr int kPart = 10;           // partial sums per item (slot kMinSlot is a min)
constexpr int kMinSlot = 9;
constexpr int kMaxPlanes = 3;       // plane constraints per vertex
constexpr int kStageBytes = 192 * 1024;  // shared-memory stage of one item's FP32 A

enum Kind : int { KIND_LOWER = 0, KIND_BOX = 1, KIND_DECOUPLED = 2, KIND_PLANES = 3 };
enum Alg : int { ALG_MONOTONE = 1, ALG_PLAIN = 2 };
enum Pre : int { PRE_NONE = 1, PRE_INFACE = 2, PRE_DECOUPLE = 3 };
enum Prec : int { PREC_FP64 = 0, PREC_MIXED = 1 };

// Vector buffers of one instance, each 3*nv doubles.
enum Buf : int {
  B_X0 = 0, B_X1, B_G0, B_G1, B_Z0, B_Z1, B_P0, B_P1, B_BT0, B_BT1,
  B_AP, B_W, B_E, B_T0, B_T1, B_W1, kNumBuf
};
// FP32 shadows of the vectors the mixed form's FP32 matrix passes read
// (z, p and the power iterate), each 3*nv floats, written by the phase that
// produces the FP64 vector.
enum Buf32 : int { F_Z0 = 0, F_Z1, F_P0, F_P1, F_W0, F_W1, kNumBuf32 };

// A solve starts with the power method (independent of x), then projects x
// if asked (the solve(A,B,J,c,x) overloads), then runs MPRGP.
enum Phase : int {
  PH_DONE = 0,
  PH_PROJ0,     // x = P(x)
  PH_POW_RAND,  // seeded start vector, |t|^2
  PH_POW,       // t_k = src/scale; w = A t_k; |w|^2, |t_k - t_{k-1}|^2
  PH_POW_LAST,  // |w_1000/|w_1000| - t_1000|
  PH_INIT,      // g = Ax - b; face; phi; z; p = z; loop-top sums
  PH_CG_ENTRY,  // Ap (and the true gradient when g is stale); p.Ap
  PH_CG_SPMV,   // p' = z - beta p on the fly; Ap'; p'.Ap'
  PH_CG_YF,     // y = x - alpha p, f(P(y)) - f(x), speculative next CG state
  PH_CG_DAD,    // delta^T A delta for an infeasible y (delta = P(y) - y)
  PH_EXP_A,     // y = P(x)
  PH_EXP_B,     // g = Ay - b; face(y); x = P(y - abar phi)
  PH_EXP_C,     // g = Ax - b; face(x); phi; z; p = z; loop-top sums
  PH_PROP_A,    // g = Ax - b and AD = A beta in one pass; g.D, D.AD
  PH_PROP_B,    // x = P(x - alpha D); g -= alpha AD; face; phi; z; p = z
  PH_RU,        // mixed form: FP64 residual replacement g = A64 x - b
  PH_FINAL,     // x = P(x)
  PH_PL_SPMV,   // plain MPRGP: Ap, p.Ap, ratio test alpha_f
  PH_PL_CG,     // plain CG step + loop-top sums
  PH_PL_EXP_A,  // plain expansion: x = P(x - af p - abar phi)
  PH_PL_EXP_B,  // g = Ax - b; face; phi; z; p = z; loop-top sums
  PH_PL_PROP_A, // AD = A D; g.D, D.AD
  kNumPhases
};

// SELL-32 copy of a 3x3-block CSR matrix: slices of 32 block rows; slot j of
// slice s holds, for lanes t = 0..31, one block per row.  The rows are laid
// out in `rowmap` order (a performance layout: vertices with several
// constraint planes are grouped after the others, so the warps that run the
// multi-plane projection are few and uniform); vectors stay in vertex order.  cols[(off+j)*32+t]
// and vals[((off+j)*9+e)*32+t] with e the row-major entry of the block, so a
// warp reads each of the nine entries as one coalesced 256 B (FP64) line.
struct SellMatrix {
  int nslices;
  const int *slice_off;  // nslices + 1, in slots
  const int *cols;       // vertex index; padding points at a valid row, value 0
  const short *cols16;   // the same as 16-bit offsets from the row's vertex; read when
  const int *c16ok;      // *c16ok: every offset fitted (nullptr: cols only)
  const double *v64;
  const float *v32;
  const int *rowmap;     // SELL row (slot) -> vertex; nullptr: slot == vertex
  int stream_l2;         // 1: the run streams more matrix bytes than L2 holds; its
                         // column and value loads are marked evict-first in L2
#ifdef MPRGP_CHECKS
  int nv;    // vertices: every column and SELL row index must lie in 0..nv-1
  int *bad;  // the instance's invalid-input word (bits 2, 4, 8: see MPRGP_CHECK)
#endif
};

struct InstState {
  int phase, pow_k, iteration, num_cg, num_exp, num_prop, power_iters, code;
  int xc, gc, zc, pc, bc;            // double-buffer selectors
  int prop, cg_prop, y_valid, y_feas, g_cons, e_nz, ev_upd, ev_src, p_is_z, active;
  int pow_src, iters_out, ev_valid, trace_n;
  double alpha_bar, spec_rad, residual, pd, pg, pe, alpha, beta_cg, zg, fx_off;
  double dfy, corr, pow_scale, pow_nrm_prev, ru_ref;
  double s_zap, s_zg, s_gp2, s_bb, s_ptp;  // speculative CG sums
  long long spmv64, spmv32, phases;
  long long pow_spmv;  // matrix passes of the power method (included in spmv64/spmv32)
};

struct InstDesc {
  SellMatrix A;
  int nv, nitems, item_begin, m;
  int kind, alg, pre, prec;
  int max_it, project_x0;
  double tol;
  unsigned long long seed;
  const double *b, *dinv;
  const int *plane_ptr;       // nv + 1 (planes kinds)
  const double *planes;       // 4 per row: nx, ny, nz, c   (J x >= c)
  const double *pl_nn;        // 1 / |n|^2 = 1 / diag(J J^T)
  const double *pl_indn;      // 1 / (n . D^-1 n) = 1 / diag(J D^-1 J^T)
  const unsigned char *pl_unit;  // per vertex: 2-3 planes whose Gram matrix is the identity
  const unsigned char *pl_axis;  // per plane row: 0..2 its normal is that unit axis, 3 other
                                 // (nullptr: every normal takes the general products)
  const double *L, *U;        // bounds kinds
  unsigned char *face;        // one per constraint row / per unknown
  double *buf[kNumBuf];
  float *buf32[kNumBuf32];    // mixed form only
  double *ev;
  double *part;               // nitems * kPart
  unsigned int *cnt;          // items finished in the current phase
  const int *bad;             // set when A held a block column outside 0..nv-1 (or,
                              // in the bounds-checked build, an index check failed)
  InstState *st;
  double *trace;              // optional step trace, 4 doubles per record
  int trace_cap, pad2;
};

struct Ctl {
  unsigned int count;   // barrier arrivals
  unsigned int gen;     // barrier generation
  int err;              // first error code (0 = none)
  int err_where;        // phase of the first error
  int active;           // instances not yet DONE
  int snap[2];          // `active` as seen at each barrier release
  int pad;
};

// Loop control of the power-method graph (see power_kernel).
struct PowCtl {
  unsigned int active;    // instances in a power phase when the current launch began
  unsigned int fin;       // settle-kernel CTAs done in the current body (power-step loop)
  unsigned int busy;      // instances still in a power phase (settle kernel) / the last
                          // phase with one (persistent power loop)
  unsigned int launches;  // launches that did work so far
  unsigned int limit;     // stop after this many launches
  unsigned int stop;      // set when the loop is over: later launches return at once
  // the phase kernel's finalizes of the current launch (low word) and, of
  // those, the instances still going on (high word), counted by one atomic
  unsigned long long finbusy;
};
constexpr int kPowerUnroll = 8;  // power launches per evaluation of the loop condition
constexpr int kPowOwn = 4;       // items per CTA of the persistent power loop
constexpr int kCodeInvalid = -5;  // MPRGP_INVALID: the result code of an invalid instance

// Small instances run on the cluster solver: one thread-block cluster per
// instance, CTA r covering items r, r + cluster, ... (at most kClusterItems
// of them); the host picks the smallest cluster size (a power of two up to
// kClusterMax) that gives every CTA one item, or else the largest size with
// up to the context's items-per-CTA limit (at most kClusterItems).
constexpr int kClusterItems = 4;
constexpr int kClusterMax = 16;
constexpr int kClusterClasses = 5;  // cluster sizes 1, 2, 4, 8, 16

struct ClusterArgs {
  const InstDesc *desc;  // the small instances, one per cluster
  int ninst;
  int max_phases;        // quantum / hard bound on phases
};

struct EngineArgs {
  const InstDesc *desc;
  const int *item_prefix;  // ninst + 1
  const int *item_inst;    // total_items: the instance of each item (nullptr: search item_prefix)
  const InstState *states; // the run's instance states, desc order (== desc[i].st), or nullptr
  int ninst, total_items;
  int max_phases;          // quantum / hard bound on macro-phases
  long long wait_ns;       // bound on a barrier wait
  long long total_ns;      // bound on the whole launch
  int stage_bytes;         // dynamic shared memory for staging (0 = off)
  int pad;
  Ctl *ctl;
  // the power-step loop's two state copies (desc order), written by the
  // launches of even / odd position in a loop body
  InstState *pst[2];
};

}  // namespace mprgp
