// Persistent MPRGP engine for sm_103a.
//
// Each macro-phase every CTA walks its share of the item list (256 vertex
// rows of one instance per item), runs that instance's current phase on those
// rows, and writes one partial-sum record per item.  The CTA that finishes an
// instance's last item reduces the records in item order and advances the
// instance's state machine.  A bounded grid barrier ends the macro-phase.
//
// Row kernels restate the per-vertex arithmetic of the reference projectors
// and preconditioners (src/MPRGPSolver/MPRGPProjection.h,
// MPRGPPrecondition.h); the state machine restates MPRGPMonotonic::solve and
// MPRGP::solve (MPRGPSolver.h:148-454).  Every constraint row touches one
// vertex, so all projector work is local to a row and fuses into the SpMV
// epilogues; only the reductions cross rows.
#include <cfloat>
#include <cstring>
#include <cstdint>

#include <cuda_runtime.h>

#include "engine.h"

namespace mprgp {

constexpr double kEps = 1e-9;  // ScalarUtil<double>::scalar_eps (MathBasic.cpp:9)

// Resident CTAs per SM the engine is compiled for (register budget).
#ifndef MPRGP_PREFETCH_DIST  // chunks ahead that a streaming matrix pass prefetches into L2
#define MPRGP_PREFETCH_DIST 1  // (0: none)
#endif
#ifndef MPRGP_SPMV_CHUNK
#define MPRGP_SPMV_CHUNK 4
#endif
#ifndef MPRGP_SPMV_MIN_BLOCKS  // resident CTAs per SM the standalone SpMV is compiled for
#define MPRGP_SPMV_MIN_BLOCKS 4
#endif
#ifndef MPRGP_CLUSTER_MIN_BLOCKS  // resident CTAs per SM the cluster solver is compiled for
#define MPRGP_CLUSTER_MIN_BLOCKS 6   // (its phases are latency-bound: more clusters in flight)
#endif
#ifndef MPRGP_POWER_MIN_BLOCKS  // ... the smaller-register power kernel (tuning variant 0)
#define MPRGP_POWER_MIN_BLOCKS 6
#endif
#ifndef MPRGP_ALLPHASE_MIN_BLOCKS  // ... and the all-phase kernel of the graph-loop engine
#define MPRGP_ALLPHASE_MIN_BLOCKS 4
#endif
#ifndef MPRGP_ENGINE_MIN_BLOCKS
#define MPRGP_ENGINE_MIN_BLOCKS 4
#endif
#ifndef MPRGP_STEP_MIN_BLOCKS  // ... and the power-step kernel (288 threads: 56 registers)
#define MPRGP_STEP_MIN_BLOCKS 4
#endif

// ------------------------------------------------------------ primitives --
// Bounds-checked debug build (-DMPRGP_CHECKS): indices the kernels read from
// device arrays -- block columns, SELL row order, plane offsets -- are checked
// before use.  A bad one sets a bit in the instance's invalid-input word
// (2: block column, 4: plane offsets, 8: SELL row) and is replaced by a safe
// index, so nothing is read out of bounds; the solve then reports
// MPRGP_INVALID.  The release build compiles the checks out.
#ifdef MPRGP_CHECKS
#define MPRGP_CHECK(cond, word, bit, fix) \
  do {                                    \
    if (!(cond)) {                        \
      if (word) atomicOr(word, bit);      \
      fix;                                \
    }                                     \
  } while (0)
#else
#define MPRGP_CHECK(cond, word, bit, fix) \
  do {                                    \
  } while (0)
#endif
__device__ __forceinline__ long long gtimer() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Read-only inputs of a launch (A, b, D^-1, planes): non-volatile ld.global.nc
// so the compiler may overlap them freely.
__device__ __forceinline__ double ldro(const double *p) {
  double r;
  asm("ld.global.nc.f64 %0, [%1];" : "=d"(r) : "l"(p));
  return r;
}
__device__ __forceinline__ float ldro(const float *p) {
  float r;
  asm("ld.global.nc.f32 %0, [%1];" : "=f"(r) : "l"(p));
  return r;
}
__device__ __forceinline__ int ldro(const int *p) {
  int r;
  asm("ld.global.nc.s32 %0, [%1];" : "=r"(r) : "l"(p));
  return r;
}
// Vectors written by other CTAs in earlier phases are read with plain loads:
// every phase boundary is a grid barrier whose gpu-scope acquire (followed
// by bar.sync) makes those writes visible, as for cooperative groups.
__device__ __forceinline__ void ld3(const double *b, int v, double o[3]) {
  const double *q = b + 3 * (size_t)v;
  o[0] = q[0];
  o[1] = q[1];
  o[2] = q[2];
}
// SELL values of one 3x3 block (slot j of the matrix, lane l of its slice),
// stored so that a lane reads its nine entries with vector loads that are
// still coalesced across the warp.  Per slot, 288 values:
//   FP32: m0..m3 as float4 at 4l, m4..m7 as float4 at 128 + 4l, m8 at 256 + l;
//   FP64: (m0,m1), (m2,m3), (m4,m5), (m6,m7) as double2 at 64k + 2l, m8 at 256 + l.
// Each slot starts on a 1152-byte (FP32) or 2304-byte (FP64) boundary.
__host__ __device__ __forceinline__ size_t sell_index(size_t j, int e, int lane, float) {
  const size_t b = j * (9 * kSlice);
  return e < 4 ? b + 4 * lane + e : (e < 8 ? b + 128 + 4 * lane + (e - 4) : b + 256 + lane);
}
__host__ __device__ __forceinline__ size_t sell_index(size_t j, int e, int lane, double) {
  const size_t b = j * (9 * kSlice);
  return e < 8 ? b + 64 * (e >> 1) + 2 * lane + (e & 1) : b + 256 + lane;
}
// L2 eviction policy of a matrix pass.  A run whose matrices together exceed
// L2 gets nothing from keeping them there (each phase evicts its own first
// rows before it reads them again), so its column and value loads are marked
// evict-first: they then replace each other and leave the vectors, and the
// matrices of other lanes' smaller instances, in L2.  Otherwise evict-normal,
// the default behaviour.
__device__ __forceinline__ unsigned long long l2_policy(int stream) {
  unsigned long long first, normal;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(first));
  asm("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(normal));
  return stream ? first : normal;
}
__device__ __forceinline__ int ldro16_pol(const short *p, unsigned long long pol) {
  short r;
  asm("ld.global.nc.L2::cache_hint.s16 %0, [%1], %2;" : "=h"(r) : "l"(p), "l"(pol));
  return (int)r;
}
__device__ __forceinline__ int ldro_pol(const int *p, unsigned long long pol) {
  int r;
  asm("ld.global.nc.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ void ld_block(const float *vals, size_t j, int lane, float m[9],
                                         unsigned long long pol) {
  const float *b = vals + j * (9 * kSlice);
  float4 p, q;
  asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
      : "=f"(p.x), "=f"(p.y), "=f"(p.z), "=f"(p.w) : "l"(b + 4 * lane), "l"(pol));
  asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
      : "=f"(q.x), "=f"(q.y), "=f"(q.z), "=f"(q.w) : "l"(b + 128 + 4 * lane), "l"(pol));
  m[0] = p.x; m[1] = p.y; m[2] = p.z; m[3] = p.w;
  m[4] = q.x; m[5] = q.y; m[6] = q.z; m[7] = q.w;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(m[8]) : "l"(b + 256 + lane), "l"(pol));
}
__device__ __forceinline__ void ld_block(const double *vals, size_t j, int lane, double m[9],
                                         unsigned long long pol) {
  const double *b = vals + j * (9 * kSlice);
#pragma unroll
  for (int k = 0; k < 4; ++k)
    asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
        : "=d"(m[2 * k]), "=d"(m[2 * k + 1]) : "l"(b + 64 * k + 2 * lane), "l"(pol));
  asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(m[8]) : "l"(b + 256 + lane), "l"(pol));
}
// The same from a shared-memory copy of whole slots.
template <typename VT>
__device__ __forceinline__ void ld_block_smem(const VT *vals, size_t j, int lane, VT m[9]) {
#pragma unroll
  for (int e = 0; e < 9; ++e) m[e] = vals[sell_index(j, e, lane, VT())];
}

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned int atom_add_acq_rel(unsigned int *p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;"
               : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ unsigned long long atom_add_acq_rel(unsigned long long *p,
                                                               unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.add.acq_rel.gpu.global.u64 %0, [%1], %2;"
               : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}
__device__ __forceinline__ void st_release(unsigned int *p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// ------------------------------------------------ shared-memory staging --
// For FP32 matrix passes an item's slice of A -- block columns and values of
// its 8 SELL slices, contiguous in global memory -- is brought into shared
// memory by one cp.async.bulk per array, completed on an mbarrier.  The
// loads of A then cost no registers and arrive as one burst per item.
extern __shared__ __align__(128) unsigned char g_stage[];
__shared__ int g_staged;             // 1 while the current item's A is staged
__shared__ int g_stage_first;        // first staged slot
__shared__ unsigned int g_stage_voff;  // byte offset of the values in g_stage
__shared__ __align__(8) unsigned long long g_stage_bar;

__device__ __forceinline__ unsigned int smem_u32(const void *p) {
  return static_cast<unsigned int>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" : : "r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" : : : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned int bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               : : "r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned int bytes,
                                         unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      : : "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned int parity) {
  unsigned int ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return ok != 0;
}
// Bounded wait on the staging barrier; false after `limit_ns`.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned int parity,
                                                  long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = gtimer();
  while (!mbar_try_wait(bar, parity))
    if (gtimer() - t0 > limit_ns) return false;
  return true;
}
__device__ __forceinline__ void st3(double *b, int v, const double o[3]) {
  double *q = b + 3 * (size_t)v;
  q[0] = o[0];
  q[1] = o[1];
  q[2] = o[2];
}
__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  unsigned long long z = x;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// Seeded stand-in for Eigen's setRandom() (MPRGPSolver.h:51): uniform [-1,1).
__device__ __forceinline__ double seeded_uniform(unsigned long long seed, unsigned long long i) {
  const unsigned long long h = mix64(seed * 0x9E3779B97F4A7C15ull + i);
  return 2.0 * ((double)(h >> 11) * 1.1102230246251565e-16) - 1.0;
}

// ------------------------------------------------------------ SpMV rows --
// One thread per block row.  The nine block entries and the column of slot j
// are lane-contiguous in the SELL layout, so each load instruction of a warp
// is one coalesced line; x is gathered per neighbour vertex.  VT is the value
// type of A and of the accumulator (FP32 accumulation for the FP32 copy).
struct SrcV {
  const double *p;
  __device__ __forceinline__ void operator()(int c, double o[3]) const { ld3(p, c, o); }
};
struct SrcPNew {  // z - beta p   (CGStep's p = z - beta*p)
  const double *z, *p;
  double beta;
  __device__ __forceinline__ void operator()(int c, double o[3]) const {
    double zz[3], pp[3];
    ld3(z, c, zz);
    ld3(p, c, pp);
    o[0] = zz[0] - beta * pp[0];
    o[1] = zz[1] - beta * pp[1];
    o[2] = zz[2] - beta * pp[2];
  }
};

// FP32 sources for the mixed form: the FP32 shadow of a vector, or the CG
// direction z - beta p formed from the shadows in FP32.
struct SrcF {
  const float *p;
  __device__ __forceinline__ void operator()(int c, float o[3]) const {
    const float *q = p + 3 * (size_t)c;
    o[0] = q[0];
    o[1] = q[1];
    o[2] = q[2];
  }
};
struct SrcPNewF {
  const float *z, *p;
  float beta;
  __device__ __forceinline__ void operator()(int c, float o[3]) const {
    const float *zq = z + 3 * (size_t)c, *pq = p + 3 * (size_t)c;
    o[0] = fmaf(-beta, pq[0], zq[0]);
    o[1] = fmaf(-beta, pq[1], zq[1]);
    o[2] = fmaf(-beta, pq[2], zq[2]);
  }
};
struct SrcVtoF {  // FP64 vector read by an FP32 pass (standalone y = A32 x)
  const double *p;
  __device__ __forceinline__ void operator()(int c, float o[3]) const {
    const double *q = p + 3 * (size_t)c;
    o[0] = (float)q[0];
    o[1] = (float)q[1];
    o[2] = (float)q[2];
  }
};
__device__ __forceinline__ void st3f(float *b, int v, const double o[3]) {
  float *q = b + 3 * (size_t)v;
  q[0] = (float)o[0];
  q[1] = (float)o[1];
  q[2] = (float)o[2];
}

// Prefetch of `n` slots from slot j of a slice into L2 (one bulk prefetch for
// the values, one for the columns; both start on 128-byte boundaries and
// span whole slots, so address and size are multiples of 16 bytes), with
// the pass's eviction policy.  Used only by passes that stream (A.stream_l2).
template <bool k16, typename VT>
__device__ __forceinline__ void prefetch_slots(const SellMatrix &A, const VT *vals, int j, int n,
                                               unsigned long long pol) {
  const VT *pv = vals + (size_t)j * (9 * kSlice);
  asm volatile("cp.async.bulk.prefetch.L2.global.L2::cache_hint [%0], %1, %2;"
               :: "l"(pv), "r"((unsigned)(n * 9 * kSlice * sizeof(VT))), "l"(pol) : "memory");
  if (k16) {  // 64 bytes per slot
    asm volatile("cp.async.bulk.prefetch.L2.global.L2::cache_hint [%0], %1, %2;"
                 :: "l"(A.cols16 + (size_t)j * kSlice), "r"((unsigned)(n * kSlice * sizeof(short))),
                 "l"(pol) : "memory");
  } else {
    asm volatile("cp.async.bulk.prefetch.L2.global.L2::cache_hint [%0], %1, %2;"
                 :: "l"(A.cols + (size_t)j * kSlice), "r"((unsigned)(n * kSlice * sizeof(int))),
                 "l"(pol) : "memory");
  }
}

// The first chunk of slice `slice` into L2: a CTA of the power loops issues
// it for the item it takes next (the next item of this launch, or its first
// item again for the next phase) while the current item reduces, so that
// the next item's rows do not start with a DRAM round trip.
template <typename VT>
__device__ __forceinline__ void prefetch_slice_head(const SellMatrix &A, const VT *vals, int slice,
                                                    unsigned long long pol) {
  const int j0 = ldro(A.slice_off + slice), j1 = ldro(A.slice_off + slice + 1);
  if (j1 <= j0) return;
  if (A.cols16 && ldro(A.c16ok)) prefetch_slots<true>(A, vals, j0, min(MPRGP_SPMV_CHUNK, j1 - j0), pol);
  else prefetch_slots<false>(A, vals, j0, min(MPRGP_SPMV_CHUNK, j1 - j0), pol);
}
__device__ __forceinline__ void prefetch_item_head(const InstDesc &D, int local_item) {
#if MPRGP_PREFETCH_DIST > 0
  const int warp = threadIdx.x >> 5;
  if (!D.A.stream_l2 || (threadIdx.x & 31) != 0 || warp >= kThreads / 32) return;
  if (local_item < 0 || local_item >= D.nitems) return;
  const int slice = local_item * (kThreads / 32) + warp;
  if (slice >= D.A.nslices) return;
  const unsigned long long pol = l2_policy(1);
  if (D.prec == PREC_MIXED) prefetch_slice_head(D.A, D.A.v32, slice, pol);
  else prefetch_slice_head(D.A, D.A.v64, slice, pol);
#endif
}

// A block column and a SELL row's vertex, checked in the debug build.
__device__ __forceinline__ int checked_col(const SellMatrix &A, int c) {
  MPRGP_CHECK(c >= 0 && c < A.nv, A.bad, 2, c = 0);
  return c;
}
__device__ __forceinline__ int row_vertex(const SellMatrix &A, int slot) {
  int v = A.rowmap ? ldro(A.rowmap + slot) : slot;
  MPRGP_CHECK(v >= 0 && v < A.nv, A.bad, 8, v = 0);
  return v;
}

// Block column of slot j, lane `lane`: the 16-bit offset from the row's
// vertex vrow (k16) or the 32-bit column.
template <bool k16>
__device__ __forceinline__ int col_of(const SellMatrix &A, size_t j, int lane, int vrow,
                                      unsigned long long pol) {
  const size_t i = j * kSlice + lane;
  if constexpr (k16) return checked_col(A, vrow + ldro16_pol(A.cols16 + i, pol));
  else return checked_col(A, ldro_pol(A.cols + i, pol));
}

// Every slot below j1 is valid (padding blocks are zero and point at a real
// row), so whole chunks of MPRGP_SPMV_CHUNK slots carry no per-slot condition
// and all their column, value and neighbour loads can be in flight together
// (0: columns of 8 slots fetched together, then one slot at a time).  The
// products are accumulated slot by slot in order either way, so the results
// are the same -- and the same whichever column form is read.
template <bool k16, typename VT, typename Src>
__device__ __forceinline__ void spmv_row_body(const SellMatrix &A, const VT *__restrict__ vals,
                                              int lane, int vrow, int j0, int j1,
                                              unsigned long long pol, const Src &src, VT &a0,
                                              VT &a1, VT &a2) {
  int jb = j0;
#if MPRGP_SPMV_CHUNK == 0
  for (; jb < j1; jb += 8) {
    int cc[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) cc[u] = (jb + u < j1) ? col_of<k16>(A, (size_t)(jb + u), lane, vrow, pol) : -1;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      if (cc[u] < 0) break;
      VT m[9];
      ld_block(vals, (size_t)(jb + u), lane, m, pol);
      VT xv[3];
      src(cc[u], xv);
      a0 = fma(m[0], xv[0], a0); a0 = fma(m[1], xv[1], a0); a0 = fma(m[2], xv[2], a0);
      a1 = fma(m[3], xv[0], a1); a1 = fma(m[4], xv[1], a1); a1 = fma(m[5], xv[2], a1);
      a2 = fma(m[6], xv[0], a2); a2 = fma(m[7], xv[1], a2); a2 = fma(m[8], xv[2], a2);
    }
  }
#else
  for (; jb + MPRGP_SPMV_CHUNK <= j1; jb += MPRGP_SPMV_CHUNK) {
    constexpr int K = MPRGP_SPMV_CHUNK;
#if MPRGP_PREFETCH_DIST > 0
    if (A.stream_l2 && lane == 0) {  // the slots this warp reads MPRGP_PREFETCH_DIST chunks on
      const int jp = jb + K * MPRGP_PREFETCH_DIST;
      if (jp < j1) prefetch_slots<k16>(A, vals, jp, min(K, j1 - jp), pol);
    }
#endif
    int c[K];
#pragma unroll
    for (int u = 0; u < K; ++u) c[u] = col_of<k16>(A, (size_t)(jb + u), lane, vrow, pol);
    VT m[K][9];
#pragma unroll
    for (int u = 0; u < K; ++u) ld_block(vals, (size_t)(jb + u), lane, m[u], pol);
    VT xv[K][3];
#pragma unroll
    for (int u = 0; u < K; ++u) src(c[u], xv[u]);
#pragma unroll
    for (int u = 0; u < K; ++u) {
      const VT x0 = xv[u][0], x1 = xv[u][1], x2 = xv[u][2];
      a0 = fma(m[u][0], x0, a0); a0 = fma(m[u][1], x1, a0); a0 = fma(m[u][2], x2, a0);
      a1 = fma(m[u][3], x0, a1); a1 = fma(m[u][4], x1, a1); a1 = fma(m[u][5], x2, a1);
      a2 = fma(m[u][6], x0, a2); a2 = fma(m[u][7], x1, a2); a2 = fma(m[u][8], x2, a2);
    }
  }
  for (; jb < j1; ++jb) {  // the last slots of the row
    const int c = col_of<k16>(A, (size_t)jb, lane, vrow, pol);
    VT m[9];
    ld_block(vals, (size_t)jb, lane, m, pol);
    VT xv[3];
    src(c, xv);
    a0 = fma(m[0], xv[0], a0); a0 = fma(m[1], xv[1], a0); a0 = fma(m[2], xv[2], a0);
    a1 = fma(m[3], xv[0], a1); a1 = fma(m[4], xv[1], a1); a1 = fma(m[5], xv[2], a1);
    a2 = fma(m[6], xv[0], a2); a2 = fma(m[7], xv[1], a2); a2 = fma(m[8], xv[2], a2);
  }
#endif
}

// One row's product with a source vector; v is the row's SELL slot.  The
// columns come from the 16-bit offsets when the matrix has them and every
// offset fitted (A.c16ok), else from the 32-bit columns.
template <typename VT, typename Src, typename OT = double>
__device__ __forceinline__ void spmv_row(const SellMatrix &A, const VT *__restrict__ vals, int v,
                                         const Src &src, OT out[3]) {
  const int s = v >> 5, lane = v & 31;
  const int j0 = ldro(A.slice_off + s), j1 = ldro(A.slice_off + s + 1);
  const unsigned long long pol = l2_policy(A.stream_l2);
  VT a0 = 0, a1 = 0, a2 = 0;
  if (A.cols16 && ldro(A.c16ok)) {
    const int vrow = A.rowmap ? ldro(A.rowmap + v) : v;
    spmv_row_body<true>(A, vals, lane, vrow, j0, j1, pol, src, a0, a1, a2);
  } else {
    spmv_row_body<false>(A, vals, lane, 0, j0, j1, pol, src, a0, a1, a2);
  }
  out[0] = (OT)a0;
  out[1] = (OT)a1;
  out[2] = (OT)a2;
}

// Two products with one pass over A (both FP64).
template <typename S1, typename S2>
__device__ __forceinline__ void spmv2_row(const SellMatrix &A, int v, const S1 &s1, const S2 &s2,
                                          double o1[3], double o2[3]) {
  const int s = v >> 5, lane = v & 31;
  const int j0 = ldro(A.slice_off + s), j1 = ldro(A.slice_off + s + 1);
  const unsigned long long pol = l2_policy(A.stream_l2);
  double a0 = 0, a1 = 0, a2 = 0, b0 = 0, b1 = 0, b2 = 0;
  for (int jb = j0; jb < j1; jb += 4) {
    int c[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) c[u] = (jb + u < j1) ? checked_col(A, ldro_pol(A.cols + (size_t)(jb + u) * kSlice + lane, pol)) : -1;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (c[u] < 0) break;
      double m[9];
      ld_block(A.v64, (size_t)(jb + u), lane, m, pol);
      double x[3], y[3];
      s1(c[u], x);
      s2(c[u], y);
      a0 = fma(m[0], x[0], a0); a0 = fma(m[1], x[1], a0); a0 = fma(m[2], x[2], a0);
      a1 = fma(m[3], x[0], a1); a1 = fma(m[4], x[1], a1); a1 = fma(m[5], x[2], a1);
      a2 = fma(m[6], x[0], a2); a2 = fma(m[7], x[1], a2); a2 = fma(m[8], x[2], a2);
      b0 = fma(m[0], y[0], b0); b0 = fma(m[1], y[1], b0); b0 = fma(m[2], y[2], b0);
      b1 = fma(m[3], y[0], b1); b1 = fma(m[4], y[1], b1); b1 = fma(m[5], y[2], b1);
      b2 = fma(m[6], y[0], b2); b2 = fma(m[7], y[1], b2); b2 = fma(m[8], y[2], b2);
    }
  }
  o1[0] = a0; o1[1] = a1; o1[2] = a2;
  o2[0] = b0; o2[1] = b1; o2[2] = b2;
}

// Same product with this item's block columns and values read from the
// shared-memory stage.
template <typename VT, typename Src, typename OT = double>
__device__ __forceinline__ void spmv_row_staged(const SellMatrix &A, int v, const Src &src,
                                                OT out[3]) {
  const int s = v >> 5, lane = v & 31;
  const int j0 = ldro(A.slice_off + s), j1 = ldro(A.slice_off + s + 1);
  const int base = g_stage_first;
  const int *cs = reinterpret_cast<const int *>(g_stage);
  const VT *vs = reinterpret_cast<const VT *>(g_stage + g_stage_voff);
  VT a0 = 0, a1 = 0, a2 = 0;
  for (int jb = j0; jb < j1; jb += 8) {
    int c[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) c[u] = (jb + u < j1) ? checked_col(A, cs[(jb + u - base) * kSlice + lane]) : -1;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      if (c[u] < 0) break;
      VT xv[3];
      src(c[u], xv);
      VT m[9];
      ld_block_smem(vs, (size_t)(jb + u - base), lane, m);
      const VT x0 = xv[0], x1 = xv[1], x2 = xv[2];
      a0 = fma(m[0], x0, a0); a0 = fma(m[1], x1, a0); a0 = fma(m[2], x2, a0);
      a1 = fma(m[3], x0, a1); a1 = fma(m[4], x1, a1); a1 = fma(m[5], x2, a1);
      a2 = fma(m[6], x0, a2); a2 = fma(m[7], x1, a2); a2 = fma(m[8], x2, a2);
    }
  }
  out[0] = (OT)a0;
  out[1] = (OT)a1;
  out[2] = (OT)a2;
}

template <typename Src64, typename Src32>
__device__ __forceinline__ void spmv_any(const InstDesc &D, bool fp32, int slot, const Src64 &src64,
                                         const Src32 &src32, double out[3]) {
  if (fp32) {
    if (g_staged) spmv_row_staged<float>(D.A, slot, src32, out);
    else spmv_row<float>(D.A, D.A.v32, slot, src32, out);
  } else {
    spmv_row<double>(D.A, D.A.v64, slot, src64, out);
  }
}

// --------------------------------------------------- vertex constraints --
struct VCons {
  int k, base, unit;  // unit: the planes' Gram matrix is the identity (k >= 2)
  int ax;             // 2 bits per plane: 0..2 the normal is that unit axis, 3 any other
  double n[kMaxPlanes][3], c[kMaxPlanes], inn[kMaxPlanes], indn[kMaxPlanes];
  double lo[3], hi[3];
};

__device__ __forceinline__ void load_cons(const InstDesc &D, int v, VCons &C) {
  C.unit = 0;
  C.ax = 0x3f;
  if (D.kind >= KIND_DECOUPLED) {
    int b = ldro(D.plane_ptr + v), e = ldro(D.plane_ptr + v + 1);
    MPRGP_CHECK(b >= 0 && e >= b && e - b <= kMaxPlanes && e <= D.m, D.A.bad, 4, (b = 0, e = 0));
    C.base = b;
    C.k = e - b;
    if (D.pl_unit && C.k >= 2) C.unit = D.pl_unit[v];
    if (D.pl_axis) {
#pragma unroll
      for (int j = 0; j < kMaxPlanes; ++j)
        if (j < C.k) C.ax = (C.ax & ~(3 << (2 * j))) | ((int)(__ldg(D.pl_axis + b + j) & 3) << (2 * j));
    }
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j) {
      if (j < C.k) {
        const double *q = D.planes + 4 * (size_t)(b + j);
        C.n[j][0] = ldro(q);
        C.n[j][1] = ldro(q + 1);
        C.n[j][2] = ldro(q + 2);
        C.c[j] = ldro(q + 3);
        C.inn[j] = ldro(D.pl_nn + b + j);
        C.indn[j] = ldro(D.pl_indn + b + j);
      } else {
        C.n[j][0] = C.n[j][1] = C.n[j][2] = C.c[j] = 0.0;
        C.inn[j] = 1.0;
        C.indn[j] = 0.0;
      }
    }
  } else {
    C.base = 3 * v;
    C.k = 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      C.lo[d] = ldro(D.L + 3 * (size_t)v + d);
      C.hi[d] = (D.kind == KIND_BOX) ? ldro(D.U + 3 * (size_t)v + d) : DBL_MAX;
    }
  }
}

// Plane products.  A plane whose normal is a unit axis vector (floor and
// walls) needs no FP64 work for them: n.v is one component of v, v += n s
// changes one component, and 1/|n|^2 is 1.  The results are the general
// forms' (0 * v_d and v_d + 0 * s leave v_d's value; only the sign of an
// exact zero can differ), and every GPU path uses these same functions.
__device__ __forceinline__ int ax_of(const VCons &C, int j) { return (C.ax >> (2 * j)) & 3; }
__device__ __forceinline__ double ndot(const VCons &C, int j, const double v[3]) {
  const int a = ax_of(C, j);
  if (a == 3) return dot3(C.n[j], v);
  return a == 0 ? v[0] : (a == 1 ? v[1] : v[2]);
}
// x / |n_j|^2 (C.inn is 1/|n|^2; exactly 1 for a unit axis)
__device__ __forceinline__ double ninn(const VCons &C, int j, double x) {
  return ax_of(C, j) == 3 ? x * C.inn[j] : x;
}
// v += n_j s
__device__ __forceinline__ void nadd(const VCons &C, int j, double s, double v[3]) {
  const int a = ax_of(C, j);
  if (a == 3) {
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] += C.n[j][d] * s;
  } else if (a == 0) {
    v[0] += s;
  } else if (a == 1) {
    v[1] += s;
  } else {
    v[2] += s;
  }
}
// v -= n_j s
__device__ __forceinline__ void nsub(const VCons &C, int j, double s, double v[3]) {
  const int a = ax_of(C, j);
  if (a == 3) {
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] -= C.n[j][d] * s;
  } else if (a == 0) {
    v[0] -= s;
  } else if (a == 1) {
    v[1] -= s;
  } else {
    v[2] -= s;
  }
}

// Face codes of the vertex's constraint rows, 2 bits each.
__device__ __forceinline__ int load_face(const InstDesc &D, const VCons &C) {
  int f = 0;
#pragma unroll
  for (int j = 0; j < 3; ++j)
    if (j < C.k) f |= (int)D.face[C.base + j] << (2 * j);
  return f;
}
__device__ __forceinline__ int fcode(int f, int j) { return (f >> (2 * j)) & 3; }

// DECIDE_FACE (MPRGPProjection.h:78-90, 187-201, 283-297).  Returns the sum
// of the codes (COUNT_CONSTRAINTS, MPRGPUtility.h:98-106).
__device__ __forceinline__ int decide_face(const InstDesc &D, const VCons &C, const double x[3],
                                           int &f) {
  f = 0;
  int cnt = 0;
  if (D.kind >= KIND_DECOUPLED) {
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j) {
      if (j < C.k) {
        const int a = fabs(ndot(C, j, x) - C.c[j]) < kEps ? 1 : 0;
        f |= a << (2 * j);
        cnt += a;
        D.face[C.base + j] = (unsigned char)a;
      }
    }
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int a = 0;
      if (fabs(x[d] - C.lo[d]) < kEps) a = 2;
      else if (D.kind == KIND_BOX && fabs(x[d] - C.hi[d]) < kEps) a = 1;
      f |= a << (2 * d);
      cnt += a;
      D.face[C.base + d] = (unsigned char)a;
    }
  }
  return cnt;
}

// Whether the Gram matrix restricted to the planes in `mask` is exactly the
// identity (mutually orthogonal unit normals, e.g. axis-aligned floor and
// walls): the small QPs below then separate by plane.
__device__ __forceinline__ bool unit_gram(const double G[3][3], int mask) {
  bool id = true;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (((mask >> i) & 1) && ((mask >> j) & 1)) id &= (i == j) ? G[i][j] == 1.0 : G[i][j] == 0.0;
  return id;
}

// Small SPD solve on the planes selected by `mask` (<= 3), Cramer's rule
// (with G the identity on `mask`, Cramer's rule gives lam = q there).
__device__ __forceinline__ bool solve_subset(const double G[3][3], const double q[3], int mask,
                                             double lam[3]) {
  lam[0] = lam[1] = lam[2] = 0.0;
  if (unit_gram(G, mask)) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
      if ((mask >> i) & 1) lam[i] = q[i];
    return true;
  }
  int idx[3], s = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if (mask & (1 << i)) idx[s++] = i;
  if (s == 1) {
    const int a = idx[0];
    if (!(G[a][a] > 0.0)) return false;
    lam[a] = q[a] / G[a][a];
  } else if (s == 2) {
    const int a = idx[0], b = idx[1];
    const double det = G[a][a] * G[b][b] - G[a][b] * G[b][a];
    if (!(det > 0.0)) return false;
    lam[a] = (q[a] * G[b][b] - G[a][b] * q[b]) / det;
    lam[b] = (G[a][a] * q[b] - G[b][a] * q[a]) / det;
  } else if (s == 3) {
    const double c00 = G[1][1] * G[2][2] - G[1][2] * G[2][1];
    const double c01 = G[1][2] * G[2][0] - G[1][0] * G[2][2];
    const double c02 = G[1][0] * G[2][1] - G[1][1] * G[2][0];
    const double det = G[0][0] * c00 + G[0][1] * c01 + G[0][2] * c02;
    if (!(det > 0.0)) return false;
    const double c10 = G[0][2] * G[2][1] - G[0][1] * G[2][2];
    const double c11 = G[0][0] * G[2][2] - G[0][2] * G[2][0];
    const double c12 = G[0][1] * G[2][0] - G[0][0] * G[2][1];
    const double c20 = G[0][1] * G[1][2] - G[0][2] * G[1][1];
    const double c21 = G[0][2] * G[1][0] - G[0][0] * G[1][2];
    const double c22 = G[0][0] * G[1][1] - G[0][1] * G[1][0];
    lam[0] = (c00 * q[0] + c10 * q[1] + c20 * q[2]) / det;
    lam[1] = (c01 * q[0] + c11 * q[1] + c21 * q[2]) / det;
    lam[2] = (c02 * q[0] + c12 * q[1] + c22 * q[2]) / det;
  }
  return true;
}

// nonneg_qp3 for G = I on `allow` (planes flagged orthonormal beforehand):
// the same scale, tolerance and multipliers without forming G.
__device__ __forceinline__ void unit_qp3(const double q[3], int allow, double lam[3]) {
  double scale = 1e-300;
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if (allow & (1 << i)) scale = fmax(scale, fabs(q[i]));
  const double tol = 1e-12 * scale;
#pragma unroll
  for (int i = 0; i < 3; ++i) lam[i] = (((allow >> i) & 1) && q[i] > tol) ? q[i] : 0.0;
}

// min 0.5 l^T G l - q^T l, l >= 0 over the planes in `allow` (bit mask), by
// enumerating supports in order of size, then mask value; the first support
// that satisfies KKT wins.  Same procedure as the oracle's per-block solver
// for solveQP(G, q, I, 0, l) (SimpleQP.h:17-48).
__device__ __forceinline__ void nonneg_qp3(const double G[3][3], const double q[3], int allow,
                                           double lam[3]) {
  double scale = 1e-300;
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if (allow & (1 << i)) scale = fmax(scale, fabs(q[i]));
  const double tol = 1e-12 * scale;
  if (unit_gram(G, allow)) {
    // Separable: the enumeration below would stop at the support
    // {i : q_i > tol} (smaller supports leave a q_i > tol unmet, larger ones
    // come later), whose solution is lam_i = q_i there and 0 elsewhere.
#pragma unroll
    for (int i = 0; i < 3; ++i) lam[i] = (((allow >> i) & 1) && q[i] > tol) ? q[i] : 0.0;
    return;
  }
  double best_viol = DBL_MAX, best[3] = {0.0, 0.0, 0.0};
  // Supports are subsets of `allow`; visit them by popcount, then value.
  for (int size = 0; size <= 3; ++size) {
    for (int mask = 0; mask < 8; ++mask) {
      if ((mask & ~allow) || __popc(mask) != size) continue;
      double t[3];
      if (!solve_subset(G, q, mask, t)) continue;
      double viol = 0.0;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        if (!(allow & (1 << i))) continue;
        if (mask & (1 << i)) {
          viol = fmax(viol, -t[i]);
        } else {
          const double gr = G[i][0] * t[0] + G[i][1] * t[1] + G[i][2] * t[2] - q[i];
          viol = fmax(viol, -gr);
        }
      }
      if (viol <= tol) {
        lam[0] = fmax(t[0], 0.0);
        lam[1] = fmax(t[1], 0.0);
        lam[2] = fmax(t[2], 0.0);
        return;
      }
      if (viol < best_viol) {
        best_viol = viol;
        best[0] = t[0];
        best[1] = t[1];
        best[2] = t[2];
      }
    }
  }
  lam[0] = fmax(best[0], 0.0);
  lam[1] = fmax(best[1], 0.0);
  lam[2] = fmax(best[2], 0.0);
}

__device__ __forceinline__ void gram(const VCons &C, double G[3][3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) G[a][b] = dot3(C.n[a], C.n[b]);
}

// project (MPRGPProjection.h:56-62, 163-169, 333-348, 412-430).
__device__ void project_v(const InstDesc &D, const VCons &C, const double x[3], double y[3]) {
  y[0] = x[0];
  y[1] = x[1];
  y[2] = x[2];
  if (D.kind == KIND_DECOUPLED) {
    double lam[kMaxPlanes];
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j)
      lam[j] = (j < C.k) ? fmax(ninn(C, j, C.c[j] - ndot(C, j, x)), 0.0) : 0.0;
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j)
      if (j < C.k)
        nadd(C, j, lam[j], y);
  } else if (D.kind == KIND_PLANES) {
    if (C.k == 0) return;
    if (C.k == 1) {  // one constraint: the QP's solution is max(q, 0) / |n|^2
      const double l = fmax(ninn(C, 0, C.c[0] - ndot(C, 0, x)), 0.0);
      nadd(C, 0, l, y);
      return;
    }
    double G[3][3], q[3], lam[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) q[j] = (j < C.k) ? C.c[j] - ndot(C, j, x) : 0.0;
    if (C.unit) unit_qp3(q, (1 << C.k) - 1, lam);  // what nonneg_qp3 returns for G = I
    else {
      gram(C, G);
      nonneg_qp3(G, q, (1 << C.k) - 1, lam);
    }
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (j < C.k)
        nadd(C, j, lam[j], y);
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) y[d] = fmin(fmax(x[d], C.lo[d]), C.hi[d]);
  }
}

// PHI (MPRGPProjection.h:63-65, 170-172, 349-367, 431-449).
__device__ void phi_v(const InstDesc &D, const VCons &C, int f, const double g[3],
                      double phi[3]) {
  phi[0] = g[0];
  phi[1] = g[1];
  phi[2] = g[2];
  if (D.kind == KIND_DECOUPLED) {
    double lam[kMaxPlanes];
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j)
      lam[j] = (j < C.k && fcode(f, j)) ? ninn(C, j, -ndot(C, j, g)) : 0.0;
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j)
      if (j < C.k)
        nadd(C, j, lam[j], phi);
  } else if (D.kind == KIND_PLANES) {
    int act = 0;
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j)
      if (j < C.k && fcode(f, j)) act |= 1 << j;
    if (!act) return;
    if (__popc(act) == 1) {
      const int j = __ffs(act) - 1;
      const double l = ninn(C, j, -ndot(C, j, g));
      nadd(C, j, l, phi);
      return;
    }
    double G[3][3], q[3], lam[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) q[j] = (act & (1 << j)) ? -ndot(C, j, g) : 0.0;
    if (C.unit) {  // what solve_subset returns for G = I
#pragma unroll
      for (int j = 0; j < 3; ++j) lam[j] = (act & (1 << j)) ? q[j] : 0.0;
    } else {
      gram(C, G);
      if (!solve_subset(G, q, act, lam)) return;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (act & (1 << j))
        nadd(C, j, lam[j], phi);
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (fcode(f, d)) phi[d] = 0.0;
  }
}

// BETA (MPRGPProjection.h:66-77, 173-186, 368-383, 450-467).
__device__ void beta_v(const InstDesc &D, const VCons &C, int f, const double g[3],
                       const double phi[3], double beta[3]) {
  if (D.kind == KIND_DECOUPLED) {
#pragma unroll
    for (int d = 0; d < 3; ++d) beta[d] = g[d] - phi[d];
    double lam[kMaxPlanes];
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j) {
      double l = (j < C.k) ? ndot(C, j, beta) : 0.0;
      if (j < C.k && fcode(f, j)) l = fmax(0.0, ninn(C, j, l));
      lam[j] = l;  // rows off the face keep (J beta)_i, as the reference does
    }
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j)
      if (j < C.k)
        nsub(C, j, lam[j], beta);
  } else if (D.kind == KIND_PLANES) {
#pragma unroll
    for (int d = 0; d < 3; ++d) beta[d] = g[d] - phi[d];
    int act = 0;
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j)
      if (j < C.k && fcode(f, j)) act |= 1 << j;
    if (!act) return;
    if (__popc(act) == 1) {
      const int j = __ffs(act) - 1;
      const double l = ninn(C, j, fmax(ndot(C, j, beta), 0.0));
      nsub(C, j, l, beta);
      return;
    }
    double G[3][3], q[3], lam[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) q[j] = (act & (1 << j)) ? ndot(C, j, beta) : 0.0;
    if (C.unit) unit_qp3(q, act, lam);
    else {
      gram(C, G);
      nonneg_qp3(G, q, act, lam);
    }
    double gp[3] = {beta[0], beta[1], beta[2]};
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (act & (1 << j))
        nadd(C, j, -lam[j], gp);
    beta[0] = gp[0];
    beta[1] = gp[1];
    beta[2] = gp[2];
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int fc = fcode(f, d);
      if (fc == 0) beta[d] = 0.0;
      else if (fc == 1) beta[d] = fmax(g[d], 0.0);
      else beta[d] = fmin(g[d], 0.0);
    }
  }
}

// Preconditioner solve (MPRGPPrecondition.h:52-64, 91-105).
__device__ void precond_v(const InstDesc &D, const VCons &C, int f, int v, const double g[3],
                          const double phi[3], double z[3]) {
  if (D.pre == PRE_NONE || (D.pre == PRE_DECOUPLE && D.m == 0)) {
    z[0] = phi[0];
    z[1] = phi[1];
    z[2] = phi[2];
    return;
  }
  double di[3];
  di[0] = ldro(D.dinv + 3 * (size_t)v);
  di[1] = ldro(D.dinv + 3 * (size_t)v + 1);
  di[2] = ldro(D.dinv + 3 * (size_t)v + 2);
  if (D.pre == PRE_INFACE) {
#pragma unroll
    for (int d = 0; d < 3; ++d) z[d] = phi[d] * di[d];
    return;
  }
  double Dg[3] = {di[0] * g[0], di[1] * g[1], di[2] * g[2]};
  double t[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int j = 0; j < kMaxPlanes; ++j) {
    if (j < C.k && fcode(f, j)) {
      const double lam = C.indn[j] * ndot(C, j, Dg);
      nadd(C, j, lam, t);
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) z[d] = Dg[d] - di[d] * t[d];
}

// Per-row term of PHITPHI (MPRGPProjection.h:91-106, 202-221, 384-393): for
// planes (x - P(x - abar phi)) . phi, scaled and clamped once in the finalizer.
__device__ double phitphi_v(const InstDesc &D, const VCons &C, double abar, const double x[3],
                            const double phi[3]) {
  if (D.kind >= KIND_DECOUPLED) {
    const double xa[3] = {x[0] - abar * phi[0], x[1] - abar * phi[1], x[2] - abar * phi[2]};
    double px[3];
    project_v(D, C, xa, px);
    return (x[0] - px[0]) * phi[0] + (x[1] - px[1]) * phi[1] + (x[2] - px[2]) * phi[2];
  }
  double s = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double t = 0.0;
    if (phi[d] > 0.0 && x[d] > C.lo[d]) t = fmin((x[d] - C.lo[d]) / abar, phi[d]);
    else if (D.kind == KIND_BOX && phi[d] < 0.0 && x[d] < C.hi[d])
      t = fmax((x[d] - C.hi[d]) / abar, phi[d]);
    s += t * phi[d];
  }
  return s;
}

// isFeasible with the eps slack (MPRGPProjection.h:108-116, 223-232, 298-310).
__device__ __forceinline__ int infeasible_v(const InstDesc &D, const VCons &C, const double y[3]) {
  if (D.kind >= KIND_DECOUPLED) {
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j)
      if (j < C.k && ndot(C, j, y) < C.c[j] - kEps) return 1;
    return 0;
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (y[d] < C.lo[d] - kEps) return 1;
    if (D.kind == KIND_BOX && y[d] > C.hi[d] + kEps) return 1;
  }
  return 0;
}

// stepLimit (MPRGPProjection.h:34-53, 139-162, 263-282), per-row minimum.
__device__ double ratio_v(const InstDesc &D, const VCons &C, const double x[3], const double p[3]) {
  double r = DBL_MAX;
  if (D.kind >= KIND_DECOUPLED) {
#pragma unroll
    for (int j = 0; j < kMaxPlanes; ++j) {
      if (j >= C.k) continue;
      const double jd = ndot(C, j, p), jx = ndot(C, j, x);
      if (jd > kEps && jx > C.c[j]) r = fmin(r, (jx - C.c[j]) / jd);
    }
    return r;
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (p[d] > kEps && x[d] > C.lo[d]) r = fmin(r, (x[d] - C.lo[d]) / p[d]);
    else if (D.kind == KIND_BOX && p[d] < -kEps && x[d] < C.hi[d])
      r = fmin(r, (x[d] - C.hi[d]) / p[d]);
  }
  return r;
}

__device__ __forceinline__ double *B(const InstDesc &D, int i) { return D.buf[i]; }

// Shared epilogue once g is final for a row and the face is re-decided:
// DECIDE_FACE(x); PHI(g); z = precond; p = z; then the loop top's BETA and
// the sums |phi+beta|^2, beta.beta, PHITPHI, z.g, COUNT_CONSTRAINTS.
__device__ void epilogue_full(const InstDesc &D, const InstState &S, const VCons &C, int v,
                              const double x[3], const double g[3], double *part) {
  int f;
  const int act = decide_face(D, C, x, f);
  double phi[3], z[3], beta[3];
  phi_v(D, C, f, g, phi);
  precond_v(D, C, f, v, g, phi, z);
  beta_v(D, C, f, g, phi, beta);
  st3(B(D, B_G0 + S.gc), v, g);
  st3(B(D, B_Z0 + S.zc), v, z);
  st3(B(D, B_P0 + S.pc), v, z);
  if (D.prec == PREC_MIXED) {
    st3f(D.buf32[F_Z0 + S.zc], v, z);
    st3f(D.buf32[F_P0 + S.pc], v, z);
  }
  st3(B(D, B_BT0 + S.bc), v, beta);
  const double gp[3] = {phi[0] + beta[0], phi[1] + beta[1], phi[2] + beta[2]};
  part[0] += dot3(gp, gp);
  part[1] += dot3(beta, beta);
  part[2] += phitphi_v(D, C, S.alpha_bar, x, phi);
  part[3] += dot3(z, g);
  part[4] += (double)act;
}

// ------------------------------------------------------------- row work --
// Mixed form of the power method: the iterate t_k and w = A t_k live only in
// FP32 (A is FP32 in this form), products and per-row sums in FP32, the
// block and instance sums (norms, the convergence test) in FP64.  t_k uses
// the FP32 shadows of z (F_Z0/F_Z1), which are idle until PH_INIT.
__device__ __forceinline__ void ld3f(const float *b, int v, float o[3]) {
  const float *q = b + 3 * (size_t)v;
  o[0] = q[0];
  o[1] = q[1];
  o[2] = q[2];
}
__device__ __forceinline__ void st3ff(float *b, int v, const float o[3]) {
  float *q = b + 3 * (size_t)v;
  q[0] = o[0];
  q[1] = o[1];
  q[2] = o[2];
}

// The matrix product of a power iteration's row before its scaling: A times
// the stored source vector `src` (a buffer id, or < 0 for the stored start
// vector ev) -- FP32 for the mixed form, FP64 otherwise.  It depends on the
// source alone, so a row can form it before the phase's scale 1/||w|| is
// known.
__device__ __forceinline__ void pow_raw32(const InstDesc &D, int src, int slot, float w[3]) {
  if (src < 0) {
    spmv_row<float, SrcVtoF, float>(D.A, D.A.v32, slot, SrcVtoF{D.ev}, w);
  } else {
    const SrcF s{D.buf32[src == B_W ? F_W0 : F_W1]};
    if (g_staged) spmv_row_staged<float, SrcF, float>(D.A, slot, s, w);
    else spmv_row<float, SrcF, float>(D.A, D.A.v32, slot, s, w);
  }
}
__device__ __forceinline__ void pow_raw64(const InstDesc &D, int src, int slot, double w[3]) {
  spmv_any(D, false, slot, SrcV{src < 0 ? D.ev : B(D, src)}, SrcF{nullptr}, w);
}

// The rest of an FP32 power row given its raw product wr (unused in
// PH_POW_LAST).
__device__ __forceinline__ void row_power32_fin(const InstDesc &D, const InstState &S, int v,
                                                const float wr[3], double *part) {
  const int k = S.pow_k;
  const float sc = (float)S.pow_scale;  // 1/||w|| (tmpOut /= norm)
  float u[3];
  if (S.pow_src < 0) {  // the stored start vector (FP64)
    double e[3];
    ld3(D.ev, v, e);
    u[0] = (float)e[0];
    u[1] = (float)e[1];
    u[2] = (float)e[2];
  } else {
    ld3f(D.buf32[S.pow_src == B_W ? F_W0 : F_W1], v, u);
  }
  u[0] *= sc;
  u[1] *= sc;
  u[2] *= sc;
  if (S.phase == PH_POW_LAST || k >= 1) {
    float t[3];
    ld3f(D.buf32[F_Z0 + ((k - 1) & 1)], v, t);
    const float d0 = u[0] - t[0], d1 = u[1] - t[1], d2 = u[2] - t[2];
    part[0] += (double)fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
  }
  if (S.phase == PH_POW_LAST) return;
  st3ff(D.buf32[F_Z0 + (k & 1)], v, u);
  float w[3] = {wr[0], wr[1], wr[2]};
  w[0] *= sc;
  w[1] *= sc;
  w[2] *= sc;
  st3ff(D.buf32[(k & 1) ? F_W1 : F_W0], v, w);
  part[1] += (double)fmaf(w[0], w[0], fmaf(w[1], w[1], w[2] * w[2]));
}

__device__ __noinline__ void row_power32(const InstDesc &D, const InstState &S, int v, int slot,
                                         double *part) {
  float w[3] = {0.f, 0.f, 0.f};
  if (S.phase != PH_POW_LAST) pow_raw32(D, S.pow_src, slot, w);
  row_power32_fin(D, S, v, w, part);
}

// PH_POW_RAND's row: the seeded start vector (tmp.setRandom()).
__device__ __forceinline__ void row_power_rand(const InstDesc &D, int v, double *part) {
  double t[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) t[d] = seeded_uniform(D.seed, 3ull * v + d);
  st3(B(D, B_W1), v, t);
  if (D.prec == PREC_MIXED) st3f(D.buf32[F_W1], v, t);
  part[0] += dot3(t, t);
}

// The rest of an FP64 power row given its raw product wr (unused in
// PH_POW_LAST).
__device__ __forceinline__ void row_power64_fin(const InstDesc &D, const InstState &S, int v,
                                                const double wr[3], double *part) {
  const bool f32 = D.prec == PREC_MIXED;
  const int k = S.pow_k;
  const double *src = S.pow_src < 0 ? D.ev : B(D, S.pow_src);
  double u[3];
  ld3(src, v, u);
  u[0] *= S.pow_scale;  // pow_scale holds 1/||w|| (tmpOut /= norm)
  u[1] *= S.pow_scale;
  u[2] *= S.pow_scale;
  if (S.phase == PH_POW_LAST || k >= 1) {
    double t[3];
    ld3(B(D, B_T0 + ((k - 1) & 1)), v, t);
    const double d[3] = {u[0] - t[0], u[1] - t[1], u[2] - t[2]};
    part[0] += dot3(d, d);
  }
  if (S.phase == PH_POW_LAST) return;
  st3(B(D, B_T0 + (k & 1)), v, u);
  double w[3] = {wr[0], wr[1], wr[2]};
  w[0] *= S.pow_scale;
  w[1] *= S.pow_scale;
  w[2] *= S.pow_scale;
  st3(B(D, (k & 1) ? B_W1 : B_W), v, w);
  if (f32) st3f(D.buf32[(k & 1) ? F_W1 : F_W0], v, w);
  part[1] += dot3(w, w);
}

__device__ __noinline__ void row_power(const InstDesc &D, const InstState &S, int v, int slot,
                                       double *part) {
  const bool f32 = D.prec == PREC_MIXED;
  if (f32 && S.phase != PH_POW_RAND) {
    row_power32(D, S, v, slot, part);
    return;
  }
  if (S.phase == PH_POW_RAND) {
    row_power_rand(D, v, part);
    return;
  }
  double w[3] = {0.0, 0.0, 0.0};
  // A (src / ||w||) = (A src) / ||w||; the stored start vector ev and every
  // source of the FP64 form take the FP64 pass
  if (S.phase != PH_POW_LAST) pow_raw64(D, S.pow_src, slot, w);
  row_power64_fin(D, S, v, w, part);
}

__device__ __noinline__ void row_init(const InstDesc &D, const InstState &S, int v, int slot,
                                      double *part) {
  VCons C;
  load_cons(D, v, C);
  if (S.phase == PH_PROJ0 || S.phase == PH_FINAL) {
    double x[3], y[3];
    ld3(B(D, B_X0 + S.xc), v, x);
    project_v(D, C, x, y);
    st3(B(D, B_X0 + S.xc), v, y);
    return;
  }
  // PH_INIT, PH_EXP_C, PH_PL_EXP_B: g = A x - b, then the full epilogue.
  if (S.phase == PH_INIT && S.ev_upd) {
    double t[3];
    if (D.prec == PREC_MIXED) {
      float f[3];
      ld3f(D.buf32[F_Z0 + (S.ev_src - B_T0)], v, f);
      t[0] = f[0];
      t[1] = f[1];
      t[2] = f[2];
    } else {
      ld3(B(D, S.ev_src), v, t);
    }
    st3(D.ev, v, t);
  }
  double x[3], ax[3];
  ld3(B(D, B_X0 + S.xc), v, x);
  spmv_row<double>(D.A, D.A.v64, slot, SrcV{B(D, B_X0 + S.xc)}, ax);
  const double g[3] = {ax[0] - ldro(D.b + 3 * (size_t)v), ax[1] - ldro(D.b + 3 * (size_t)v + 1),
                       ax[2] - ldro(D.b + 3 * (size_t)v + 2)};
  epilogue_full(D, S, C, v, x, g, part);
}

__device__ __noinline__ void row_cg_spmv(const InstDesc &D, const InstState &S, int v, int slot,
                                         double *part) {
  const bool f32 = D.prec == PREC_MIXED;
  double p[3], ap[3], g[3];
  ld3(B(D, B_G0 + S.gc), v, g);
  if (S.phase == PH_CG_ENTRY || (S.phase == PH_PL_SPMV && S.p_is_z)) {
    const double *pp = B(D, B_P0 + S.pc);
    ld3(pp, v, p);
    if (S.phase == PH_CG_ENTRY && !S.g_cons) {
      double ax[3];
      spmv_row<double>(D.A, D.A.v64, slot, SrcV{B(D, B_X0 + S.xc)}, ax);
      double e[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) e[d] = (ax[d] - ldro(D.b + 3 * (size_t)v + d)) - g[d];
      st3(B(D, B_E), v, e);
      part[2] += dot3(p, e);
    }
    spmv_any(D, f32 && S.phase != PH_PL_SPMV, slot, SrcV{pp},
             SrcF{f32 ? D.buf32[F_P0 + S.pc] : nullptr}, ap);
  } else {
    const double *zz = B(D, B_Z0 + S.zc), *po = B(D, B_P0 + S.pc);
    double z[3];
    ld3(zz, v, z);
    ld3(po, v, p);
#pragma unroll
    for (int d = 0; d < 3; ++d) p[d] = z[d] - S.beta_cg * p[d];
    st3(B(D, B_P0 + (S.pc ^ 1)), v, p);
    const bool f32p = f32 && S.phase != PH_PL_SPMV;
    if (f32p) st3f(D.buf32[F_P0 + (S.pc ^ 1)], v, p);
    spmv_any(D, f32p, slot, SrcPNew{zz, po, S.beta_cg},
             SrcPNewF{f32p ? D.buf32[F_Z0 + S.zc] : nullptr,
                      f32p ? D.buf32[F_P0 + S.pc] : nullptr, (float)S.beta_cg}, ap);
    if (S.e_nz && S.phase == PH_CG_SPMV) {
      double e[3];
      ld3(B(D, B_E), v, e);
      part[2] += dot3(p, e);
    }
  }
  st3(B(D, B_AP), v, ap);
  part[0] += dot3(p, ap);
  part[1] += dot3(p, g);
  if (S.phase == PH_PL_SPMV) {
    VCons C;
    load_cons(D, v, C);
    double x[3];
    ld3(B(D, B_X0 + S.xc), v, x);
    part[kMinSlot] = fmin(part[kMinSlot], ratio_v(D, C, x, p));
  }
}

// Candidate y = x - alpha p: feasibility, the f(P(y)) correction terms and
// the CG state that committing y would produce (CGMonotonicStep, :287-313).
__device__ __noinline__ void row_cg_yf(const InstDesc &D, const InstState &S, int v, int slot,
                                       double *part) {
  VCons C;
  load_cons(D, v, C);
  const int f = load_face(D, C);
  double x[3], p[3], ap[3], g[3];
  ld3(B(D, B_X0 + S.xc), v, x);
  ld3(B(D, B_P0 + S.pc), v, p);
  ld3(B(D, B_AP), v, ap);
  ld3(B(D, B_G0 + S.gc), v, g);
  double y[3], gy[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    y[d] = x[d] - S.alpha * p[d];
    gy[d] = g[d] - S.alpha * ap[d];
  }
  st3(B(D, B_X0 + (S.xc ^ 1)), v, y);
  st3(B(D, B_G0 + (S.gc ^ 1)), v, gy);
  double py[3];
  project_v(D, C, y, py);
  const double dl[3] = {py[0] - y[0], py[1] - y[1], py[2] - y[2]};
  st3(B(D, B_W), v, dl);
  if (dl[0] != 0.0 || dl[1] != 0.0 || dl[2] != 0.0) {
    double gt[3] = {gy[0], gy[1], gy[2]};
    if (S.e_nz) {
      double e[3];
      ld3(B(D, B_E), v, e);
      gt[0] += e[0];
      gt[1] += e[1];
      gt[2] += e[2];
    }
    part[0] += dot3(dl, gt);
    part[1] += 1.0;
  }
  part[2] += (double)infeasible_v(D, C, y);
  double phi[3], z[3], beta[3];
  phi_v(D, C, f, gy, phi);
  precond_v(D, C, f, v, gy, phi, z);
  beta_v(D, C, f, gy, phi, beta);
  st3(B(D, B_Z0 + (S.zc ^ 1)), v, z);
  if (D.prec == PREC_MIXED) st3f(D.buf32[F_Z0 + (S.zc ^ 1)], v, z);
  st3(B(D, B_BT0 + (S.bc ^ 1)), v, beta);
  const double gp[3] = {phi[0] + beta[0], phi[1] + beta[1], phi[2] + beta[2]};
  part[3] += dot3(z, ap);
  part[4] += dot3(z, gy);
  part[5] += dot3(gp, gp);
  part[6] += dot3(beta, beta);
  part[7] += phitphi_v(D, C, S.alpha_bar, y, phi);
}

// delta^T A delta over the rows where P(y) moved y (rare).
__device__ __noinline__ void row_cg_dad(const InstDesc &D, const InstState &S, int v, int slot,
                                        double *part) {
  (void)S;
  double dl[3];
  ld3(B(D, B_W), v, dl);
  if (dl[0] == 0.0 && dl[1] == 0.0 && dl[2] == 0.0) return;
  double ad[3];
  spmv_row<double>(D.A, D.A.v64, slot, SrcV{B(D, B_W)}, ad);
  part[0] += dot3(dl, ad);
}

// FP64 residual replacement for the mixed form: g = A64 x - b with the face
// kept, then phi, z, beta and the sums for the current x.
__device__ __noinline__ void row_ru(const InstDesc &D, const InstState &S, int v, int slot, double *part) {
  VCons C;
  load_cons(D, v, C);
  const int f = load_face(D, C);
  double x[3], ax[3], ap[3];
  ld3(B(D, B_X0 + S.xc), v, x);
  ld3(B(D, B_AP), v, ap);
  spmv_row<double>(D.A, D.A.v64, slot, SrcV{B(D, B_X0 + S.xc)}, ax);
  const double g[3] = {ax[0] - ldro(D.b + 3 * (size_t)v), ax[1] - ldro(D.b + 3 * (size_t)v + 1),
                       ax[2] - ldro(D.b + 3 * (size_t)v + 2)};
  double phi[3], z[3], beta[3];
  phi_v(D, C, f, g, phi);
  precond_v(D, C, f, v, g, phi, z);
  beta_v(D, C, f, g, phi, beta);
  st3(B(D, B_G0 + S.gc), v, g);
  st3(B(D, B_Z0 + S.zc), v, z);
  st3f(D.buf32[F_Z0 + S.zc], v, z);  // residual replacement runs in the mixed form only
  st3(B(D, B_BT0 + S.bc), v, beta);
  const double gp[3] = {phi[0] + beta[0], phi[1] + beta[1], phi[2] + beta[2]};
  part[0] += dot3(gp, gp);
  part[1] += dot3(beta, beta);
  part[2] += phitphi_v(D, C, S.alpha_bar, x, phi);
  part[3] += dot3(z, g);
  part[4] += dot3(z, ap);
}

__device__ __noinline__ void row_exp(const InstDesc &D, const InstState &S, int v, int slot, double *part) {
  VCons C;
  load_cons(D, v, C);
  if (S.phase == PH_EXP_A) {  // y = P(x)
    double x[3], y[3];
    ld3(B(D, B_X0 + S.xc), v, x);
    project_v(D, C, x, y);
    st3(B(D, B_X0 + (S.xc ^ 1)), v, y);
    return;
  }
  if (S.phase == PH_EXP_B) {  // g = A y - b; DECIDE_FACE(y); PHI; x = P(y - abar phi)
    const double *yb = B(D, B_X0 + (S.xc ^ 1));
    double y[3], ay[3];
    ld3(yb, v, y);
    spmv_row<double>(D.A, D.A.v64, slot, SrcV{yb}, ay);
    const double g[3] = {ay[0] - ldro(D.b + 3 * (size_t)v),
                         ay[1] - ldro(D.b + 3 * (size_t)v + 1),
                         ay[2] - ldro(D.b + 3 * (size_t)v + 2)};
    st3(B(D, B_G0 + S.gc), v, g);
    int f;
    decide_face(D, C, y, f);
    double phi[3];
    phi_v(D, C, f, g, phi);
    const double yn[3] = {y[0] - S.alpha_bar * phi[0], y[1] - S.alpha_bar * phi[1],
                          y[2] - S.alpha_bar * phi[2]};
    part[0] += (double)infeasible_v(D, C, yn);
    double x[3];
    project_v(D, C, yn, x);
    st3(B(D, B_X0 + S.xc), v, x);
    return;
  }
  // PH_PL_EXP_A (ExpStep, :196-218): xt = x - af p; g -= af AP;
  // DECIDE_FACE(xt); PHI(g); x = P(xt - abar phi).
  double x[3], p[3], ap[3], g[3];
  ld3(B(D, B_X0 + S.xc), v, x);
  ld3(B(D, B_P0 + S.pc), v, p);
  ld3(B(D, B_AP), v, ap);
  ld3(B(D, B_G0 + S.gc), v, g);
  double xt[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    xt[d] = x[d] - S.alpha * p[d];
    g[d] -= S.alpha * ap[d];
  }
  st3(B(D, B_G0 + S.gc), v, g);
  int f;
  decide_face(D, C, xt, f);
  double phi[3];
  phi_v(D, C, f, g, phi);
#pragma unroll
  for (int d = 0; d < 3; ++d) xt[d] -= S.alpha_bar * phi[d];
  double xn[3];
  project_v(D, C, xt, xn);
  st3(B(D, B_X0 + S.xc), v, xn);
}

__device__ __noinline__ void row_prop(const InstDesc &D, const InstState &S, int v, int slot,
                                      double *part) {
  const double *db = B(D, B_BT0 + S.bc);
  if (S.phase == PH_PROP_A || S.phase == PH_PL_PROP_A) {
    double dd[3], ad[3], g[3];
    ld3(db, v, dd);
    if (S.phase == PH_PROP_A) {  // g = A x - B and AD = A D in one pass
      double ax[3];
      spmv2_row(D.A, slot, SrcV{B(D, B_X0 + S.xc)}, SrcV{db}, ax, ad);
#pragma unroll
      for (int d = 0; d < 3; ++d) g[d] = ax[d] - ldro(D.b + 3 * (size_t)v + d);
      st3(B(D, B_G0 + S.gc), v, g);
    } else {
      ld3(B(D, B_G0 + S.gc), v, g);
      spmv_row<double>(D.A, D.A.v64, slot, SrcV{db}, ad);
    }
    st3(B(D, B_W), v, ad);
    part[0] += dot3(g, dd);
    part[1] += dot3(dd, ad);
    return;
  }
  // PH_PROP_B (PropStep, :219-243): x = P(x - alpha D); g -= alpha AD.
  VCons C;
  load_cons(D, v, C);
  double x[3], dd[3], ad[3], g[3];
  ld3(B(D, B_X0 + S.xc), v, x);
  ld3(db, v, dd);
  ld3(B(D, B_W), v, ad);
  ld3(B(D, B_G0 + S.gc), v, g);
  double xt[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    xt[d] = x[d] - S.alpha * dd[d];
    g[d] -= S.alpha * ad[d];
  }
  double xn[3];
  project_v(D, C, xt, xn);
  if (xn[0] != xt[0] || xn[1] != xt[1] || xn[2] != xt[2]) part[5] += 1.0;
  st3(B(D, B_X0 + S.xc), v, xn);
  epilogue_full(D, S, C, v, xn, g, part);
}

__device__ __noinline__ void row_pl_cg(const InstDesc &D, const InstState &S, int v, int slot,
                                       double *part) {
  // CGStep (:182-195) then the loop top's BETA and sums.
  VCons C;
  load_cons(D, v, C);
  const int f = load_face(D, C);
  double x[3], p[3], ap[3], g[3];
  ld3(B(D, B_X0 + S.xc), v, x);
  ld3(B(D, B_P0 + S.pc), v, p);
  ld3(B(D, B_AP), v, ap);
  ld3(B(D, B_G0 + S.gc), v, g);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    x[d] -= S.alpha * p[d];
    g[d] -= S.alpha * ap[d];
  }
  st3(B(D, B_X0 + S.xc), v, x);
  st3(B(D, B_G0 + S.gc), v, g);
  double phi[3], z[3], beta[3];
  phi_v(D, C, f, g, phi);
  precond_v(D, C, f, v, g, phi, z);
  beta_v(D, C, f, g, phi, beta);
  st3(B(D, B_Z0 + S.zc), v, z);
  st3(B(D, B_BT0 + S.bc), v, beta);
  const double gp[3] = {phi[0] + beta[0], phi[1] + beta[1], phi[2] + beta[2]};
  part[0] += dot3(gp, gp);
  part[1] += dot3(beta, beta);
  part[2] += phitphi_v(D, C, S.alpha_bar, x, phi);
  part[3] += dot3(z, g);
  part[5] += dot3(z, ap);
}

__device__ void row_op(const InstDesc &D, const InstState &S, int v, int slot, double *part) {
  switch (S.phase) {
    case PH_POW_RAND:
    case PH_POW:
    case PH_POW_LAST: row_power(D, S, v, slot, part); break;
    case PH_PROJ0:
    case PH_FINAL:
    case PH_INIT:
    case PH_EXP_C:
    case PH_PL_EXP_B: row_init(D, S, v, slot, part); break;
    case PH_CG_ENTRY:
    case PH_CG_SPMV:
    case PH_PL_SPMV: row_cg_spmv(D, S, v, slot, part); break;
    case PH_CG_YF: row_cg_yf(D, S, v, slot, part); break;
    case PH_CG_DAD: row_cg_dad(D, S, v, slot, part); break;
    case PH_RU: row_ru(D, S, v, slot, part); break;
    case PH_EXP_A:
    case PH_EXP_B:
    case PH_PL_EXP_A: row_exp(D, S, v, slot, part); break;
    case PH_PROP_A:
    case PH_PROP_B:
    case PH_PL_PROP_A: row_prop(D, S, v, slot, part); break;
    case PH_PL_CG: row_pl_cg(D, S, v, slot, part); break;
    default: break;
  }
}

// ------------------------------------------------------ state transitions --
__device__ __forceinline__ double ptp_value(const InstDesc &D, const InstState &S, double s) {
  if (D.kind >= KIND_DECOUPLED) {  // ((x-px).phi)*(1/abar), clamped at 0
    const double v = s * (1.0 / S.alpha_bar);
    return v > 0.0 ? v : 0.0;
  }
  return s;
}

// Step trace record {event, iteration, residual, value}: 1 CG commit and
// 2 CG exit (value f(P(y)) - f(x)), 3 expansion, 4 proportioning, 5 loop top
// (value = proportional).  The CPU oracle records the same events.
__device__ __forceinline__ void trace(const InstDesc &D, InstState &S, int ev, double val) {
  if (D.trace && S.trace_n < D.trace_cap) {
    double *r = D.trace + 4 * (size_t)S.trace_n;
    r[0] = ev;
    r[1] = S.iteration;
    r[2] = S.residual;
    r[3] = val;
    S.trace_n++;
  }
}

__device__ void go_final(const InstDesc &D, InstState &S) {
  if (D.alg == ALG_MONOTONE) {
    S.phase = PH_FINAL;
  } else {  // MPRGP::solve has no final projection
    S.code = S.residual <= D.tol ? 0 : -1;
    S.phase = PH_DONE;
  }
}

// Top of MPRGPMonotonic::solve's loop (:416-440) after a step that ended with
// the loop-top sums s[0..4].
__device__ void outer_top(const InstDesc &D, InstState &S, const double *s) {
  S.active = (int)s[4];
  if (S.iteration >= D.max_it) { go_final(D, S); return; }
  S.residual = sqrt(s[0]);
  if (S.residual != S.residual) {  // NaN: A, b or x carry a NaN; no step can converge
    S.code = -2;                   // MPRGP_BREAKDOWN
    S.phase = PH_DONE;
    return;
  }
  if (S.residual <= D.tol) {
    if (D.alg == ALG_PLAIN) S.iters_out = S.iteration;
    go_final(D, S);
    return;
  }
  S.zg = s[3];
  S.prop = (s[1] <= ptp_value(D, S, s[2])) ? 1 : 0;  // gamma = 1
  trace(D, S, 5, S.prop);
  if (D.alg == ALG_PLAIN) {
    S.phase = S.prop ? PH_PL_SPMV : PH_PL_PROP_A;
    return;
  }
  if (S.prop) {
    S.cg_prop = 1;
    S.ru_ref = S.residual;
    S.phase = PH_CG_ENTRY;
  } else if (!S.y_valid || !S.y_feas) {
    S.phase = PH_EXP_A;
  } else {
    S.phase = PH_PROP_A;
  }
}

// The while-condition of CGMonotonicStep (:288-289) and what follows it.
__device__ void cg_decide(const InstDesc &D, InstState &S, double dfy, double corr) {
  const bool cont = S.cg_prop && S.residual > D.tol && (dfy <= 0.0) && S.iteration < D.max_it;
  if (cont) {
    S.xc ^= 1;
    S.gc ^= 1;
    S.zc ^= 1;
    S.bc ^= 1;
    S.iteration++;
    S.num_cg++;
    S.fx_off = -corr;  // fx := f(P(y)) while x := y
    S.beta_cg = S.s_zap / S.pd;
    S.residual = sqrt(S.s_gp2);
    S.cg_prop = (S.s_bb <= ptp_value(D, S, S.s_ptp)) ? 1 : 0;
    S.zg = S.s_zg;
    trace(D, S, 1, dfy);
    if (D.prec == PREC_MIXED && (S.residual <= D.tol || S.residual < 0.1 * S.ru_ref)) {
      S.phase = PH_RU;
      return;
    }
    if (S.residual <= D.tol) { go_final(D, S); return; }  // loop exits, then `break`
    S.phase = PH_CG_SPMV;
    return;
  }
  trace(D, S, 2, dfy);
  if (S.residual <= D.tol) { go_final(D, S); return; }
  if (S.cg_prop || !S.y_valid || !S.y_feas) S.phase = PH_EXP_A;
  else S.phase = PH_PROP_A;
}

// Transitions of the power method (specRad, MPRGPSolver.h:42-79), shared by
// the persistent engine and the dedicated power kernel.
__device__ void advance_power(const InstDesc &D, InstState &S, const double *s) {
  const double eps = D.tol;  // specRad(A, ev, tol): eps = tol (MPRGPSolver.h:28)
  switch (S.phase) {
    case PH_POW_RAND:
      S.pow_k = 0;
      S.pow_src = B_W1;
      S.pow_scale = 1.0 / sqrt(s[0]);  // tmp.normalize()
      S.phase = PH_POW;
      break;
    case PH_POW: {
      const int k = S.pow_k;
      const double nrm = sqrt(s[1]);
      if (D.prec == PREC_MIXED) S.spmv32++; else S.spmv64++;
      S.pow_spmv++;
      if (k >= 1 && sqrt(s[0]) <= eps) {  // iteration k-1 converged
        S.spec_rad = S.pow_nrm_prev;
        S.ev_upd = 1;
        S.ev_src = B_T0 + ((k - 1) & 1);
        S.power_iters = k - 1;
        S.phase = PH_INIT;
        break;
      }
      if (nrm < kEps) {
        S.spec_rad = kEps;
        S.ev_upd = 1;
        S.ev_src = B_T0 + (k & 1);
        S.power_iters = k;
        S.phase = PH_INIT;
        break;
      }
      S.pow_nrm_prev = nrm;
      S.pow_scale = 1.0 / nrm;
      S.pow_src = (k & 1) ? B_W1 : B_W;
      if (k == 1000) {
        S.pow_k = 1001;
        S.phase = PH_POW_LAST;
      } else {
        S.pow_k = k + 1;
      }
      break;
    }
    case PH_POW_LAST:
      S.spec_rad = S.pow_nrm_prev;
      if (sqrt(s[0]) <= eps) {
        S.ev_upd = 1;
        S.ev_src = B_T0 + (1000 & 1);
        S.power_iters = 1000;
      } else {
        S.power_iters = 1001;
      }
      S.phase = PH_INIT;
      break;
    default:
      break;
  }
  if (S.phase == PH_INIT) {  // leaving the power method
    S.alpha_bar = 2.0 / S.spec_rad;  // MPRGPSolver.h:28
    if (D.project_x0) S.phase = PH_PROJ0;
  }
}

__device__ void advance(const InstDesc &D, InstState &S, const double *s) {
  S.phases++;
  switch (S.phase) {
    case PH_POW_RAND:
    case PH_POW:
    case PH_POW_LAST:
      advance_power(D, S, s);
      break;
    case PH_PROJ0:
      S.phase = PH_INIT;
      break;
    case PH_INIT:
      S.spmv64++;
      S.iteration = 0;
      S.g_cons = 1;
      S.e_nz = 0;
      S.p_is_z = 1;
      outer_top(D, S, s);
      break;
    case PH_CG_ENTRY:
    case PH_CG_SPMV:
      if (S.phase == PH_CG_SPMV) S.pc ^= 1;
      if (D.prec == PREC_MIXED) S.spmv32++; else S.spmv64++;
      if (S.phase == PH_CG_ENTRY) {
        S.fx_off = 0.0;
        if (!S.g_cons) { S.e_nz = 1; S.spmv64++; }
      }
      S.pd = s[0];
      S.pg = s[1];
      S.pe = S.e_nz ? s[2] : 0.0;
      S.alpha = S.zg / S.pd;
      S.phase = PH_CG_YF;
      break;
    case PH_CG_YF: {
      const double a = S.alpha;
      S.dfy = -a * (S.pg + S.pe) + 0.5 * a * a * S.pd;  // f(y) - f(x)
      S.corr = s[0];
      S.y_valid = 1;
      S.y_feas = (s[2] == 0.0) ? 1 : 0;
      S.s_zap = s[3];
      S.s_zg = s[4];
      S.s_gp2 = s[5];
      S.s_bb = s[6];
      S.s_ptp = s[7];
      if (s[1] > 0.0) {
        S.phase = PH_CG_DAD;
      } else {
        cg_decide(D, S, S.dfy + S.fx_off, 0.0);
      }
      break;
    }
    case PH_CG_DAD: {
      S.spmv64++;
      const double corr = S.corr + 0.5 * s[0];  // f(P(y)) - f(y)
      cg_decide(D, S, S.dfy + corr + S.fx_off, corr);
      break;
    }
    case PH_RU:
      S.spmv64++;
      S.e_nz = 0;
      S.g_cons = 1;
      S.residual = sqrt(s[0]);
      S.cg_prop = (s[1] <= ptp_value(D, S, s[2])) ? 1 : 0;
      S.zg = s[3];
      S.beta_cg = s[4] / S.pd;
      S.ru_ref = S.residual;
      if (S.residual <= D.tol) go_final(D, S);
      else S.phase = PH_CG_SPMV;
      break;
    case PH_EXP_A:
      S.phase = PH_EXP_B;
      break;
    case PH_EXP_B:
      S.spmv64++;
      S.y_valid = 1;
      S.y_feas = (s[0] == 0.0) ? 1 : 0;
      S.phase = PH_EXP_C;
      break;
    case PH_EXP_C:
      S.spmv64++;
      S.num_exp++;
      S.iteration++;
      S.g_cons = 1;
      S.e_nz = 0;
      trace(D, S, 3, 0.0);
      outer_top(D, S, s);
      break;
    case PH_PROP_A:
    case PH_PL_PROP_A:
      S.spmv64 += (S.phase == PH_PROP_A) ? 2 : 1;
      S.alpha = s[0] / s[1];
      S.phase = PH_PROP_B;
      break;
    case PH_PROP_B:
      S.num_prop++;
      S.iteration++;
      S.g_cons = (s[5] == 0.0) ? 1 : 0;
      S.e_nz = 0;
      S.p_is_z = 1;
      trace(D, S, 4, 0.0);
      outer_top(D, S, s);
      break;
    case PH_FINAL:
      S.code = S.residual <= D.tol ? 0 : -1;
      S.iters_out = S.iteration;
      S.phase = PH_DONE;
      break;
    case PH_PL_SPMV: {
      S.spmv64++;
      if (!S.p_is_z) S.pc ^= 1;
      S.p_is_z = 0;
      S.pd = s[0];
      const double acg = S.zg / S.pd;
      double af = s[kMinSlot];
      if (D.kind >= KIND_DECOUPLED) {  // BaseGeneralConProjector starts from alpha_cg + eps
        const double a0 = (acg == DBL_MAX) ? acg : acg + kEps;
        af = fmin(a0, af);
      }
      if (acg <= af) {
        S.alpha = acg;
        S.phase = PH_PL_CG;
      } else {
        S.alpha = af;
        S.phase = PH_PL_EXP_A;
      }
      break;
    }
    case PH_PL_CG:
      S.num_cg++;
      S.iteration++;
      S.beta_cg = s[5] / S.pd;
      {
        double t[5] = {s[0], s[1], s[2], s[3], (double)S.active};
        outer_top(D, S, t);
      }
      break;
    case PH_PL_EXP_A:
      S.phase = PH_PL_EXP_B;
      break;
    case PH_PL_EXP_B:
      S.spmv64++;
      S.num_exp++;
      S.iteration++;
      S.p_is_z = 1;
      outer_top(D, S, s);
      break;
    default:
      S.phase = PH_DONE;
      break;
  }
  // A NaN step length in a proportioning or plain step means the iteration
  // broke down (p^T A p or D^T A D was 0); the monotone CG step tolerates it
  // the way the reference does (its comparisons fail and it expands).
  if ((S.phase == PH_PROP_B || S.phase == PH_PL_CG || S.phase == PH_PL_EXP_A) &&
      !(S.alpha == S.alpha)) {
    S.code = -2;
    S.phase = PH_DONE;
  }
}

// -------------------------------------------------------- reductions -----
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Partial sums each phase produces (slot kMinSlot only for PH_PL_SPMV).
__device__ __forceinline__ int nslots(int phase) {
  switch (phase) {
    case PH_POW_RAND: case PH_POW_LAST: case PH_CG_DAD: case PH_EXP_B: return 1;
    case PH_POW: case PH_PROP_A: case PH_PL_PROP_A: case PH_PL_SPMV: return 2;
    case PH_CG_ENTRY: case PH_CG_SPMV: return 3;
    case PH_INIT: case PH_EXP_C: case PH_PL_EXP_B: case PH_RU: return 5;
    case PH_PROP_B: case PH_PL_CG: return 6;
    case PH_CG_YF: return 8;
    default: return 0;
  }
}

// Block reduction of the first `ns` slots of part[] (and the min slot when
// `with_min`; at most kRedSlots slots in all), in a fixed order: every
// thread's values go to shared memory; warp w reduces slot w -- lane l takes
// the values of threads l, l+32, ..., l+224 in that order, then a 5-level
// shuffle tree -- and thread k gets slot k.  One warp per slot keeps the FP64
// work at about a dozen warp instructions per slot (GB300 issues FP64 warp
// instructions slowly), against five per warp and slot for a shuffle tree in
// every warp.
constexpr int kRedSlots = 8;
struct RedBuf {
  double v[kRedSlots][kThreads];
  double out[kRedSlots];
};

__device__ double block_reduce(double *part, RedBuf &red, int ns, bool with_min) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kPart; ++k) {
    if (k == kMinSlot ? !with_min : k >= ns) continue;
    red.v[k == kMinSlot ? ns : k][threadIdx.x] = part[k];
  }
  __syncthreads();
  const int nrows = ns + (with_min ? 1 : 0);
  if (warp < nrows) {
    const bool is_min = with_min && warp == ns;
    const double *src = red.v[warp];
    double acc = src[lane];
#pragma unroll
    for (int i = 1; i < kThreads / 32; ++i) {
      const double x = src[lane + 32 * i];
      acc = is_min ? fmin(acc, x) : acc + x;
    }
    acc = is_min ? warp_min(acc) : warp_sum(acc);
    if (lane == 0) red.out[warp] = acc;
  }
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < ns) r = red.out[threadIdx.x];
  else if (with_min && threadIdx.x == kMinSlot) r = red.out[ns];
  __syncthreads();
  return r;
}

// The finalize of an instance's item partials (stride kPart) with one warp
// per slot and no block barrier: lane l of warp k forms what threads l,
// l+32, ..., l+224 of the block form hold (each the identity plus its items
// t, t+256, ..., in that order), adds them in block_reduce's order and closes
// with the same shuffle tree -- block_reduce's operations in its order, so
// the sums are bitwise the block form's.  For instances of up to kThreads
// items (one item per thread at most).  Writes sums[0..kPart) (the slots the
// phase does not produce as 0.0); the caller syncs before reading them.
__device__ void warp_finalize(const double *pp, int nitems, int ns, bool wmin, double *sums) {
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int nrows = ns + (wmin ? 1 : 0);
  if (threadIdx.x < kPart && threadIdx.x >= ns && !(wmin && threadIdx.x == kMinSlot))
    sums[threadIdx.x] = 0.0;
  if (wp >= nrows) return;
  const bool is_min = wmin && wp == ns;
  const int k = is_min ? kMinSlot : wp;
  double a = 0.0;
#pragma unroll
  for (int i = 0; i < kThreads / 32; ++i) {
    const int t = lane + 32 * i;
    double th = is_min ? DBL_MAX : 0.0;
    if (t < nitems) {
      const double x = pp[(size_t)t * kPart + k];
      th = is_min ? fmin(th, x) : th + x;
    }
    a = (i == 0) ? th : (is_min ? fmin(a, th) : a + th);
  }
  a = is_min ? warp_min(a) : warp_sum(a);
  if (lane == 0) sums[k] = a;
}

// Bounded grid barrier in the style of cooperative groups' grid sync:
// arrival is an acq_rel atomic, the last CTA publishes the next generation
// with a release store, the others poll it with acquire loads (bounded by
// wait_ns and by the error flag), then bar.sync spreads the acquire to the CTA.
__device__ bool grid_barrier(Ctl *ctl, long long wait_ns, int &active_out) {
  __shared__ int s_ok, s_active;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile int *verr = &ctl->err;
    const unsigned int g = ld_acquire(&ctl->gen);
    const unsigned int arrived = atom_add_acq_rel(&ctl->count, 1u);
    int ok = 1;
    if (arrived == gridDim.x - 1) {
      ctl->snap[(g + 1) & 1] = *(volatile int *)&ctl->active;
      ctl->count = 0u;
      st_release(&ctl->gen, g + 1);
    } else {
      const long long t0 = gtimer();
      while (ld_acquire(&ctl->gen) == g) {
        if (*verr) { ok = 0; break; }
        if (gtimer() - t0 > wait_ns) {
          atomicCAS(&ctl->err, 0, -4);  // MPRGP_TIMEOUT
          ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    s_ok = ok && (*verr == 0);
    s_active = *(volatile int *)&ctl->snap[(g + 1) & 1];
  }
  __syncthreads();
  active_out = s_active;
  return s_ok;
}

__device__ __forceinline__ int find_instance(const int *prefix, int n, int item) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (ldro(prefix + mid) <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
// The instance of an item: one load from the run's item map, or a search of
// the item prefix when the run has no map.
__device__ __forceinline__ int instance_of(const int *item_inst, const int *prefix, int n,
                                           int item) {
  if (n == 1) return 0;  // a run of one instance needs no load
  return item_inst ? ldro(item_inst + item) : find_instance(prefix, n, item);
}

__global__ void __launch_bounds__(kThreads, MPRGP_ENGINE_MIN_BLOCKS) engine_kernel(EngineArgs args) {
  __shared__ InstDesc sD;
  __shared__ InstState sS;
  __shared__ RedBuf red;
  __shared__ double sums[kPart];
  __shared__ int s_last;
  Ctl *ctl = args.ctl;
  const long long t_start = gtimer();
  __shared__ int s_cache_inst, s_cache_ph;  // instance/phase of the sD, sS copies
  if (threadIdx.x == 0) {
    mbar_init(&g_stage_bar);
    g_staged = 0;
    s_cache_inst = -1;
    s_cache_ph = -1;
  }
  __syncthreads();
  unsigned int stage_parity = 0;
  for (int ph = 0; ph < args.max_phases; ++ph) {
    for (int item = blockIdx.x; item < args.total_items; item += gridDim.x) {
      const int inst = instance_of(args.item_inst, args.item_prefix, args.ninst, item);
      if (inst != s_cache_inst || ph != s_cache_ph) {
        const int *srcd = reinterpret_cast<const int *>(args.desc + inst);
        int *dstd = reinterpret_cast<int *>(&sD);
        for (int w = threadIdx.x; w < (int)(sizeof(InstDesc) / 4); w += kThreads)
          dstd[w] = ldro(srcd + w);
        const int *srcs = reinterpret_cast<const int *>(args.desc[inst].st);
        int *dsts = reinterpret_cast<int *>(&sS);
        for (int w = threadIdx.x; w < (int)(sizeof(InstState) / 4); w += kThreads)
          dsts[w] = srcs[w];
        __syncthreads();
        if (threadIdx.x == 0) {
          s_cache_inst = inst;
          s_cache_ph = ph;
        }
      }
      __syncthreads();
      if (sS.phase == PH_DONE) {
        __syncthreads();
        continue;
      }
      const int local = item - sD.item_begin;
      const int slot = local * kThreads + threadIdx.x;
      const int v = slot < sD.nv ? row_vertex(sD.A, slot) : slot;
      // Stage A for the FP32 matrix passes when the item's slice fits.
      const bool fp32_pass = sD.prec == PREC_MIXED &&
                             (sS.phase == PH_POW || sS.phase == PH_CG_SPMV ||
                              (sS.phase == PH_CG_ENTRY && sS.g_cons));
      if (fp32_pass && args.stage_bytes > 0) {
        if (threadIdx.x == 0) {
          const int s0 = local * (kThreads / kSlice);
          const int s1 = min(s0 + kThreads / kSlice, sD.A.nslices);
          const int f = ldro(sD.A.slice_off + s0), l = ldro(sD.A.slice_off + s1);
          const unsigned int cb = (unsigned int)(l - f) * kSlice * 4u;
          const unsigned int vb = (unsigned int)(l - f) * kSlice * 9u * 4u;
          if (cb + vb <= (unsigned int)args.stage_bytes && l > f) {
            g_staged = 1;
            g_stage_first = f;
            g_stage_voff = cb;
            asm volatile("fence.proxy.async.shared::cta;" : : : "memory");
            mbar_expect_tx(&g_stage_bar, cb + vb);
            bulk_g2s(g_stage, sD.A.cols + (size_t)f * kSlice, cb, &g_stage_bar);
            bulk_g2s(g_stage + cb, sD.A.v32 + (size_t)f * kSlice * 9, vb, &g_stage_bar);
          } else {
            g_staged = 0;
          }
        }
        __syncthreads();
        if (g_staged) {
          if (!mbar_wait_bounded(&g_stage_bar, stage_parity, args.wait_ns)) {
            // Record the failure, give the copy a second bounded wait so no
            // transfer lands after exit, then leave.
            if (threadIdx.x == 0) atomicCAS(&ctl->err, 0, -4);
            mbar_wait_bounded(&g_stage_bar, stage_parity, args.wait_ns);
            return;
          }
          stage_parity ^= 1u;
        }
      }
      double part[kPart];
#pragma unroll
      for (int k = 0; k < kPart; ++k) part[k] = (k == kMinSlot) ? DBL_MAX : 0.0;
      if (slot < sD.nv) row_op(sD, sS, v, slot, part);
      const int ns = nslots(sS.phase);
      const bool wmin = sS.phase == PH_PL_SPMV;
      const double r = block_reduce(part, red, ns, wmin);
      if (threadIdx.x < ns || (wmin && threadIdx.x == kMinSlot))
        sD.part[(size_t)local * kPart + threadIdx.x] = r;
      __syncthreads();
      if (threadIdx.x == 0) {
        const unsigned int old = atom_add_acq_rel(sD.cnt, 1u);
        s_last = (old == (unsigned int)sD.nitems - 1u);
      }
      __syncthreads();
      if (s_last) {
        if (sD.nitems <= kThreads) {
          warp_finalize(sD.part, sD.nitems, ns, wmin, sums);
        } else {
          double acc[kPart];
#pragma unroll
          for (int k = 0; k < kPart; ++k) acc[k] = (k == kMinSlot) ? DBL_MAX : 0.0;
          for (int it = threadIdx.x; it < sD.nitems; it += kThreads) {
#pragma unroll
            for (int k = 0; k < kPart; ++k) {
              if (k == kMinSlot ? !wmin : k >= ns) continue;
              const double x = sD.part[(size_t)it * kPart + k];
              acc[k] = (k == kMinSlot) ? fmin(acc[k], x) : acc[k] + x;
            }
          }
          const double t = block_reduce(acc, red, ns, wmin);
          if (threadIdx.x < kPart) sums[threadIdx.x] = t;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          InstState S = sS;
          advance(sD, S, sums);
          *sD.st = S;
          *sD.cnt = 0u;
          if (S.phase == PH_DONE) atomicSub(&ctl->active, 1);
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) g_staged = 0;
    }
    int active;
    if (!grid_barrier(ctl, args.wait_ns, active)) return;
    if (active == 0) return;
    if (gtimer() - t_start > args.total_ns) {
      if (threadIdx.x == 0) atomicCAS(&ctl->err, 0, -4);  // MPRGP_TIMEOUT
      return;
    }
  }
}

// ------------------------------------------------------- power kernel ----
// The power-method phases as ordinary launches of one kernel, the launch
// boundary as the phase barrier: the same per-row work, reductions and
// transitions as the persistent engine (hence the same results).  Its small
// register budget keeps every SM full of warps, which the latency-bound SpMV
// of these phases needs.  The launches are either the body of a CUDA-graph
// WHILE node (kPowerUnroll launches per body) or plain stream launches.  The
// finalize that completes the last power-phase instance of a launch decides
// whether another launch is needed: it sets a stop flag (the launches after
// it return at once) and, in the graph, the loop condition -- so the up to
// 1003 dependent phases run without a host launch each and stop as soon as
// every instance has left the power phases.
__device__ __forceinline__ bool power_phase(int ph) {
  return ph == PH_POW_RAND || ph == PH_POW || ph == PH_POW_LAST;
}

// One item of a phase launch.  kAll = false: power-method phases only (the
// other instances' items return at once); kAll = true: whatever phase each
// instance is in, with the same per-row work, reductions and transitions as
// the persistent engine -- so any phase can run as a launch of a graph loop.
template <bool kAll>
__device__ __forceinline__ void phase_item(const EngineArgs &args, int item, PowCtl *pc,
                                           cudaGraphConditionalHandle h, int signal,
                                           InstDesc &sD, InstState &sS, RedBuf &red,
                                           double (&sums)[kPart], int &s_last,
                                           unsigned int active) {
  const int inst = instance_of(args.item_inst, args.item_prefix, args.ninst, item);
  __syncthreads();  // the previous item's readers of sD/sS are done
  // desc and state in one round of loads when the run's states are an array
  // (desc order), else the state after the desc that points at it
  {
    const int *srcd = reinterpret_cast<const int *>(args.desc + inst);
    int *dstd = reinterpret_cast<int *>(&sD);
    for (int w = threadIdx.x; w < (int)(sizeof(InstDesc) / 4); w += kThreads) dstd[w] = ldro(srcd + w);
  }
  if (args.states) {
    const int *srcs = reinterpret_cast<const int *>(args.states + inst);
    int *dsts = reinterpret_cast<int *>(&sS);
    for (int w = threadIdx.x; w < (int)(sizeof(InstState) / 4); w += kThreads) dsts[w] = srcs[w];
    __syncthreads();
  } else {
    __syncthreads();
    const int *srcs = reinterpret_cast<const int *>(sD.st);
    int *dsts = reinterpret_cast<int *>(&sS);
    for (int w = threadIdx.x; w < (int)(sizeof(InstState) / 4); w += kThreads) dsts[w] = srcs[w];
    __syncthreads();
  }
  const int phase = sS.phase;
  if (kAll ? phase == PH_DONE : !power_phase(phase)) return;
  const int local = item - sD.item_begin;
  const int slot = local * kThreads + threadIdx.x;
  const bool wmin = kAll && phase == PH_PL_SPMV;
  double part[kPart];
#pragma unroll
  for (int k = 0; k < kPart; ++k) part[k] = (k == kMinSlot) ? DBL_MAX : 0.0;
  if (slot < sD.nv) {
    const int v = row_vertex(sD.A, slot);
    if (kAll) row_op(sD, sS, v, slot, part);
    else row_power(sD, sS, v, slot, part);
  }
  const int ns = nslots(phase);
  const double r = block_reduce(part, red, ns, wmin);
  if (threadIdx.x < ns || (wmin && threadIdx.x == kMinSlot))
    sD.part[(size_t)local * kPart + threadIdx.x] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int old = atom_add_acq_rel(sD.cnt, 1u);
    s_last = (old == (unsigned int)sD.nitems - 1u);
  }
  __syncthreads();
  if (!s_last) return;
  if (sD.nitems <= kThreads) {
    warp_finalize(sD.part, sD.nitems, ns, wmin, sums);
  } else {
    double acc[kPart];
#pragma unroll
    for (int k = 0; k < kPart; ++k) acc[k] = (k == kMinSlot) ? DBL_MAX : 0.0;
    for (int it = threadIdx.x; it < sD.nitems; it += kThreads) {
#pragma unroll
      for (int k = 0; k < kPart; ++k) {
        if (k == kMinSlot ? !wmin : k >= ns) continue;
        const double x = sD.part[(size_t)it * kPart + k];
        acc[k] = (k == kMinSlot) ? fmin(acc[k], x) : acc[k] + x;
      }
    }
    const double t = block_reduce(acc, red, ns, wmin);
    if (threadIdx.x < kPart) sums[threadIdx.x] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    InstState S = sS;
    if (kAll) {
      advance(sD, S, sums);
    } else {
      S.phases++;
      advance_power(sD, S, sums);
    }
    *sD.st = S;
    *sD.cnt = 0u;
    // One atomic counts this finalize (low word) and, if the instance goes
    // on, a busy instance (high word); `active` was read at the launch's
    // start (only the last finalize of a launch rewrites it).  The next
    // launch sees these writes at the kernel boundary.
    const bool still = kAll ? S.phase != PH_DONE : power_phase(S.phase);
    const unsigned long long old =
        atom_add_acq_rel(&pc->finbusy, 1ull + (still ? (1ull << 32) : 0ull));
    if ((unsigned int)old == active - 1u) {
      const unsigned int busy = (unsigned int)(old >> 32) + (still ? 1u : 0u);
      const unsigned int launches = pc->launches + 1u;
      const bool more = busy > 0u && launches < pc->limit;
      pc->launches = launches;
      pc->active = busy;
      pc->finbusy = 0ull;
      pc->stop = more ? 0u : 1u;
      if (signal) cudaGraphSetConditional(h, more ? 1u : 0u);
    }
  }
}

// The phase kernel: power-only with two register budgets -- 40 registers (6
// CTAs per SM, for grids that fill the SMs) or 64 (4 CTAs per SM, more loads
// in flight per thread) -- or every phase (kAll, 64 registers like the
// persistent engine).  The context's tuning picks one.
template <int kMinBlocks, bool kAll>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    phase_kernel(const EngineArgs *__restrict__ pargs, PowCtl *pc, cudaGraphConditionalHandle h,
                 int signal) {
  __shared__ InstDesc sD;
  __shared__ InstState sS;
  __shared__ RedBuf red;
  __shared__ double sums[kPart];
  __shared__ int s_last;
  // the loop control and the arguments in one round of loads (the stop test
  // would otherwise hold back the others)
  const unsigned int stop = *(volatile unsigned int *)&pc->stop;  // written by an earlier launch
  const unsigned int active = *(volatile unsigned int *)&pc->active;
  const EngineArgs args = *pargs;
  if (stop) return;
  if (threadIdx.x == 0) g_staged = 0;  // this kernel never stages A (no dynamic smem)
  for (int item = blockIdx.x; item < args.total_items; item += gridDim.x)
    phase_item<kAll>(args, item, pc, h, signal, sD, sS, red, sums, s_last, active);
}

// ------------------------------------------------- power-step loop -----
// The power method as a graph loop whose body is kPowerUnroll launches of
// power_step_kernel and one of power_settle_kernel.  No launch finalizes its
// own phase: launch j of a body reads the states launch j-1 left (launch 0:
// the run's state array) and, for an instance whose rows ran there, the item
// partials they wrote.  Every CTA reduces those partials in the launch
// form's finalize order with one extra warp and advances its own copy of the
// state from the sums, while its row warps already form their rows' products
// with the source vector the advanced state will name (the previous phase's
// output, which the state before the advance determines).  So a phase's
// serial reduction and FP64 update overlap the next phase's matrix pass and
// no launch waits on a last CTA.  The launches of even / odd position keep
// their states and (two per item) partials in separate copies.  The settle
// kernel applies the body's last partials, writes every state back to the
// run's array and sets the loop condition.  Each copy of a state advances
// from the same sums, summed in the same order, as the launch form's
// finalize, so results are bitwise those of the launch form.
constexpr int kStepThreads = kThreads + 32;  // the row warps + the reduction warp
constexpr int kNoSrc = -1000;                 // no power product for the rows

// Slots 0 and 1 of an instance's item partials (two per item) reduced by
// one warp in the finalize's order: thread t of phase_item's finalize sums
// items t, t + kThreads, ...; block_reduce's warp then adds the sums of
// threads l, l + 32, ..., l + 224 and closes with warp_sum.  Lane l keeps
// the sums of threads l + 32 i.  The partials come through shared memory,
// kSumStage items at a time, by asynchronous 16-byte copies that are all in
// flight together (plain loads would each wait for the previous add).
constexpr int kSumStage = 6 * kThreads;  // items per staged round (24 KB)
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void warp_item_sums(const double *pp, int nitems, int lane,
                                               double2 *stage, double s[2]) {
  double t0[kThreads / 32], t1[kThreads / 32];
#pragma unroll
  for (int i = 0; i < kThreads / 32; ++i) t0[i] = t1[i] = 0.0;
  for (int base = 0; base < nitems; base += kSumStage) {
    const int n = min(kSumStage, nitems - base);
    __syncwarp();  // the previous round's readers are done
    for (int j = lane; j < n; j += 32) cp_async16(stage + j, pp + 2 * (size_t)(base + j));
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncwarp();
    // round by round (base is a multiple of kThreads), so the sixteen sums of
    // a round are independent; each thread's items still add in item order
    for (int r = 0; r < n; r += kThreads) {
#pragma unroll
      for (int i = 0; i < kThreads / 32; ++i) {
        const int j = r + lane + 32 * i;
        if (j < n) {
          const double2 q = stage[j];
          t0[i] += q.x;
          t1[i] += q.y;
        }
      }
    }
  }
  double a0 = t0[0], a1 = t1[0];
#pragma unroll
  for (int i = 1; i < kThreads / 32; ++i) {
    a0 = a0 + t0[i];
    a1 = a1 + t1[i];
  }
  s[0] = warp_sum(a0);
  s[1] = warp_sum(a1);
}

// block_reduce of slots 0 and 1 over the row threads of a kStepThreads
// block (the same order); every thread takes part in the barriers.
__device__ double block_reduce_rows(const double part[2], RedBuf &red, int ns) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < kThreads) {
    red.v[0][threadIdx.x] = part[0];
    if (ns > 1) red.v[1][threadIdx.x] = part[1];
  }
  __syncthreads();
  if (warp < ns) {
    const double *src = red.v[warp];
    double acc = src[lane];
#pragma unroll
    for (int i = 1; i < kThreads / 32; ++i) acc = acc + src[lane + 32 * i];
    acc = warp_sum(acc);
    if (lane == 0) red.out[warp] = acc;
  }
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < ns) r = red.out[threadIdx.x];
  __syncthreads();
  return r;
}

// Advances a copy of a power-phase state by the phase's sums (the launch
// form's finalize).
__device__ __forceinline__ void advance_power_sums(const InstDesc &D, InstState &S,
                                                   const double s2[2]) {
  double sums[kPart];
#pragma unroll
  for (int k = 0; k < kPart; ++k) sums[k] = k < 2 ? s2[k] : 0.0;
  S.phases++;
  advance_power(D, S, sums);
}

// The reduction warp's work for one instance: `out` = `in` advanced by the
// partials pp (lane 0 writes it).  Not inlined, so that its FP64 state
// update does not take registers from the row warps' matrix pass.
__device__ __noinline__ void step_advance(const InstDesc &D, const InstState &in, InstState &out,
                                          const double *pp, int lane, double2 *stage) {
  {  // the whole warp copies, lane 0 then advances the copy in place
    const int *a = reinterpret_cast<const int *>(&in);
    int *b = reinterpret_cast<int *>(&out);
    for (int w = lane; w < (int)(sizeof(InstState) / 4); w += 32) b[w] = a[w];
  }
  double s2[2];
  warp_item_sums(pp, D.nitems, lane, stage, s2);
  __syncwarp();
  if (lane == 0) advance_power_sums(D, out, s2);
}

template <int kMinBlocks>
__global__ void __launch_bounds__(kStepThreads, kMinBlocks)
    power_step_kernel(const EngineArgs *__restrict__ pargs, PowCtl *pc, int node) {
  __shared__ InstDesc sD;
  __shared__ InstState sIn, sCur;
  __shared__ RedBuf red;
  __shared__ __align__(16) double2 sItems[kSumStage];
  __shared__ int s_inst;
  // the stop flag and the arguments in one round of loads
  const unsigned int stop = *(volatile unsigned int *)&pc->stop;  // the loop is over
  const EngineArgs args = *pargs;
  if (stop) return;
  if (threadIdx.x == 0) {
    g_staged = 0;
    s_inst = -1;
  }
  const int par = node & 1;
  const InstState *st_in = node == 0 ? args.states : args.pst[par ^ 1];
  InstState *st_out = args.pst[par];
  const int lane = threadIdx.x & 31;
  for (int item = blockIdx.x; item < args.total_items; item += gridDim.x) {
    const int inst = instance_of(args.item_inst, args.item_prefix, args.ninst, item);
    __syncthreads();  // the previous item is done with the shared copies
    // a CTA's consecutive items of one instance share its advanced state
    const bool fresh = inst != s_inst;
    if (fresh) {
      const int *srcd = reinterpret_cast<const int *>(args.desc + inst);
      int *dstd = reinterpret_cast<int *>(&sD);
      for (int w = threadIdx.x; w < (int)(sizeof(InstDesc) / 4); w += kStepThreads) dstd[w] = ldro(srcd + w);
      const int *srcs = reinterpret_cast<const int *>(st_in + inst);
      int *dsts = reinterpret_cast<int *>(&sIn);
      for (int w = threadIdx.x; w < (int)(sizeof(InstState) / 4); w += kStepThreads) dsts[w] = srcs[w];
      __syncthreads();
    }
    const int phase_in = fresh ? sIn.phase : sCur.phase;
    const bool pend = fresh && node > 0 && power_phase(phase_in);
    // the source vector of the product the rows will need
    int src = kNoSrc;
    if (pend) {
      if (phase_in == PH_POW_RAND) src = B_W1;
      else if (phase_in == PH_POW) src = (sIn.pow_k & 1) ? B_W1 : B_W;
    } else if (phase_in == PH_POW) {
      src = fresh ? sIn.pow_src : sCur.pow_src;
    }
    const int local = item - sD.item_begin;
    const int slot = local * kThreads + threadIdx.x;
    const bool row = threadIdx.x < kThreads && slot < sD.nv;
    const bool f32 = sD.prec == PREC_MIXED;
    float wf[3] = {0.f, 0.f, 0.f};
    double wd[3] = {0.0, 0.0, 0.0};
    if (row && src != kNoSrc) {
      if (f32) pow_raw32(sD, src, slot, wf);
      else pow_raw64(sD, src, slot, wd);
    }
    if (fresh && threadIdx.x >= kThreads) {  // the reduction warp
      if (pend) {
        step_advance(sD, sIn, sCur, sD.part + (size_t)(par ^ 1) * sD.nitems * 2, lane, sItems);
      } else {
        const int *a = reinterpret_cast<const int *>(&sIn);
        int *b = reinterpret_cast<int *>(&sCur);
        for (int w = lane; w < (int)(sizeof(InstState) / 4); w += 32) b[w] = a[w];
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) s_inst = inst;
    const int phase = sCur.phase;
    if (power_phase(phase)) {
      double part[2] = {0.0, 0.0};
      if (row) {
        const int v = row_vertex(sD.A, slot);
        if (phase == PH_POW_RAND) {
          row_power_rand(sD, v, part);
        } else {
          if (phase == PH_POW && sCur.pow_src != src) {  // not the predicted source
            if (f32) pow_raw32(sD, sCur.pow_src, slot, wf);
            else pow_raw64(sD, sCur.pow_src, slot, wd);
          }
          if (f32) row_power32_fin(sD, sCur, v, wf, part);
          else row_power64_fin(sD, sCur, v, wd, part);
        }
      }
      // the item this CTA takes next: its next item of this instance in this
      // launch, else its first item again in the next launch
      if (item + (int)gridDim.x < sD.item_begin + sD.nitems) prefetch_item_head(sD, local + (int)gridDim.x);
      else if (item + (int)gridDim.x >= args.total_items && (int)blockIdx.x >= sD.item_begin)
        prefetch_item_head(sD, (int)blockIdx.x - sD.item_begin);
      const double r = block_reduce_rows(part, red, nslots(phase));
      if (threadIdx.x < 2) sD.part[(size_t)par * sD.nitems * 2 + 2 * (size_t)local + threadIdx.x] = r;
    }
    if (threadIdx.x == 0 && item == sD.item_begin) st_out[inst] = sCur;
  }
}

// The end of a loop body: each instance's state from the body's last launch,
// advanced by that launch's partials when its rows ran, back to the run's
// state array; the last CTA to finish sets the loop condition (more bodies
// while an instance is in a power phase and fewer than PowCtl::limit launches
// have run).  One warp per CTA, instances grid-strided.
__global__ void __launch_bounds__(32)
    power_settle_kernel(const EngineArgs *__restrict__ pargs, PowCtl *pc,
                        cudaGraphConditionalHandle h, int signal) {
  __shared__ __align__(16) double2 sItems[kSumStage];
  const unsigned int stop = *(volatile unsigned int *)&pc->stop;
  const EngineArgs args = *pargs;
  if (stop) return;
  constexpr int last = (kPowerUnroll - 1) & 1;
  const InstState *st_in = args.pst[last];
  InstState *st_out = const_cast<InstState *>(args.states);
  const int lane = threadIdx.x;
  unsigned int busy = 0u;
  for (int inst = blockIdx.x; inst < args.ninst; inst += gridDim.x) {
    const InstDesc &D = args.desc[inst];
    InstState S = st_in[inst];
    if (power_phase(S.phase)) {
      double s2[2];
      warp_item_sums(D.part + (size_t)last * D.nitems * 2, D.nitems, lane, sItems, s2);
      advance_power_sums(D, S, s2);
    }
    if (lane == 0) {
      st_out[inst] = S;
      busy += power_phase(S.phase) ? 1u : 0u;
    }
  }
  if (lane == 0) {
    if (busy) atomicAdd(&pc->busy, busy);
    const unsigned int old = atom_add_acq_rel(&pc->fin, 1u);
    if (old == gridDim.x - 1u) {
      const unsigned int b = atomicAdd(&pc->busy, 0u);
      const unsigned int launches = pc->launches + (unsigned int)kPowerUnroll;
      const bool more = b > 0u && launches < pc->limit;
      pc->launches = launches;
      pc->busy = 0u;
      pc->fin = 0u;
      pc->stop = more ? 0u : 1u;
      __threadfence();
      if (signal) cudaGraphSetConditional(h, more ? 1u : 0u);
    }
  }
}

// ------------------------------------------------ persistent power loop -----
// Every power-method phase of a run's large instances in one cooperative
// launch, a bounded grid barrier as the phase boundary, with the power-step
// loop's overlap: a phase's reduction and state update run in one extra warp
// while the row warps already form the next phase's matrix products.
//
// Each CTA owns up to kPowOwn items (item b, b + grid, ...; the host sizes
// the grid so that the CTAs own equally many) and keeps their desc and state
// in shared memory for the whole loop.  Phase t: the reduction warp applies
// phase t-1's item partials to each owned item's copy of the state (the
// launch form's finalize order, warp_item_sums) while the row warps form the
// first owned item's raw product A src with the source the advanced state
// will name; then each owned item in a power phase finishes its rows with
// the advanced state (scale, store, partials of phase t, double-buffered by
// phase parity).  Every copy advances from the same sums in the same order as
// the launch form, so results are bitwise those of the launch form.  The loop
// ends after the first phase in which no instance had rows (each CTA with
// rows publishes the phase with atomicMax before the barrier), or after
// `limit` phases; then the CTA owning an instance's first item writes its
// state back.
// The reduction warp's work for one owned item: S advanced by the partials
// pp.  Not inlined, so that its sums do not take registers from the rows.
__device__ __noinline__ void persistent_apply(const InstDesc &D, InstState &S, const double *pp,
                                              int lane, double2 *stage) {
  double s2[2];
  warp_item_sums(pp, D.nitems, lane, stage, s2);
  __syncwarp();
  if (lane == 0) advance_power_sums(D, S, s2);
  __syncwarp();
}

template <int kMinBlocks>
__global__ void __launch_bounds__(kStepThreads, kMinBlocks)
    power_persistent_kernel(EngineArgs args, PowCtl *pc, int limit) {
  __shared__ InstDesc sD[kPowOwn];
  __shared__ InstState sS[kPowOwn];
  __shared__ RedBuf red;
  __shared__ __align__(16) double2 sItems[kSumStage];
  if (threadIdx.x == 0) g_staged = 0;
  const int lane = threadIdx.x & 31;
  const bool rw = threadIdx.x >= kThreads;  // the reduction warp
  // owned items: blockIdx.x + o * gridDim.x, o < nown
  const int nown = min(kPowOwn, (args.total_items - (int)blockIdx.x + (int)gridDim.x - 1) /
                                    (int)gridDim.x);
  for (int o = 0; o < nown; ++o) {
    const int inst = instance_of(args.item_inst, args.item_prefix, args.ninst, (int)(blockIdx.x + o * gridDim.x));
    const int *srcd = reinterpret_cast<const int *>(args.desc + inst);
    int *dstd = reinterpret_cast<int *>(&sD[o]);
    for (int w = threadIdx.x; w < (int)(sizeof(InstDesc) / 4); w += kStepThreads)
      dstd[w] = ldro(srcd + w);
    const int *srcs = reinterpret_cast<const int *>(args.states ? args.states + inst : nullptr);
    int *dsts = reinterpret_cast<int *>(&sS[o]);
    if (srcs)
      for (int w = threadIdx.x; w < (int)(sizeof(InstState) / 4); w += kStepThreads)
        dsts[w] = srcs[w];
  }
  __syncthreads();
  if (!args.states) {  // the states live at the descs' home
    for (int o = 0; o < nown; ++o) {
      const int *srcs = reinterpret_cast<const int *>(sD[o].st);
      int *dsts = reinterpret_cast<int *>(&sS[o]);
      for (int w = threadIdx.x; w < (int)(sizeof(InstState) / 4); w += kStepThreads)
        dsts[w] = srcs[w];
    }
    __syncthreads();
  }
  unsigned int pend = 0u;  // bit o: item o's rows ran in the previous phase
  int t = 0;
  for (;; ++t) {
    const int par = t & 1;
    // The first owned item's source vector, predicted from its state before
    // the advance (the previous phase's output when rows ran there).
    int src0 = kNoSrc;
    if (nown > 0) {
      const InstState &S0 = sS[0];
      if (pend & 1u) {
        if (S0.phase == PH_POW_RAND) src0 = B_W1;
        else if (S0.phase == PH_POW) src0 = (S0.pow_k & 1) ? B_W1 : B_W;
      } else if (S0.phase == PH_POW) {
        src0 = S0.pow_src;
      }
    }
    float wf[3] = {0.f, 0.f, 0.f};
    double wd[3] = {0.0, 0.0, 0.0};
    if (!rw && src0 != kNoSrc) {
      const int slot = ((int)blockIdx.x - sD[0].item_begin) * kThreads + threadIdx.x;
      if (slot < sD[0].nv) {
        if (sD[0].prec == PREC_MIXED) pow_raw32(sD[0], src0, slot, wf);
        else pow_raw64(sD[0], src0, slot, wd);
      }
    }
    if (rw) {  // apply the previous phase's partials to every owned state
      for (int o = 0; o < nown; ++o) {
        if (!((pend >> o) & 1u)) continue;
        persistent_apply(sD[o], sS[o], sD[o].part + (size_t)(par ^ 1) * sD[o].nitems * 2, lane,
                         sItems);
      }
    }
    __syncthreads();
    unsigned int ran = 0u;
    for (int o = 0; o < nown; ++o) {
      const int phase = sS[o].phase;
      if (!power_phase(phase)) continue;
      ran |= 1u << o;
      const InstDesc &D = sD[o];
      const int local = (int)(blockIdx.x + o * gridDim.x) - D.item_begin;
      const int slot = local * kThreads + threadIdx.x;
      const bool row = !rw && slot < D.nv;
      const bool f32 = D.prec == PREC_MIXED;
      double part[2] = {0.0, 0.0};
      if (row) {
        const int v = row_vertex(D.A, slot);
        if (phase == PH_POW_RAND) {
          row_power_rand(D, v, part);
        } else {
          const int src = sS[o].pow_src;
          if (phase == PH_POW && (o > 0 || src != src0)) {  // not formed above
            if (f32) pow_raw32(D, src, slot, wf);
            else pow_raw64(D, src, slot, wd);
          }
          if (f32) row_power32_fin(D, sS[o], v, wf, part);
          else row_power64_fin(D, sS[o], v, wd, part);
        }
      }
      // the item this CTA takes next: its next owned item, else its first
      // owned item in the next phase
      if (o + 1 < nown) prefetch_item_head(sD[o + 1], (int)(blockIdx.x + (o + 1) * gridDim.x) - sD[o + 1].item_begin);
      else prefetch_item_head(sD[0], (int)blockIdx.x - sD[0].item_begin);
      const double r = block_reduce_rows(part, red, nslots(phase));
      if (threadIdx.x < 2) D.part[(size_t)par * D.nitems * 2 + 2 * (size_t)local + threadIdx.x] = r;
    }
    pend = ran;
    if (ran && threadIdx.x == 0) atomicMax(&pc->busy, (unsigned int)(t + 1));
    int unused;
    if (!grid_barrier(args.ctl, args.wait_ns, unused)) return;
    if (*(volatile unsigned int *)&pc->busy < (unsigned int)(t + 1)) break;  // no rows anywhere
    if (t + 1 >= limit) {  // the last phase's partials, then stop
      if (rw) {
        for (int o = 0; o < nown; ++o) {
          if (!((pend >> o) & 1u)) continue;
          persistent_apply(sD[o], sS[o], sD[o].part + (size_t)par * sD[o].nitems * 2, lane,
                           sItems);
        }
      }
      __syncthreads();
      ++t;
      break;
    }
  }
  // the working phases run (the launch form's launch count)
  if (blockIdx.x == 0 && threadIdx.x == 0) pc->launches = (unsigned int)t;
  for (int o = 0; o < nown; ++o)
    if ((int)(blockIdx.x + o * gridDim.x) == sD[o].item_begin && threadIdx.x == 0) *sD[o].st = sS[o];
}

// ---------------------------------------------------- cluster solver -----
// One thread-block cluster per small instance.  Every CTA of the cluster
// holds the instance's desc and state in shared memory and advances its own
// copy of the state from the same sums, so the copies never diverge and no
// state travels through global memory between phases.  A phase: each CTA runs
// the per-row work of its items and reduces each item in the block (as the
// engine does); the item partials stay in shared memory; one cluster barrier
// (release/acquire, which also orders the phase's global vector writes); then
// every CTA reads all item partials through distributed shared memory in item
// order and reduces them exactly as the engine's finalize does -- so results
// are bitwise those of the persistent engine.  The partials are double
// buffered by phase parity, so one barrier per phase suffices.
__device__ __forceinline__ void cluster_sync_acq_rel() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;"
               ::: "memory");
}
__device__ __forceinline__ unsigned int cluster_rank() {
  unsigned int r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned int cluster_size() {
  unsigned int r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned int cluster_index() {
  unsigned int r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
// Address of `p` (this CTA's shared memory) in the shared memory of CTA `rank`.
__device__ __forceinline__ unsigned int dsmem_addr(const void *p, unsigned int rank) {
  const unsigned int a = (unsigned int)__cvta_generic_to_shared(p);
  unsigned int r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ double ld_dsmem(unsigned int addr) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}

__global__ void __launch_bounds__(kThreads, MPRGP_CLUSTER_MIN_BLOCKS) cluster_kernel(ClusterArgs args) {
  __shared__ InstDesc sD;
  __shared__ InstState sS;
  __shared__ RedBuf red;
  __shared__ double sums[kPart];
  __shared__ __align__(8) double cpart[2][kClusterItems][kPart];
  const unsigned int rank = cluster_rank(), csize = cluster_size();
  const int inst = (int)cluster_index();
  if (inst >= args.ninst) return;  // the whole cluster leaves together
  {
    const int *srcd = reinterpret_cast<const int *>(args.desc + inst);
    int *dstd = reinterpret_cast<int *>(&sD);
    for (int w = threadIdx.x; w < (int)(sizeof(InstDesc) / 4); w += kThreads) dstd[w] = ldro(srcd + w);
  }
  __syncthreads();
  {
    const int *srcs = reinterpret_cast<const int *>(sD.st);
    int *dsts = reinterpret_cast<int *>(&sS);
    for (int w = threadIdx.x; w < (int)(sizeof(InstState) / 4); w += kThreads) dsts[w] = srcs[w];
  }
  if (threadIdx.x == 0) {
    g_staged = 0;
    if (rank != 0) sD.trace = nullptr;  // CTA 0 alone records the trace
  }
  __syncthreads();
  const int nitems = sD.nitems;
  int par = 0;
  for (int ph = 0; ph < args.max_phases && sS.phase != PH_DONE; ++ph) {
    const int phase = sS.phase;
    const int ns = nslots(phase);
    const bool wmin = phase == PH_PL_SPMV;
    int li = 0;
    for (int item = (int)rank; item < nitems && li < kClusterItems; item += (int)csize, ++li) {
      double part[kPart];
#pragma unroll
      for (int k = 0; k < kPart; ++k) part[k] = (k == kMinSlot) ? DBL_MAX : 0.0;
      const int slot = item * kThreads + threadIdx.x;
      if (slot < sD.nv) {
        const int v = row_vertex(sD.A, slot);
        row_op(sD, sS, v, slot, part);
      }
      const double r = block_reduce(part, red, ns, wmin);
      if (threadIdx.x < ns || (wmin && threadIdx.x == kMinSlot)) cpart[par][li][threadIdx.x] = r;
    }
    cluster_sync_acq_rel();
    if (nitems <= 32) {
      // One warp per slot does what the block reduction below does when each
      // thread holds at most one item: lane l takes item l (thread l's sum),
      // then seven more terms from threads that hold none (the identity:
      // +0.0, or DBL_MAX for the min slot), then the shuffle tree -- the same
      // operations in the same order, without the block's barriers.
      const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
      const int nrows = ns + (wmin ? 1 : 0);
      // the slots this phase does not produce read as 0.0
      if (threadIdx.x < kPart && threadIdx.x >= ns && !(wmin && threadIdx.x == kMinSlot))
        sums[threadIdx.x] = 0.0;
      if (wp < nrows) {
        const bool is_min = wmin && wp == ns;
        const int k = is_min ? kMinSlot : wp;
        double a = is_min ? DBL_MAX : 0.0;
        if (lane < nitems) {
          const unsigned int base =
              dsmem_addr(&cpart[par][lane / (int)csize][0], (unsigned int)lane % csize);
          const double x = ld_dsmem(base + 8u * (unsigned int)k);
          a = is_min ? fmin(a, x) : a + x;
        }
#pragma unroll
        for (int i = 1; i < kThreads / 32; ++i) a = is_min ? fmin(a, DBL_MAX) : a + 0.0;
        a = is_min ? warp_min(a) : warp_sum(a);
        if (lane == 0) sums[k] = a;
      }
    } else {
      double acc[kPart];
#pragma unroll
      for (int k = 0; k < kPart; ++k) acc[k] = (k == kMinSlot) ? DBL_MAX : 0.0;
      for (int it = threadIdx.x; it < nitems; it += kThreads) {
        const unsigned int base = dsmem_addr(&cpart[par][it / (int)csize][0], (unsigned int)it % csize);
#pragma unroll
        for (int k = 0; k < kPart; ++k) {
          if (k == kMinSlot ? !wmin : k >= ns) continue;
          const double x = ld_dsmem(base + 8u * (unsigned int)k);
          acc[k] = (k == kMinSlot) ? fmin(acc[k], x) : acc[k] + x;
        }
      }
      const double t = block_reduce(acc, red, ns, wmin);
      if (threadIdx.x < kPart) sums[threadIdx.x] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) advance(sD, sS, sums);  // in place: no copy of the state
    __syncthreads();
    par ^= 1;
  }
  if (rank == 0 && threadIdx.x == 0) *sD.st = sS;
  cluster_sync_acq_rel();  // no CTA leaves while another may read its partials
}

// ------------------------------------------------------ setup kernels -----
// BSR (row_ptr, cols, 9 values per block, row-major) -> SELL-32, plus
// D^-1 = 1/diag(A) (getDiagonal, MPRGPUtility.h:503-515).
__global__ void bsr_to_sell_kernel(int nv, const int *__restrict__ row_ptr,
                                   const int *__restrict__ cols, const double *__restrict__ vals,
                                   const int *__restrict__ slice_off,
                                   const int *__restrict__ rowmap, int *out_cols,
                                   short *out_cols16, int *c16ok, double *out64, float *out32,
                                   double *dinv, int *bad) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;  // SELL row (slot)
  const int s = q >> 5, lane = q & 31;
  const int nslices = (nv + kSlice - 1) / kSlice;
  if (s >= nslices) return;
  const int r = (q < nv && rowmap) ? rowmap[q] : q;      // its vertex
  const int j0 = slice_off[s], w = slice_off[s + 1] - j0;
  const int b = (q < nv) ? row_ptr[r] : 0;
  const int len = (q < nv) ? row_ptr[r + 1] - b : 0;
  double dg[3] = {0.0, 0.0, 0.0};
  for (int j = 0; j < w; ++j) {
    const size_t slot = (size_t)(j0 + j);
    int c;
    double m[9];
    if (j < len) {
      c = cols[b + j];
      for (int e = 0; e < 9; ++e) m[e] = vals[9 * (size_t)(b + j) + e];
      if (c < 0 || c >= nv) {  // invalid input: flag it, keep every index in range
        if (bad) atomicOr(bad, 1);
        c = r;
        for (int e = 0; e < 9; ++e) m[e] = 0.0;
      } else if (c == r) {
        dg[0] = m[0];
        dg[1] = m[4];
        dg[2] = m[8];
      }
    } else {
      c = (q < nv) ? r : 0;
      for (int e = 0; e < 9; ++e) m[e] = 0.0;
    }
    out_cols[slot * kSlice + lane] = c;
    if (out_cols16) {  // the offset from the row's vertex; one that does not fit
      const int d = c - ((q < nv) ? r : 0);  // sends every pass to the 32-bit columns
      const bool fits = d >= -32768 && d <= 32767;
      out_cols16[slot * kSlice + lane] = fits ? (short)d : (short)0;
      if (!fits) *c16ok = 0;
    }
    for (int e = 0; e < 9; ++e) {
      if (out64) out64[sell_index(slot, e, lane, double())] = m[e];
      if (out32) out32[sell_index(slot, e, lane, float())] = (float)m[e];
    }
  }
  if (q < nv)
    for (int d = 0; d < 3; ++d) dinv[3 * (size_t)r + d] = 1.0 / dg[d];
}

// Planes (n, p) with n.x + p >= 0 -> rows (n, c = -p) of J x >= c, with
// 1/diag(J J^T) and 1/diag(J D^-1 J^T) (MPRGPPrecondition.h:81-89).
__global__ void planes_setup_kernel(int nv, const int *__restrict__ plane_ptr,
                                    const double *__restrict__ in, double *out, double *nn,
                                    double *indn, const double *__restrict__ dinv,
                                    unsigned char *unit) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  if (unit) {  // 2-3 planes with an identity Gram matrix (same products as gram())
    const int b = plane_ptr[v], k = plane_ptr[v + 1] - b;
    bool id = k >= 2 && k <= kMaxPlanes;
    for (int i = 0; id && i < k; ++i)
      for (int j = 0; j < k; ++j) {
        const double *ni = in + 4 * (size_t)(b + i), *nj = in + 4 * (size_t)(b + j);
        const double gij = dot3(ni, nj);
        id &= (i == j) ? gij == 1.0 : gij == 0.0;
      }
    unit[v] = id ? 1 : 0;
  }
  for (int q = plane_ptr[v]; q < plane_ptr[v + 1]; ++q) {
    const double n0 = in[4 * (size_t)q], n1 = in[4 * (size_t)q + 1], n2 = in[4 * (size_t)q + 2];
    out[4 * (size_t)q] = n0;
    out[4 * (size_t)q + 1] = n1;
    out[4 * (size_t)q + 2] = n2;
    out[4 * (size_t)q + 3] = -in[4 * (size_t)q + 3];
    nn[q] = 1.0 / (n0 * n0 + n1 * n1 + n2 * n2);
    if (dinv) {
      const double t = n0 * n0 * dinv[3 * (size_t)v] + n1 * n1 * dinv[3 * (size_t)v + 1] +
                       n2 * n2 * dinv[3 * (size_t)v + 2];
      indn[q] = 1.0 / t;
    }
  }
}

// Axis code of every plane row: d when its normal (raw, before the sign
// change of the offset) is exactly the unit vector e_d, else 3.
__global__ void planes_axis_kernel(int m, const double *__restrict__ in, unsigned char *axis) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  const double n0 = in[4 * (size_t)q], n1 = in[4 * (size_t)q + 1], n2 = in[4 * (size_t)q + 2];
  unsigned char a = 3;
  if (n0 == 1.0 && n1 == 0.0 && n2 == 0.0) a = 0;
  else if (n0 == 0.0 && n1 == 1.0 && n2 == 0.0) a = 1;
  else if (n0 == 0.0 && n1 == 0.0 && n2 == 1.0) a = 2;
  axis[q] = a;
}

// Standalone y = A x (FixedSparseMatrix::multiply, MPRGPSolver.h:469-473).
template <typename VT>
__global__ void __launch_bounds__(256, MPRGP_SPMV_MIN_BLOCKS) spmv_kernel(SellMatrix A, const VT *__restrict__ vals,
                                                   int nv, const double *__restrict__ x,
                                                   double *__restrict__ y) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nv) return;
  const int v = row_vertex(A, slot);
  double o[3];
  if constexpr (sizeof(VT) == 4) spmv_row<VT>(A, vals, slot, SrcVtoF{x}, o);
  else spmv_row<VT>(A, vals, slot, SrcV{x}, o);
  st3(y, v, o);
}

// During an engine run the instance states live in one array in desc order
// (the run's desc entries point into it), so a launch can fetch an item's
// desc and state in one round of loads.  Between runs each state lives with
// its problem (`home`).  Before a run the fresh instances' initial states are
// already in the array (uploaded from the host) and their phase-item counters
// are cleared, the others' states are copied in from home; after it every
// state is copied back home (the array then also goes to the host).  One CTA
// per instance.
static_assert(sizeof(InstState) % 8 == 0, "InstState is copied as 8-byte words");
constexpr int kStateWords = (int)(sizeof(InstState) / 8);

__global__ void state_scatter_kernel(const InstDesc *__restrict__ desc, int n, InstState *states,
                                     InstState *const *__restrict__ home,
                                     const int *__restrict__ fresh) {
  const int j = blockIdx.x;
  if (j >= n) return;
  if (fresh[j]) {
    if (threadIdx.x == 0) *desc[j].cnt = 0u;
    return;
  }
  const unsigned long long *src = reinterpret_cast<const unsigned long long *>(home[j]);
  unsigned long long *dst = reinterpret_cast<unsigned long long *>(states + j);
  for (int w = threadIdx.x; w < kStateWords; w += blockDim.x) dst[w] = src[w];
}

__global__ void state_gather_kernel(const InstDesc *__restrict__ desc, int n, InstState *states,
                                    InstState *const *__restrict__ home) {
  const int j = blockIdx.x;
  if (j >= n) return;
  // An instance whose A had a block column outside 0..nv-1 (the conversion
  // kept its indices in range) reports MPRGP_INVALID whatever it computed.
  if (threadIdx.x == 0 && desc[j].bad && *desc[j].bad) states[j].code = kCodeInvalid;
  __syncthreads();
  const unsigned long long *src = reinterpret_cast<const unsigned long long *>(states + j);
  unsigned long long *dst = reinterpret_cast<unsigned long long *>(home[j]);
  for (int w = threadIdx.x; w < kStateWords; w += blockDim.x) dst[w] = src[w];
}

// Host-side launch helpers (declared in capi.cu).
void launch_state_scatter(const InstDesc *desc, int n, InstState *states, InstState *const *home,
                          const int *fresh, cudaStream_t st) {
  if (n > 0) state_scatter_kernel<<<n, 64, 0, st>>>(desc, n, states, home, fresh);
}
void launch_state_gather(const InstDesc *desc, int n, InstState *states, InstState *const *home,
                         cudaStream_t st) {
  if (n > 0) state_gather_kernel<<<n, 64, 0, st>>>(desc, n, states, home);
}
cudaError_t launch_engine(const EngineArgs &args, int grid, cudaStream_t stream) {
  void *params[] = {(void *)&args};
  return cudaLaunchCooperativeKernel((const void *)engine_kernel, dim3(grid), dim3(kThreads),
                                     params, (size_t)args.stage_bytes, stream);
}
// Resident engine CTAs per SM with `stage_bytes` of dynamic shared memory.
cudaError_t engine_max_blocks_per_sm(int *n, int stage_bytes) {
  cudaError_t e = cudaFuncSetAttribute(engine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kStageBytes);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, engine_kernel, kThreads, stage_bytes);
}
// A graph whose WHILE node runs phase_kernel over `grid` CTAs until no
// instance is left in a power phase or PowCtl::limit launches have run.  The
// kernel reads its EngineArgs and PowCtl from device memory, so one
// instantiation serves every later run with the same grid.
// variant 0: power phases, 40 registers; 1: power phases, 64 registers;
// 2: every phase (the graph form of the engine).
// 3: the power-step loop (power_step_kernel, kStepThreads threads).
const void *power_kernel_fn(int variant) {
  return variant == 3 ? (const void *)power_step_kernel<MPRGP_STEP_MIN_BLOCKS>
         : variant == 2 ? (const void *)phase_kernel<MPRGP_ALLPHASE_MIN_BLOCKS, true>
         : variant   ? (const void *)phase_kernel<4, false>
                     : (const void *)phase_kernel<MPRGP_POWER_MIN_BLOCKS, false>;
}
int power_block_threads(int variant) { return variant == 3 ? kStepThreads : kThreads; }
constexpr int kSettleGrid = 32;  // CTAs of power_settle_kernel (instances grid-strided)
cudaError_t build_power_graph(int grid, int variant, const EngineArgs *d_args, PowCtl *d_pc,
                              cudaGraph_t *graph, cudaGraphExec_t *exec) {
  *graph = nullptr;
  *exec = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle h;
  e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cond;
  if (e == cudaSuccess) e = cudaGraphAddNode(&cond, g, nullptr, nullptr, 0, &cp);
  if (e == cudaSuccess && variant == 3) {
    // kPowerUnroll step launches (their position in the body as argument),
    // then the settle kernel, which sets the condition
    cudaGraphNode_t prev = nullptr;
    for (int u = 0; u < kPowerUnroll && e == cudaSuccess; ++u) {
      int node = u;
      void *kargs[] = {(void *)&d_args, (void *)&d_pc, (void *)&node};
      cudaKernelNodeParams kp;
      memset(&kp, 0, sizeof(kp));
      kp.func = (void *)power_kernel_fn(3);
      kp.gridDim = dim3(grid);
      kp.blockDim = dim3(kStepThreads);
      kp.kernelParams = kargs;
      cudaGraphNode_t kn;
      e = cudaGraphAddKernelNode(&kn, cp.conditional.phGraph_out[0], prev ? &prev : nullptr,
                                 prev ? 1 : 0, &kp);
      prev = kn;
    }
    if (e == cudaSuccess) {
      int signal = 1;
      void *kargs[] = {(void *)&d_args, (void *)&d_pc, (void *)&h, (void *)&signal};
      cudaKernelNodeParams kp;
      memset(&kp, 0, sizeof(kp));
      kp.func = (void *)power_settle_kernel;
      kp.gridDim = dim3(kSettleGrid);
      kp.blockDim = dim3(32);
      kp.kernelParams = kargs;
      cudaGraphNode_t kn;
      e = cudaGraphAddKernelNode(&kn, cp.conditional.phGraph_out[0], &prev, 1, &kp);
    }
  } else if (e == cudaSuccess) {
    int signal = 1;
    void *kargs[] = {(void *)&d_args, (void *)&d_pc, (void *)&h, (void *)&signal};
    cudaKernelNodeParams kp;
    memset(&kp, 0, sizeof(kp));
    kp.func = (void *)power_kernel_fn(variant);
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(kThreads);
    kp.kernelParams = kargs;
    cudaGraphNode_t prev = nullptr;
    for (int u = 0; u < kPowerUnroll && e == cudaSuccess; ++u) {
      cudaGraphNode_t kn;
      e = cudaGraphAddKernelNode(&kn, cp.conditional.phGraph_out[0], prev ? &prev : nullptr,
                                 prev ? 1 : 0, &kp);
      prev = kn;
    }
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    *exec = nullptr;
    return e;
  }
  *graph = g;
  return cudaSuccess;
}
// The same loop as plain stream launches (`launches` of them; those after the
// last working one return at once).
cudaError_t launch_power_direct(int grid, int variant, int launches, const EngineArgs *d_args,
                                PowCtl *d_pc, cudaStream_t stream) {
  if (variant == 3) {  // whole bodies: kPowerUnroll steps and the settle kernel
    const cudaGraphConditionalHandle h0 = 0;
    for (int k = 0; k < launches; k += kPowerUnroll) {
      for (int u = 0; u < kPowerUnroll; ++u)
        power_step_kernel<MPRGP_STEP_MIN_BLOCKS><<<grid, kStepThreads, 0, stream>>>(d_args, d_pc, u);
      power_settle_kernel<<<kSettleGrid, 32, 0, stream>>>(d_args, d_pc, h0, 0);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  for (int k = 0; k < launches; ++k) {
    const cudaGraphConditionalHandle h0 = 0;
    if (variant == 2) phase_kernel<MPRGP_ALLPHASE_MIN_BLOCKS, true><<<grid, kThreads, 0, stream>>>(d_args, d_pc, h0, 0);
    else if (variant) phase_kernel<4, false><<<grid, kThreads, 0, stream>>>(d_args, d_pc, h0, 0);
    else phase_kernel<MPRGP_POWER_MIN_BLOCKS, false><<<grid, kThreads, 0, stream>>>(d_args, d_pc, h0, 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}
cudaError_t launch_cluster(const ClusterArgs &args, int csize, cudaStream_t stream) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned int)(args.ninst * csize));
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned int)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, cluster_kernel, args);
}
// Clusters of `csize` CTAs that can be resident at once (0 if none).
cudaError_t cluster_max_active(int csize, int *n) {
  *n = 0;
  if (csize > 8) {
    cudaError_t e = cudaFuncSetAttribute(cluster_kernel,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned int)csize);
  cfg.blockDim = dim3(kThreads);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned int)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaOccupancyMaxActiveClusters(n, cluster_kernel, &cfg);
}
cudaError_t launch_power_persistent(const EngineArgs &args, PowCtl *d_pc, int limit, int grid,
                                    cudaStream_t stream) {
  void *params[] = {(void *)&args, (void *)&d_pc, (void *)&limit};
  return cudaLaunchCooperativeKernel((const void *)power_persistent_kernel<4>, dim3(grid),
                                     dim3(kStepThreads), params, 0, stream);
}
cudaError_t power_persistent_max_blocks_per_sm(int *n) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, power_persistent_kernel<4>, kStepThreads,
                                                       0);
}
cudaError_t power_max_blocks_per_sm(int variant, int *n) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, power_kernel_fn(variant),
                                                       power_block_threads(variant), 0);
}
void launch_bsr_to_sell(int nv, const int *row_ptr, const int *cols, const double *vals,
                        const int *slice_off, const int *rowmap, int *out_cols, short *out_cols16,
                        int *c16ok, double *out64, float *out32, double *dinv, int *bad,
                        cudaStream_t st) {
  const int nslices = (nv + kSlice - 1) / kSlice;
  const int threads = nslices * kSlice;
  // (the caller sets *c16ok = 1 before the conversion)
  bsr_to_sell_kernel<<<(threads + 255) / 256, 256, 0, st>>>(nv, row_ptr, cols, vals, slice_off,
                                                            rowmap, out_cols, out_cols16, c16ok,
                                                            out64, out32, dinv, bad);
}
void launch_planes_setup(int nv, const int *plane_ptr, const double *in, double *out, double *nn,
                         double *indn, const double *dinv, unsigned char *unit, cudaStream_t st) {
  planes_setup_kernel<<<(nv + 255) / 256, 256, 0, st>>>(nv, plane_ptr, in, out, nn, indn, dinv,
                                                        unit);
}
void launch_planes_axis(int m, const double *in, unsigned char *axis, cudaStream_t st) {
  if (m > 0) planes_axis_kernel<<<(m + 255) / 256, 256, 0, st>>>(m, in, axis);
}
void launch_spmv(const SellMatrix &A, int nv, bool fp32, const double *x, double *y,
                 cudaStream_t st) {
  if (fp32) spmv_kernel<float><<<(nv + 255) / 256, 256, 0, st>>>(A, A.v32, nv, x, y);
  else spmv_kernel<double><<<(nv + 255) / 256, 256, 0, st>>>(A, A.v64, nv, x, y);
}

}  // namespace mprgp
