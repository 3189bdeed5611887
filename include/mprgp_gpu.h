/* include/mprgp_gpu.h -- C ABI of the GB300 MPRGP solver (libmprgp_gb300.so).
 *
 * The reference (simba518/MPRGP) is a header-only C++ template library with
 * no FFI: callers instantiate MATH::MPRGPDecoupledCon<double>::solve and its
 * siblings directly (src/MPRGPSolver/MPRGPSolver.h:503-626).  This header is
 * the thin boundary that replaces those instantiations; the C++ template
 * façade in include/mprgp/MPRGPSolver.h keeps the reference's class names and
 * signatures and forwards to the functions below.  Every function is plain
 * C: pointers, sizes and status codes, no C++ or torch types.
 *
 * Conventions
 *   - A QP instance has nv vertices and n = 3*nv unknowns (x, y, z per vertex).
 *   - A is given as 3x3-block CSR ("BSR"): row_ptr[nv+1], cols[nnzb] (vertex
 *     indices), vals[9*nnzb], each block row-major.  It must be symmetric
 *     positive definite, as the reference requires.
 *   - Plane constraints are per vertex, in the reference's VVVec4d form
 *     (MprgpFemSolver.h:107, MPRGPUtility.h:120-154): plane (nx, ny, nz, p)
 *     on vertex v means nx*x_v + ny*y_v + nz*z_v + p >= 0, i.e. the row of J
 *     is n at the vertex's three columns and c = -p.  plane_ptr[nv+1] lists
 *     the planes of each vertex (CSR by vertex); at most 3 per vertex.
 *   - Bound constraints are per unknown: L[n] (and U[n] for a box).
 *   - Returned codes follow the reference: 0 converged, -1 not converged
 *     (MPRGPSolver.h:390, :445); negative values below -1 are errors.
 */
#ifndef MPRGP_GPU_H
#define MPRGP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MPRGP_OK 0
#define MPRGP_NOT_CONVERGED (-1) /* reference result_code -1 */
#define MPRGP_BREAKDOWN (-2)     /* NaN in a step length */
#define MPRGP_OOM (-3)           /* device allocation failed / admission cap */
#define MPRGP_TIMEOUT (-4)       /* a bounded device wait ran out */
#define MPRGP_INVALID (-5)       /* bad argument or unsupported shape */
#define MPRGP_CUDA_ERROR (-6)    /* CUDA runtime error */
#define MPRGP_NO_DEVICE (-7)     /* no CUDA device / extension unusable */
#define MPRGP_BUSY (-8)          /* resource in use (server slot table full) */

/* ---- projector kinds (which reference façade the solve mirrors) -------- */
#define MPRGP_KIND_LOWER 0     /* MPRGPLowerBound   (MPRGPSolver.h:503-517) */
#define MPRGP_KIND_BOX 1       /* MPRGPBoxBound     (MPRGPSolver.h:520-535) */
#define MPRGP_KIND_DECOUPLED 2 /* MPRGPDecoupledCon (MPRGPSolver.h:538-590) */
#define MPRGP_KIND_PLANES 3    /* MPRGPGeneralCon   (MPRGPSolver.h:593-626),
                                  per-vertex plane blocks solved exactly */

/* ---- algorithm --------------------------------------------------------- */
#define MPRGP_ALG_DEFAULT 0  /* what the façade of `kind` uses */
#define MPRGP_ALG_MONOTONE 1 /* MPRGPMonotonic::solve (MPRGPSolver.h:412-454) */
#define MPRGP_ALG_PLAIN 2    /* MPRGP::solve         (MPRGPSolver.h:356-396) */

/* ---- preconditioner ---------------------------------------------------- */
#define MPRGP_PRECOND_DEFAULT 0  /* what the façade of `kind` uses */
#define MPRGP_PRECOND_NONE 1     /* the façade's preconditioned=false: z = phi */
#define MPRGP_PRECOND_INFACE 2   /* DiagonalInFacePreconSolver (Precondition.h:36-69) */
#define MPRGP_PRECOND_DECOUPLE 3 /* DiagonalDecouplePreconSolver (Precondition.h:72-110) */

/* ---- precision form ---------------------------------------------------- */
#define MPRGP_PREC_FP64 0  /* plain FP64 everywhere */
#define MPRGP_PREC_MIXED 1 /* A stored/multiplied in FP32 (FP32 accumulate) for
                              CG and power-method products; FP64 for dots,
                              steps, projection, residual refinement and the
                              stopping test */

typedef struct mprgp_options {
  double tol;          /* absolute tolerance on ||phi+beta|| (tolerance_factor) */
  int max_it;          /* max_iterations */
  int kind;            /* MPRGP_KIND_* */
  int algorithm;       /* MPRGP_ALG_* */
  int precond;         /* MPRGP_PRECOND_* */
  int precision;       /* MPRGP_PREC_* */
  int project_x0;      /* 1: x <- P(x) first (the solve(A,B,J,c,x) overloads) */
  int use_ev;          /* 1: start the power method from the stored vector */
  uint64_t seed;       /* seed of the power method's start vector */
  double wait_limit_s; /* bound on any device-side wait (0 = 5 s) */
} mprgp_options;

typedef struct mprgp_stats {
  int code;        /* 0 converged, -1 not converged, < -1 error */
  int iterations;  /* iterations_out */
  int num_cg, num_exp, num_prop;
  int power_iters; /* specRad's iteration count */
  int active;      /* COUNT_CONSTRAINTS(face) (MPRGPUtility.h:98-106) */
  int ev_updated;  /* 1 if the power method converged and stored its vector */
  double residual; /* residual_out */
  double alpha_bar, spec_rad;
  long long spmv_fp64, spmv_fp32; /* matrix passes by precision */
  long long phases;               /* device phases executed */
  double device_ms;               /* kernel time of the solve */
  long long power_passes;         /* matrix passes of the power method (in spmv_*) */
} mprgp_stats;

/* ---- library ------------------------------------------------------------ */
int mprgp_version(void);
const char *mprgp_status_string(int status);
/* Text of the last failure on the calling thread (for diagnostics). */
const char *mprgp_last_error(void);
void mprgp_default_options(mprgp_options *opt);
int mprgp_device_count(int *count);

/* ---- context: one device, one stream ------------------------------------ */
typedef struct mprgp_context mprgp_context;
int mprgp_context_create(int device, mprgp_context **out);
int mprgp_context_destroy(mprgp_context *ctx);
void *mprgp_context_stream(mprgp_context *ctx); /* the cudaStream_t it launches on */
int mprgp_context_sync(mprgp_context *ctx);
/* SM count and resident engine CTAs per SM (the persistent grid's shape). */
int mprgp_context_info(mprgp_context *ctx, int *nsm, int *blocks_per_sm);
/* No counterpart in the reference.  Device bytes that new problems of the
 * context can take now: the device's free memory (cudaMemGetInfo, so other
 * users of the GPU count) plus the blocks the context's memory pool holds
 * but no problem uses.  The server's admission reads the same figure. */
int mprgp_context_room(mprgp_context *ctx, size_t *bytes);
/* Counters since the context was created: kernels launched (engine runs,
 * cluster-solver launches, setup kernels and every iteration of the
 * power-method graph loop), the device time of the solver runs (power loop,
 * cluster solver and engine) and of the power loop alone, in milliseconds. */
int mprgp_context_counters(mprgp_context *ctx, long long *launches, double *solver_ms,
                           double *power_ms);
/* Launch shape of later solves on this context (chosen by the autotuner,
 * mprgp_gb300/autotune.py): bit 0 of stage = 1 brings each item's FP32
 * matrix slice into shared memory with bulk async copies (one CTA per SM),
 * 0 reads it from global memory; bit 1 of stage = 1 runs the power method in
 * the persistent engine instead of the dedicated power kernel; bit 2 = 1
 * issues the power kernel's launches from the host stream instead of a
 * CUDA-graph WHILE loop (and likewise the graph loop of bit 4 when a run has
 * a phase quantum: one launch per phase of it); bit 3 = 1 builds the phase
 * kernel of bit 6 for 64 registers per thread (4 CTAs per SM) instead of 40
 * (6 CTAs per SM);
 * bit 4 = 1 runs the large instances' phases as a CUDA-graph loop of
 * ordinary launches (one phase per launch) instead of the persistent
 * cooperative engine; bit 5 = 1 runs the power method as one persistent
 * cooperative launch (a grid barrier per phase, state kept on chip) in
 * synchronous runs whose items fit four per resident CTA, the graph loop
 * otherwise.  By default the power kernel runs as the power-step loop: no
 * launch finalizes its own phase -- every CTA of the next launch reduces the
 * item partials and advances its copy of the state with one extra warp while
 * its rows already form their products, and a settle kernel ends each graph
 * body; bit 6 = 1 runs the phase kernel instead, whose last CTA finalizes
 * each launch (bit 2 applies to both loops).  ctas_per_sm
 * caps the persistent grid (0 = every resident CTA).  Every setting gives
 * bitwise the same results. */
int mprgp_context_set_tuning(mprgp_context *ctx, int stage, int ctas_per_sm);
/* Small instances -- up to `cluster` items of 256 vertices -- are solved by
 * one thread-block cluster each, one CTA per item (state in shared memory,
 * reductions through distributed shared memory, cluster barriers between
 * phases), grouped by cluster size (1, 2, 4, 8, 16) and run concurrently; the
 * others by the persistent engine.  `cluster` is the largest cluster size (a
 * power of two, 16 by default where the device allows it); 0 sends every
 * instance to the engine. */
int mprgp_context_set_cluster(mprgp_context *ctx, int cluster);
/* Instances larger than the largest cluster also take the cluster solver
 * when each CTA of that cluster covers at most `items` items (1..4; default
 * 1, the others then go to the persistent engine). */
int mprgp_context_set_cluster_items(mprgp_context *ctx, int items);

/* ---- problem: one QP instance resident in device memory ----------------- */
/* Replaces the reference's FixedSparseMatrix<T> + projector objects
 * (MPRGPSolver.h:459-500, MPRGPProjection.h): A, b, the constraints, x and
 * the power-method vector stay on the device between solves (warm starts). */
typedef struct mprgp_problem mprgp_problem;
int mprgp_problem_create(mprgp_context *ctx, int nv, mprgp_problem **out);
int mprgp_problem_destroy(mprgp_problem *prob);
/* precisions: bit 0 keep FP64 values, bit 1 keep an FP32 copy. on_device: the
 * pointers are device pointers (0 = host), holding their data when the call is
 * made (work on another stream that writes them has completed). */
int mprgp_problem_set_matrix(mprgp_problem *prob, int nnzb, const int *row_ptr, const int *cols,
                             const double *vals, int precisions, int on_device);
int mprgp_problem_set_rhs(mprgp_problem *prob, const double *b, int on_device);
int mprgp_problem_set_planes(mprgp_problem *prob, const int *plane_ptr, const double *planes,
                             int on_device);
int mprgp_problem_set_bounds(mprgp_problem *prob, const double *L, const double *U);
int mprgp_problem_set_x(mprgp_problem *prob, const double *x, int on_device);
int mprgp_problem_get_x(mprgp_problem *prob, double *x, int on_device);
/* face codes as the reference's projector.getFace(): one per constraint row
 * (planes, in plane_ptr order) or one per unknown (bounds). */
int mprgp_problem_num_constraints(mprgp_problem *prob, int *m);
int mprgp_problem_num_vertices(mprgp_problem *prob, int *nv);
/* The plane constraints as set: plane_ptr[nv+1] and planes[4 m] in the
 * (n, p) form (host arrays). */
int mprgp_problem_get_planes(mprgp_problem *prob, int *plane_ptr, double *planes);
int mprgp_problem_get_face(mprgp_problem *prob, unsigned char *face);
/* Power-method reuse (on by default): a solve whose power method starts from
 * the seeded random vector (no stored start vector in use) reuses the result
 * of the problem's last such power method when A, the seed and the precision
 * form are unchanged -- the power method is a deterministic function of
 * those, so alpha_bar, and with it the solve, are bitwise the same; the
 * skipped matrix passes do not appear in the stats.  set_matrix invalidates
 * it; enable = 0 turns it off (every solve runs the power method). */
int mprgp_problem_set_power_cache(mprgp_problem *prob, int enable);
int mprgp_problem_set_ev(mprgp_problem *prob, const double *ev);
int mprgp_problem_get_ev(mprgp_problem *prob, double *ev, int *valid);
/* Device-resident solve: x (set_x) is solved in place.  Mirrors
 * MPRGPxxx<double>::solve(A, B, projector, x, tol, max_it, name, ev). */
int mprgp_problem_solve(mprgp_problem *prob, const mprgp_options *opt, mprgp_stats *stats);
/* Step trace of the next solves (diagnostics): capacity records of 4 doubles
 * {event, iteration, residual, value}; event 1 CG commit / 2 CG exit (value
 * f(P(y)) - f(x)), 3 expansion, 4 proportioning, 5 loop top (value =
 * proportional test).  capacity 0 turns it off. */
int mprgp_problem_set_trace(mprgp_problem *prob, int capacity);
int mprgp_problem_get_trace(mprgp_problem *prob, double *out, int capacity, int *count);
/* y = A x with device pointers (FixedSparseMatrix::multiply, MPRGPSolver.h:469-473).
 * precision: MPRGP_PREC_FP64 or MPRGP_PREC_MIXED (FP32 values, FP32 accumulate). */
int mprgp_problem_spmv(mprgp_problem *prob, const double *x_dev, double *y_dev, int precision);
/* Device bytes held by a problem of this shape (admission accounting). */
size_t mprgp_problem_bytes(int nv, int nnzb, int nplanes, int precisions);

/* ---- one-call solve with host buffers ------------------------------------ */
/* Uploads A, b, constraints and x, solves, downloads x (and face).  This is
 * the entry the C++ façade calls for MPRGPDecoupledCon/GeneralCon/BoxBound/
 * LowerBound::solve.  plane_ptr/planes for kinds DECOUPLED/PLANES, L/U for
 * LOWER/BOX (U ignored for LOWER). ev may be NULL; if non-NULL it is the
 * reference's `Vec *ev` (length n): used as the power start when opt->use_ev
 * is set, and overwritten when the power method converges. */
int mprgp_solve_bsr(mprgp_context *ctx, int nv, int nnzb, const int *row_ptr, const int *cols,
                    const double *vals, const double *b, const int *plane_ptr,
                    const double *planes, const double *L, const double *U,
                    const mprgp_options *opt, double *x, unsigned char *face, double *ev,
                    mprgp_stats *stats);

/* ---- solve without allocating device memory ------------------------------ */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * while they solve (a real-time loop kept off the allocator, which can
 * synchronize the device; a plug-in inside a host program that owns all
 * device memory; a host under a fixed GPU memory quota).  Every pointer is
 * a device pointer the caller owns:
 * A as 3x3-block CSR, b, the per-vertex planes (n, p) with n.x + p >= 0, x
 * (solved in place) and optionally face (one byte per plane row).  The
 * solver's working memory lives in one 64 MiB file-scope device array that
 * every GPU loading the library holds until exit; problems that do not fit
 * (about 37k vertices in FP64) are rejected with MPRGP_INVALID.  The first
 * call on a device looks up that array's address (one-time set-up; make it
 * before any stream capture; the address is kept, so a device reset after
 * it is not supported).  All calls share the array: calls whose GPU work
 * overlaps race and must be serialized.  On an error status x and face are
 * left unchanged.  Kinds DECOUPLED and PLANES, monotone algorithm, FP64 or
 * MIXED; no stored power vector (use_ev = 0). */
int mprgp_solve_noalloc(void *stream, int nv, int nnzb, const int *row_ptr, const int *cols,
                        const double *vals, const double *b, const int *plane_ptr,
                        const double *planes, const mprgp_options *opt, double *x,
                        unsigned char *face, mprgp_stats *stats);

/* ---- ICA: the reference's comparison contact solver ---------------------- */
/* Replaces ICASolver (src/MPRGPSolver/ICASolver.h:287-463): ICASolver(max_it,
 * tol, gs_max_it, gs_tol); reset(A, r); solve(J, p, x) -> bool;
 * getIterations(), getResidual(), getLambda().  Solves
 *   A x = r + J^T lambda,  0 <= lambda _|_ J x - p >= 0
 * with A as 3x3-block CSR (host arrays, 9 values per block, row-major; every
 * row holds its diagonal block) and J as per-vertex planes (n, q) with
 * p = -q (0..3 planes a vertex; the reference's defaults are gs_max_it = 20,
 * gs_tol = 1e-3).  x: initial guess in, solution out (3 nv); lambda: one
 * multiplier per plane, in plane order.  Returns MPRGP_OK when the residual
 * ||A x - r - J^T lambda|| reached tol (the reference's true), else
 * MPRGP_NOT_CONVERGED; MPRGP_BUSY while the context's server has
 * asynchronous runs in flight. */
typedef struct mprgp_ica_stats {
  int iterations;       /* the reference's getIterations() */
  int converged;        /* 1: residual <= tol */
  double residual;      /* getResidual() */
  long long pgs_sweeps; /* projected Gauss-Seidel sweeps, all iterations */
  int levels;           /* dependency levels of the 3x3-block sweep */
  double device_ms;     /* device time of the solve */
} mprgp_ica_stats;
int mprgp_ica_solve(mprgp_context *ctx, int nv, int nnzb, const int *row_ptr, const int *cols,
                    const double *vals, const double *r, const int *plane_ptr,
                    const double *planes, double *x, double *lambda, int max_it, double tol,
                    int gs_max_it, double gs_tol, mprgp_ica_stats *stats);

/* ---- batched: many instances advance in one persistent launch ----------- */
int mprgp_solve_batch(mprgp_context *ctx, int count, mprgp_problem *const *probs,
                      const mprgp_options *opts, mprgp_stats *stats);

/* ---- serving: continuous batching of QP requests ------------------------- */
/* No counterpart in the reference API (its FEM driver solves one QP per frame,
 * MprgpFemSolver.cpp:521-533); this is the serving form of the solver.
 * A request is a new scene (BSR A, b, planes, x0; project_x0 applies) or,
 * with row_ptr == NULL, the next timestep of a live scene: only b is new, and
 * A, the planes, x (the last solution) and the face stay resident on the
 * device and warm-start the solve.  mode 0: the arrays are host memory,
 * copied at submit (num_planes may be -1: plane_ptr[nv] is used); mode 1:
 * device memory and mode 2: host memory (pinned memory is copied by DMA),
 * both read at admission, so the caller keeps them unchanged until the
 * request has completed; mode 1 needs num_planes = plane_ptr[nv].  Each step
 * admits
 * queued requests into free slots while their device footprint fits the HBM
 * budget (idle scenes are evicted least-recently-used first), advances all
 * admitted requests together by one engine quantum and retires the finished
 * ones.  Results do not depend on the mix: every instance reduces in a fixed
 * order.  Plane kinds (DECOUPLED, PLANES). */
typedef struct mprgp_server_config {
  size_t hbm_budget;  /* device bytes for resident scenes (0 = 80% of free) */
  int max_slots;      /* requests in flight (0 = 64) */
  int quantum_phases; /* engine macro-phases per step (0 = 256, < 0 = run
                         every admitted request to completion in one step) */
  int power_launches; /* power-method loop iterations per step (0..1003) */
  int cluster_quantum; /* phases per step of the small instances (cluster
                          solver; 0 = run them to completion in the step) */
  int lanes;          /* 0: each step runs every admitted request in one
                         engine run and waits for it; 2: small requests
                         (cluster solver) and large ones run on two
                         asynchronous lanes -- a step retires the runs that
                         finished, admits, starts a new run on every idle
                         lane and returns without waiting for it; 3..6: as
                         2, plus lanes - 2 lanes that run the large requests'
                         power method (power_launches per run; they share one
                         queue) before they join the large lane */
  size_t hbm_reserve; /* device bytes admission leaves free for other users of
                         the GPU: a new scene is admitted only while the
                         device's free memory (re-read at admission, plus the
                         context pool's unused blocks) stays above this after
                         it; otherwise it waits, and completes with MPRGP_OOM
                         if nothing else is in flight (0 = none) */
} mprgp_server_config;
typedef struct mprgp_server mprgp_server;
int mprgp_server_create(mprgp_context *ctx, const mprgp_server_config *cfg, mprgp_server **out);
int mprgp_server_destroy(mprgp_server *srv);
int mprgp_server_submit(mprgp_server *srv, int scene, int nv, int nnzb, const int *row_ptr,
                        const int *cols, const double *vals, const double *b,
                        const int *plane_ptr, const double *planes, const double *x0,
                        int num_planes, int mode, const mprgp_options *opt,
                        long long *ticket);
int mprgp_server_step(mprgp_server *srv, int *running, int *queued, int *completed);
/* Tickets that completed since the last poll (at most `capacity`, oldest
 * first); *count receives how many were written. */
int mprgp_server_poll(mprgp_server *srv, long long *tickets, int capacity, int *count);
/* state: 0 queued, 1 running, 2 done.  When done, copies x (3 nv), face and
 * stats, times = {submit, admit, done} in seconds, releases the ticket and
 * returns the solve's code. */
int mprgp_server_result(mprgp_server *srv, long long ticket, double *x, unsigned char *face,
                        mprgp_stats *stats, double *times, int *state);
int mprgp_server_info(mprgp_server *srv, size_t *budget, size_t *used, int *scenes);

/* ---- beam generator (synthetic implicit-Euler FEM QPs) ------------------- */
typedef struct mprgp_beam_params {
  int a, b, c;          /* cube counts along x, y (up), z */
  double edge;          /* cube edge [m] */
  double young, poisson, rho;
  double dt;            /* time step h */
  double gravity;       /* signed y acceleration, e.g. -9.8 */
  double lift;          /* lowest layer placed at y = -lift */
  double v0_sigma;      /* v0 ~ N(0, sigma^2) per component */
  int extra_planes_max; /* extra planes: per facet vertex (mode 1) or global (mode 0), */
  int extra_planes_min; /*   seeded in [min, max] */
  double active_frac;   /* mode 1: fraction of candidate vertices given facets;
                           mode 0: plane penetration at x0 as a fraction of lift */
  uint64_t seed;
  double plane_band;    /* a vertex gets a global plane if its gap at x0 < band */
  double max_tilt;      /* plane normals: uniform on the cap within max_tilt of +y */
  int plane_mode;       /* 2: corner walls x,z (default), 1: contact facets,
                           0: global tilted planes */
  int facet_layers;     /* facets go to vertices of the lowest facet_layers layers */
} mprgp_beam_params;
void mprgp_beam_default(mprgp_beam_params *p);
int mprgp_beam_sizes(const mprgp_beam_params *p, int *nv, int *nnzb, int *nplanes);
/* Fills BSR A = M + h^2 K (linear elasticity, lumped mass, Kuhn 6-tet cubes),
 * b = M(x0 + h v0) + h^2 M g + h^2 K X, x0 (unprojected), and the planes:
 * the floor y >= 0 on every vertex, then each global plane (normal uniform
 * on the upper hemisphere) on the vertices within plane_band of it. */
int mprgp_beam_build(const mprgp_beam_params *p, int *row_ptr, int *cols, double *vals,
                     double *b, double *x0, int *plane_ptr, double *planes);
/* The beam's tetrahedral mesh: tets[4 * 6abc] (vertex ids, the six Kuhn
 * tets of each cube), rest shape X[3 nv], and optionally the initial
 * positions x0[3 nv] and velocities v0[3 nv] that mprgp_beam_build uses. */
int mprgp_beam_mesh(const mprgp_beam_params *p, int *tets, double *X, double *x0, double *v0);

/* ---- plane-constraint generation on the GPU ---------------------------- */
/* The proximity query of LinearConCollider::handle(body, plane, delta)
 * (LinearConCollider.cpp:140-161) for planes[4 nplanes] = (n, p), |n| = 1,
 * in order: plane q becomes a constraint of vertex v when n.x_v + p - delta
 * <= 0, unless v already holds a plane within 1e-4 of it in (n, p)
 * (addConPlane, LinearConCollider.cpp:43-56); with decoupled = 1 only the
 * first such plane of a vertex (LinearConCollider.cpp:153-158).  x: vertex
 * positions (3 nv; host, or device with on_device = 1; NULL = the problem's
 * current x).  The lists replace the problem's constraints
 * (mprgp_problem_set_planes); a vertex that would need more than 3 planes
 * is an MPRGP_INVALID error.  *num_constraints receives the total. */
int mprgp_planes_collide(mprgp_context *ctx, mprgp_problem *prob, const double *x, int on_device,
                         int nplanes, const double *planes, double delta, int decoupled,
                         int *num_constraints);

/* ---- FEM assembly on the GPU ------------------------------------------- */
/* The system the reference's FEM driver builds before each solve
 * (MprgpFemSolver.cpp:315-356, FEMSystem::buildSystem FEMSystem.cpp:167-193)
 * for a linear material (FEMEnergy.cpp:657) and lumped mass
 * (FEMMesh.cpp:501-511):  A = M + h^2 K,  b = M (x + h v) + h^2 M g + h^2 K X.
 * mprgp_fem_create builds the block pattern (host, once per mesh) and the
 * per-tet geometry (device) from tets[4 ntet] and the rest shape X[3 nv];
 * mprgp_fem_assemble computes A and b on the device (one thread per block
 * row, deterministic) and loads them into `prob` (matrix with `precisions`,
 * right-hand side); mprgp_fem_rhs recomputes only b for a later timestep.
 * x, v: current positions and velocities (host, or device with
 * on_device = 1; v may be NULL).  mprgp_fem_get copies the last assembly
 * (row_ptr[nv+1], cols[nnzb], vals[9 nnzb], b[3 nv], mass[nv]) to the host. */
typedef struct mprgp_fem mprgp_fem;
int mprgp_fem_create(mprgp_context *ctx, int nv, int ntet, const int *tets, const double *X,
                     double young, double poisson, double rho, mprgp_fem **out);
int mprgp_fem_destroy(mprgp_fem *fem);
int mprgp_fem_sizes(mprgp_fem *fem, int *nv, int *nnzb);
int mprgp_fem_assemble(mprgp_fem *fem, double h, const double gravity[3], const double *x,
                       const double *v, int on_device, mprgp_problem *prob, int precisions);
int mprgp_fem_rhs(mprgp_fem *fem, double h, const double gravity[3], const double *x,
                  const double *v, int on_device, mprgp_problem *prob);
int mprgp_fem_get(mprgp_fem *fem, int *row_ptr, int *cols, double *vals, double *b,
                  double *mass);

#ifdef __cplusplus
}
#endif
#endif /* MPRGP_GPU_H */
