// Continuous-batching QP server (the serving form).
//
// Requests are either new scenes (host A, b, planes, x0, copied at submit) or
// follow-up timesteps of a live scene (a new b; A, the planes, x and the face
// stay resident from the previous solve and warm-start the next one, as the
// reference's FEM driver re-solves each frame, MprgpFemSolver.cpp:521-533).
// Each mprgp_server_step admits queued requests into free slots while their
// device footprint fits the HBM budget (evicting idle scenes, least recently
// used first), then advances every admitted request -- small ones on the
// cluster solver to completion (or by cluster_quantum phases), large ones by
// one engine quantum, all in the same run, so their work overlaps on the
// device -- and retires the ones that finished.  In the asynchronous form
// (two lanes) small and large requests run on separate engine lanes, each on
// its own stream: a step retires the lane runs that finished, admits, starts
// a run on every idle lane and returns without waiting, so a small request
// that arrives while the large ones are mid-solve starts at once.  A
// request's result does not depend on what else is in flight or on the form:
// each instance's reductions run in a fixed order.
#include <algorithm>
#include <chrono>
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
int engine_run(mprgp_context *c, int n, mprgp_problem *const *probs, const mprgp_options *opts,
               const int *fresh, int quantum, int power_launches, int cluster_quantum,
               mprgp_stats *stats, int *done);
int engine_begin(mprgp_context *c, int lane, int n, mprgp_problem *const *probs,
                 const mprgp_options *opts, const int *fresh, int quantum, int power_launches,
                 int cluster_quantum);
int engine_ready(mprgp_context *c, int lane);
int engine_end(mprgp_context *c, int lane, mprgp_stats *stats, int *done);
int engine_lane_of(const mprgp_context *c, int nv);
int context_room(mprgp_context *c, size_t *room);
int engine_needs_power(const mprgp_problem *p, const mprgp_options *o);
int engine_in_power(const mprgp_problem *p);
int problem_read_result(mprgp_problem *p, double *x, unsigned char *face);
void set_last_error(const char *what);
}  // namespace mprgp

namespace {

struct Request {
  long long ticket = 0;
  int scene = 0;
  bool followup = false;
  int nv = 0, nnzb = 0, m = 0;
  std::vector<int> row_ptr, cols, plane_ptr;
  std::vector<double> vals, b, planes, x0;
  // by-reference submission (mode 1 device, 2 host): the caller's arrays,
  // read at admission; mode 0 keeps the copies above
  int mode = 0;
  const int *p_row_ptr = nullptr, *p_cols = nullptr, *p_plane_ptr = nullptr;
  const double *p_vals = nullptr, *p_b = nullptr, *p_planes = nullptr, *p_x0 = nullptr;
  mprgp_options opt{};
  int state = 0;  // 0 queued, 1 running, 2 done
  int lane = 0;   // asynchronous form: 0 small, 1 large, 2 large in the power method
  bool fresh = true;  // the next run starts its solve
  int code = 0;
  std::vector<double> x;
  std::vector<unsigned char> face;
  mprgp_stats stats{};
  double t_submit = 0, t_admit = 0, t_done = 0;
};

constexpr int kMaxPowerLanes = 4;  // asynchronous power-method lanes at most

struct Scene {
  mprgp_problem *prob = nullptr;
  size_t bytes = 0;
  long long last_use = 0;
  bool busy = false;
  int m = 0;
};

double now_s() {
  using clk = std::chrono::steady_clock;
  static const clk::time_point t0 = clk::now();
  return std::chrono::duration<double>(clk::now() - t0).count();
}

int err(int code, const char *what) {
  mprgp::set_last_error(what);
  return code;
}

}  // namespace

struct mprgp_server {
  mprgp_context *ctx = nullptr;
  size_t budget = 0, used = 0;
  size_t reserve = 0;  // device bytes admission leaves free for other users
  int max_slots = 64, quantum = 256, power_launches = 256, cluster_quantum = 0;
  long long next_ticket = 1, clock = 0;
  std::deque<long long> queue;
  std::map<long long, Request> reqs;
  std::map<int, Scene> scenes;
  std::vector<long long> running;
  std::vector<char> fresh_flag;  // parallel to running
  std::deque<long long> completed;  // finished, not yet polled
  // asynchronous form: per lane (small; large; large in the power method,
  // three-lane form only) the admitted requests waiting for its next run and
  // those in its run in flight.  Server lane l runs on engine lane l + 1.
  int lanes = 0, npow = 0;  // npow: power lanes (lanes - 2 when lanes >= 3)
  int unretired = 0;        // finished in this step, results not read back yet
  struct LaneQ {
    std::vector<long long> pending, in_run;
    bool active = false;
  } lane[2 + kMaxPowerLanes];  // the power lanes share lane[2].pending
};

namespace {

void release_scene(mprgp_server *s, std::map<int, Scene>::iterator it) {
  mprgp_problem_destroy(it->second.prob);
  s->used -= it->second.bytes;
  s->scenes.erase(it);
}

// Frees idle scenes, least recently used first, until `need` bytes fit.
bool make_room(mprgp_server *s, size_t need) {
  while (s->used + need > s->budget) {
    auto victim = s->scenes.end();
    for (auto it = s->scenes.begin(); it != s->scenes.end(); ++it)
      if (!it->second.busy && (victim == s->scenes.end() ||
                               it->second.last_use < victim->second.last_use))
        victim = it;
    if (victim == s->scenes.end()) return false;
    release_scene(s, victim);
  }
  return true;
}

// Device room for new scenes, read once per admission pass (lazily) and
// tracked as scenes are admitted or evicted within it.
struct Room {
  bool known = false;
  size_t bytes = 0;
};

// Whether a new scene of `need` bytes leaves the server's reserve free on the
// device.  The device's free memory is re-read (other users of the GPU
// allocate too), and idle scenes are evicted, least recently used first,
// while it does not fit (their memory returns to the context's pool, which
// counts as room).
int device_fits(mprgp_server *s, Room &room, size_t need, bool *fits) {
  for (;;) {
    if (!room.known) {
      const int rc = mprgp::context_room(s->ctx, &room.bytes);
      if (rc) return rc;
      room.known = true;
    }
    if (room.bytes >= need && room.bytes - need >= s->reserve) {
      *fits = true;
      return MPRGP_OK;
    }
    auto victim = s->scenes.end();
    for (auto it = s->scenes.begin(); it != s->scenes.end(); ++it)
      if (!it->second.busy && (victim == s->scenes.end() ||
                               it->second.last_use < victim->second.last_use))
        victim = it;
    if (victim == s->scenes.end()) {
      *fits = false;
      return MPRGP_OK;
    }
    release_scene(s, victim);
    room.known = false;
  }
}

int admit(mprgp_server *s, Request &r) {
  if (r.followup) {
    auto it = s->scenes.find(r.scene);
    Scene &sc = it->second;
    int rc = r.mode ? mprgp_problem_set_rhs(sc.prob, r.p_b, r.mode == 1)
                    : mprgp_problem_set_rhs(sc.prob, r.b.data(), 0);
    if (rc) return rc;
    sc.busy = true;
    sc.last_use = ++s->clock;
    return MPRGP_OK;
  }
  const int prec = r.opt.precision == MPRGP_PREC_MIXED ? 3 : 1;
  const size_t bytes = mprgp_problem_bytes(r.nv, r.nnzb, r.m, prec);
  auto old = s->scenes.find(r.scene);
  if (old != s->scenes.end() && !old->second.busy) release_scene(s, old);
  Scene sc;
  int rc = mprgp_problem_create(s->ctx, r.nv, &sc.prob);
  // planes before the matrix: the SELL layout (which depends on the planes)
  // is then built once
  if (r.mode) {
    const int dev = r.mode == 1;
    if (!rc) rc = mprgp_problem_set_planes(sc.prob, r.p_plane_ptr, r.p_planes, dev);
    if (!rc) rc = mprgp_problem_set_matrix(sc.prob, r.nnzb, r.p_row_ptr, r.p_cols, r.p_vals, prec, dev);
    if (!rc) rc = mprgp_problem_set_rhs(sc.prob, r.p_b, dev);
    if (!rc) rc = mprgp_problem_set_x(sc.prob, r.p_x0, dev);
  } else {
    if (!rc) rc = mprgp_problem_set_planes(sc.prob, r.plane_ptr.data(), r.planes.data(), 0);
    if (!rc) rc = mprgp_problem_set_matrix(sc.prob, r.nnzb, r.row_ptr.data(), r.cols.data(),
                                           r.vals.data(), prec, 0);
    if (!rc) rc = mprgp_problem_set_rhs(sc.prob, r.b.data(), 0);
    if (!rc) rc = mprgp_problem_set_x(sc.prob, r.x0.data(), 0);
  }
  if (rc) {
    if (sc.prob) mprgp_problem_destroy(sc.prob);
    return rc;
  }
  sc.bytes = bytes;
  sc.busy = true;
  sc.last_use = ++s->clock;
  sc.m = r.m;
  s->used += bytes;
  s->scenes[r.scene] = sc;
  // host copies are no longer needed
  std::vector<int>().swap(r.row_ptr);
  std::vector<int>().swap(r.cols);
  std::vector<double>().swap(r.vals);
  return MPRGP_OK;
}

}  // namespace

namespace {

int in_flight(const mprgp_server *s) {
  if (!s->lanes) return (int)s->running.size();
  int k = s->unretired;  // their scenes are still busy
  for (const auto &q : s->lane) k += (int)(q.pending.size() + q.in_run.size());
  return k;
}

// Admission: FIFO, skipping requests that do not fit yet.  A new scene that
// does not fit while nothing else is in flight can never fit: it completes
// with MPRGP_OOM.
void admit_queued(mprgp_server *s) {
  mprgp::NvtxScope range("mprgp admit");
  Room room;
  for (auto it = s->queue.begin(); it != s->queue.end();) {
    if (in_flight(s) >= s->max_slots) break;
    Request &r = s->reqs[*it];
    bool ok = true;
    if (r.followup) {
      auto sc = s->scenes.find(r.scene);
      if (sc == s->scenes.end()) {  // evicted meanwhile: cannot warm start
        r.state = 2;
        r.code = MPRGP_INVALID;
        r.stats.code = r.code;
        s->completed.push_back(r.ticket);
        it = s->queue.erase(it);
        continue;
      }
      ok = !sc->second.busy;
    } else {
      const int prec = r.opt.precision == MPRGP_PREC_MIXED ? 3 : 1;
      const size_t bytes = mprgp_problem_bytes(r.nv, r.nnzb, r.m, prec);
      auto sc = s->scenes.find(r.scene);
      ok = (sc == s->scenes.end() || !sc->second.busy) && make_room(s, bytes);
      if (ok) {
        const int rc = device_fits(s, room, bytes, &ok);
        if (rc == MPRGP_OK && !ok && in_flight(s) == 0) {
          mprgp::set_last_error("server: a new scene does not fit in the device's free memory");
          r.state = 2;
          r.code = MPRGP_OOM;
          r.stats.code = r.code;
          s->completed.push_back(r.ticket);
          it = s->queue.erase(it);
          continue;
        }
        ok = ok && rc == MPRGP_OK;
      }
    }
    if (!ok) {
      ++it;
      continue;
    }
    const int rc = admit(s, r);
    if (rc == MPRGP_OOM && in_flight(s) > 0) {  // an allocation failed: retry later
      room.known = false;
      ++it;
      continue;
    }
    if (!r.followup) room.known = false;  // the new scene took device memory
    if (rc) {
      r.state = 2;
      r.code = rc;
      r.stats.code = r.code;
      s->completed.push_back(r.ticket);
      it = s->queue.erase(it);
      continue;
    }
    r.state = 1;
    r.t_admit = now_s();
    r.fresh = true;
    if (s->lanes) {
      r.lane = mprgp::engine_lane_of(s->ctx, r.nv) == 1 ? 0 : 1;
      if (r.lane == 1 && s->npow > 0 &&
          mprgp::engine_needs_power(s->scenes[r.scene].prob, &r.opt))
        r.lane = 2;
      s->lane[r.lane].pending.push_back(r.ticket);
    } else {
      s->running.push_back(r.ticket);
      s->fresh_flag.push_back(1);
    }
    it = s->queue.erase(it);
  }
}

// A finished request: its solution and face are read back, its scene freed
// for the next request.
void retire(mprgp_server *s, Request &r, const mprgp_stats &st) {
  Scene &sc = s->scenes[r.scene];
  r.stats = st;
  r.code = st.code;
  mprgp::problem_read_result(sc.prob, r.x.data(), sc.m > 0 ? r.face.data() : nullptr);
  sc.busy = false;
  r.state = 2;
  r.t_done = now_s();
  s->completed.push_back(r.ticket);
}

// An engine run's return code that ends the step: a device or runtime
// failure.  A request's own result code (breakdown, an invalid matrix) is
// its result and leaves the others running.
bool fatal(int rc) {
  return rc == MPRGP_TIMEOUT || rc == MPRGP_CUDA_ERROR || rc == MPRGP_NO_DEVICE ||
         rc == MPRGP_OOM;
}

// The synchronous form: one engine run over every admitted request.
int step_sync(mprgp_server *s, int *ncomp) {
  const int n = (int)s->running.size();
  if (n == 0) return MPRGP_OK;
  std::vector<mprgp_problem *> probs(n);
  std::vector<mprgp_options> opts(n);
  std::vector<int> fresh(n), done(n, 0);
  std::vector<mprgp_stats> st(n);
  for (int i = 0; i < n; ++i) {
    Request &r = s->reqs[s->running[i]];
    probs[i] = s->scenes[r.scene].prob;
    opts[i] = r.opt;
    fresh[i] = s->fresh_flag[i];
  }
  const int rc = mprgp::engine_run(s->ctx, n, probs.data(), opts.data(), fresh.data(),
                                   s->quantum, s->power_launches, s->cluster_quantum,
                                   st.data(), done.data());
  if (fatal(rc)) return rc;
  std::vector<long long> still;
  std::vector<char> still_fresh;
  for (int i = 0; i < n; ++i) {
    Request &r = s->reqs[s->running[i]];
    if (!done[i]) {
      still.push_back(r.ticket);
      still_fresh.push_back(0);
      continue;
    }
    retire(s, r, st[i]);
    ++*ncomp;
  }
  s->running.swap(still);
  s->fresh_flag.swap(still_fresh);
  return MPRGP_OK;
}

// Takes the results of lane l's run if it has finished.  Unfinished
// requests lead the lane's next run (a power lane's, the shared power
// queue), except that those of a power lane that have left the power method
// move on to the large lane.  Finished requests go to `fin` (ticket and
// stats); the caller reads their results back.
int finish_lane(mprgp_server *s, int l, std::vector<std::pair<long long, mprgp_stats>> &fin) {
  auto &q = s->lane[l];
  if (!q.active || mprgp::engine_ready(s->ctx, 1 + l) == 0) return MPRGP_OK;
  const int n = (int)q.in_run.size();
  std::vector<mprgp_stats> st(n);
  std::vector<int> done(n, 0);
  q.active = false;
  const int rc = mprgp::engine_end(s->ctx, 1 + l, st.data(), done.data());
  if (fatal(rc)) return rc;
  std::vector<long long> keep;
  for (int i = 0; i < n; ++i) {
    Request &r = s->reqs[q.in_run[i]];
    if (!done[i]) {
      r.fresh = false;
      if (l >= 2 && !mprgp::engine_in_power(s->scenes[r.scene].prob)) {
        r.lane = 1;
        s->lane[1].pending.push_back(r.ticket);
      } else {
        keep.push_back(r.ticket);
      }
      continue;
    }
    fin.emplace_back(r.ticket, st[i]);
  }
  q.in_run.clear();
  auto &pend = l >= 2 ? s->lane[2].pending : q.pending;
  pend.insert(pend.begin(), keep.begin(), keep.end());
  return MPRGP_OK;
}

// Starts a run on lane l over its pending requests (a power lane: the shared
// power queue) if the lane is idle.
int start_lane(mprgp_server *s, int l) {
  auto &q = s->lane[l];
  auto &pend = l >= 2 ? s->lane[2].pending : q.pending;
  if (q.active || pend.empty()) return MPRGP_OK;
  q.in_run.swap(pend);
  pend.clear();
  const int n = (int)q.in_run.size();
  std::vector<mprgp_problem *> probs(n);
  std::vector<mprgp_options> opts(n);
  std::vector<int> fresh(n);
  for (int i = 0; i < n; ++i) {
    Request &r = s->reqs[q.in_run[i]];
    probs[i] = s->scenes[r.scene].prob;
    opts[i] = r.opt;
    fresh[i] = r.fresh ? 1 : 0;
  }
  // a power lane runs the power loop alone; with power lanes, the large lane
  // runs no power loop of its own
  const int quantum = l >= 2 ? -1 : s->quantum;
  const int power = (l == 1 && s->npow > 0) ? 0 : s->power_launches;
  const int rc = mprgp::engine_begin(s->ctx, 1 + l, n, probs.data(), opts.data(), fresh.data(),
                                     quantum, power, s->cluster_quantum);
  if (rc) return rc;
  q.active = true;
  return MPRGP_OK;
}

// The asynchronous form: take what the lanes finished, admit, start every
// idle lane, and only then read the finished requests' results back (so a
// lane with work does not wait for the reads), admitting and starting once
// more for follow-ups whose scene those requests held; when none of that
// happened, wait a little for a lane to finish (the caller may have requests
// to submit meanwhile).
int step_async(mprgp_server *s, int *ncomp) {
  const int nl = 2 + s->npow;
  std::vector<std::pair<long long, mprgp_stats>> fin;
  auto read_back = [&]() {  // every finished request, also on an error return
    mprgp::NvtxScope range("mprgp read back");
    for (auto &f : fin) {
      retire(s, s->reqs[f.first], f.second);
      ++*ncomp;
    }
    fin.clear();
    s->unretired = 0;
  };
  for (int l = nl - 1; l >= 0; --l) {  // the power lanes first: they feed the large lane
    const int rc = finish_lane(s, l, fin);
    if (rc) {
      read_back();
      return rc;
    }
  }
  const size_t queued = s->queue.size();
  bool started = false;
  s->unretired = (int)fin.size();
  for (int pass = 0; pass < 2; ++pass) {
    admit_queued(s);
    for (int l = 0; l < nl; ++l) {
      const bool idle = !s->lane[l].active;
      const int rc = start_lane(s, l);
      if (rc) {
        read_back();
        return rc;
      }
      started |= idle && s->lane[l].active;
    }
    if (fin.empty()) break;
    read_back();
  }
  if (*ncomp || started || s->queue.size() != queued) return MPRGP_OK;
  const double until = now_s() + 5e-4;
  while (now_s() < until) {
    bool any = false, ready = false;
    for (int l = 0; l < nl; ++l) {
      if (!s->lane[l].active) continue;
      any = true;
      ready |= mprgp::engine_ready(s->ctx, 1 + l) != 0;
    }
    if (!any || ready) break;
  }
  return MPRGP_OK;
}

}  // namespace

extern "C" {

int mprgp_server_create(mprgp_context *ctx, const mprgp_server_config *cfg, mprgp_server **out) {
  if (!ctx || !out) return err(MPRGP_INVALID, "server_create");
  auto *s = new mprgp_server();
  s->ctx = ctx;
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  s->budget = (cfg && cfg->hbm_budget) ? cfg->hbm_budget : (size_t)(0.8 * (double)fr);
  s->reserve = cfg ? cfg->hbm_reserve : 0;
  if (cfg && cfg->max_slots > 0) s->max_slots = cfg->max_slots;
  if (cfg && cfg->quantum_phases > 0) s->quantum = cfg->quantum_phases;
  if (cfg && cfg->quantum_phases < 0) s->quantum = 0;  // each step runs to completion
  if (cfg && cfg->cluster_quantum > 0) s->cluster_quantum = cfg->cluster_quantum;
  if (cfg && cfg->power_launches >= 0) s->power_launches = std::min(cfg->power_launches, 1003);
  if (cfg && (cfg->lanes == 1 || cfg->lanes < 0 || cfg->lanes > 2 + kMaxPowerLanes)) {
    delete s;
    return err(MPRGP_INVALID, "server_create: lanes must be 0 or 2..6");
  }
  s->lanes = cfg ? cfg->lanes : 0;
  s->npow = s->lanes >= 3 ? s->lanes - 2 : 0;
  *out = s;
  return MPRGP_OK;
}

int mprgp_server_destroy(mprgp_server *s) {
  if (!s) return MPRGP_OK;
  for (int l = 0; l < 2 + kMaxPowerLanes; ++l)  // runs in flight end before their problems go
    if (s->lane[l].active) mprgp::engine_end(s->ctx, 1 + l, nullptr, nullptr);
  for (auto &kv : s->scenes) mprgp_problem_destroy(kv.second.prob);
  delete s;
  return MPRGP_OK;
}

int mprgp_server_submit(mprgp_server *s, int scene, int nv, int nnzb, const int *row_ptr,
                        const int *cols, const double *vals, const double *b,
                        const int *plane_ptr, const double *planes, const double *x0,
                        int num_planes, int mode, const mprgp_options *opt,
                        long long *ticket) {
  if (!s || !opt || !ticket || nv <= 0 || !b) return err(MPRGP_INVALID, "server_submit");
  if (opt->kind != MPRGP_KIND_DECOUPLED && opt->kind != MPRGP_KIND_PLANES)
    return err(MPRGP_INVALID, "server_submit: plane kinds only");
  Request r;
  r.scene = scene;
  r.opt = *opt;
  r.nv = nv;
  if (mode < 0 || mode > 2) return err(MPRGP_INVALID, "server_submit: mode");
  r.mode = mode;
  const size_t n = 3 * (size_t)nv;
  if (r.mode) r.p_b = b;
  else r.b.assign(b, b + n);
  if (row_ptr == nullptr) {  // follow-up timestep of a live scene
    auto it = s->scenes.find(scene);
    if (it == s->scenes.end()) return err(MPRGP_INVALID, "server_submit: scene not resident");
    r.followup = true;
    r.opt.project_x0 = 0;  // x is the scene's last solution (feasible)
    r.m = it->second.m;
  } else {
    if (!cols || !vals || !plane_ptr || !x0 || nnzb <= 0)
      return err(MPRGP_INVALID, "server_submit: missing arrays");
    r.nnzb = nnzb;
    if (r.mode == 1) {
      if (num_planes < 0) return err(MPRGP_INVALID, "server_submit: num_planes");
      r.m = num_planes;
    } else {
      r.m = plane_ptr[nv];
      if (num_planes >= 0 && num_planes != r.m)
        return err(MPRGP_INVALID, "server_submit: num_planes != plane_ptr[nv]");
    }
    if (r.mode) {
      r.p_row_ptr = row_ptr;
      r.p_cols = cols;
      r.p_vals = vals;
      r.p_plane_ptr = plane_ptr;
      r.p_planes = planes;
      r.p_x0 = x0;
    } else {
      r.row_ptr.assign(row_ptr, row_ptr + nv + 1);
      r.cols.assign(cols, cols + nnzb);
      r.vals.assign(vals, vals + 9 * (size_t)nnzb);
      r.plane_ptr.assign(plane_ptr, plane_ptr + nv + 1);
      r.planes.assign(planes, planes + 4 * (size_t)r.m);
      r.x0.assign(x0, x0 + n);
    }
  }
  r.face.assign(std::max(r.m, 1), 0);
  r.ticket = s->next_ticket++;
  r.x.assign(n, 0.0);
  r.t_submit = now_s();
  *ticket = r.ticket;
  s->queue.push_back(r.ticket);
  s->reqs.emplace(r.ticket, std::move(r));
  return MPRGP_OK;
}

int mprgp_server_step(mprgp_server *s, int *running, int *queued, int *completed) {
  if (!s) return err(MPRGP_INVALID, "server_step");
  int ncomp = 0, rc;
  if (s->lanes) {
    rc = step_async(s, &ncomp);
  } else {
    admit_queued(s);
    rc = step_sync(s, &ncomp);
  }
  if (rc) return rc;
  if (running) *running = in_flight(s);
  if (queued) *queued = (int)s->queue.size();
  if (completed) *completed = ncomp;
  return MPRGP_OK;
}

int mprgp_server_result(mprgp_server *s, long long ticket, double *x, unsigned char *face,
                        mprgp_stats *stats, double *times, int *state) {
  if (!s) return err(MPRGP_INVALID, "server_result");
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return err(MPRGP_INVALID, "server_result: unknown ticket");
  Request &r = it->second;
  if (state) *state = r.state;
  if (r.state != 2) return MPRGP_OK;
  if (x) std::copy(r.x.begin(), r.x.end(), x);
  if (face) std::copy(r.face.begin(), r.face.end(), face);
  if (stats) *stats = r.stats;
  if (times) {
    times[0] = r.t_submit;
    times[1] = r.t_admit;
    times[2] = r.t_done;
  }
  const int code = r.code;
  s->reqs.erase(it);
  return code;
}

int mprgp_server_poll(mprgp_server *s, long long *tickets, int capacity, int *count) {
  if (!s || !count || capacity < 0 || (capacity > 0 && !tickets))
    return err(MPRGP_INVALID, "server_poll");
  int k = 0;
  while (k < capacity && !s->completed.empty()) {
    tickets[k++] = s->completed.front();
    s->completed.pop_front();
  }
  *count = k;
  return MPRGP_OK;
}

int mprgp_server_info(mprgp_server *s, size_t *budget, size_t *used, int *scenes) {
  if (!s) return err(MPRGP_INVALID, "server_info");
  if (budget) *budget = s->budget;
  if (used) *used = s->used;
  if (scenes) *scenes = (int)s->scenes.size();
  return MPRGP_OK;
}

}  // extern "C"
