// server.cu -- a solve server with continuous batching.
//
// Requests (one Poisson solve each: dim, n nodes per side, f on the host,
// zero Dirichlet data, mixed form to rtol) are admitted as soon as a worker
// slot is free and the device memory of a solver for that size fits in the
// HBM budget.  Solvers (hierarchies, graphs) stay device-resident in a pool
// keyed by size and are reused; idle solvers of other sizes are evicted
// least-recently-used first when a new size needs room.  2D requests of one
// size waiting together are merged into one group solve (fishgpu_group: the
// batch's plane-stacked kernels, one launch per phase for all of them), up
// to batch_max; groups of 1, 2, 4, ... instances are pooled like solvers.
// Every worker drives its solve on its own stream, so requests that arrive
// while others run are admitted and their kernels overlap on the device.
// Latency is measured on the host from submission to completion.
#include <math.h>
#include <string.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/fishgpu.h"

namespace {

using clk = std::chrono::steady_clock;

struct Req {
  long long id;
  int dim, n;
  const double *f;
  double *u;
  clk::time_point t_submit, t_start, t_end;
  int status = -1;  // -1 queued, -2 running, >= 0 library status
  int its = 0, outer = 0;
  double relres = 0.0;
};

struct Pooled {
  fishgpu_solver *s;  // a solver, or
  fishgpu_group *g;   // a group of `count` 2D instances
  int dim, n, count;
  long long bytes;
  bool busy;
  clk::time_point last;
};

// the work a worker picked: requests (one, or up to batch_max merged 2D
// ones), the pooled entry (-1: create one, `need` bytes reserved)
struct Job {
  std::vector<long long> ids;
  int dim = 0, n = 0, count = 0;  // count > 0: a group of that many instances
  int slot = -1;
  long long need = 0;
};

}  // namespace

struct fishgpu_server_s {
  fishgpu_server_opts o;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<long long> queue;
  std::map<long long, Req> reqs;
  std::vector<Pooled> pool;
  long long used = 0;  // bytes of pooled solvers
  long long next_id = 1;
  bool stop = false;
  int device = 0;
  std::vector<std::thread> workers;
  // statistics
  long long completed = 0, created = 0, evicted = 0, group_solves = 0, grouped = 0;
};

static void make_opts(const fishgpu_server_opts &so, int dim, int n, fishgpu_opts *o) {
  fishgpu_opts_default(o);
  o->ctx.dim = dim;
  o->ctx.problem = FISHGPU_USER;
  o->mx = o->my = o->mz = n;
  if (dim < 3) o->mz = 1;
  if (dim < 2) o->my = 1;
  int levels = 1;
  for (int m = n; m > 3 && (m - 1) % 2 == 0; m = (m - 1) / 2 + 1) levels++;
  o->mg_levels = levels;
  o->pc_type = FISHGPU_PC_MG;
  o->precision = so.precision;
  o->rtol = so.rtol;
  o->norm_type = FISHGPU_NORM_UNPRECONDITIONED;
  // no persistent solves (nor cooperative V-cycle tails): one holds a block
  // on every SM for the whole solve, which serialises the concurrent solves a
  // server overlaps (measured on the serving stream: 978 against 1156
  // solves/s with them)
  o->persist = 0;
  o->coop_tail = 0;
}

static void group_opts(const fishgpu_server_opts &so, fishgpu_batch_opts *bo) {
  fishgpu_batch_opts_default(bo);
  bo->rtol = so.rtol;
  bo->tune = 0;  // fixed tiles: an instance's result does not depend on its group
  bo->tune_sweeps = 0;
}

// device bytes of a pooled entry, before it exists (replaced by the exact
// figure once it is created)
static long long entry_bytes(const fishgpu_server_opts &so, int dim, int n, int count) {
  fishgpu_opts o;
  make_opts(so, dim, n, &o);
  const long long b = fishgpu_solver_estimate_bytes(&o);
  if (b < 0 || count <= 0) return b;
  return count * (b + 2LL * n * n * (long long)sizeof(double)) + (1LL << 20);
}

// evicts idle entries, least recently used first, until `b` more bytes fit;
// false if they do not
static bool make_room(fishgpu_server_s *S, long long b) {
  while (S->used + b > S->o.hbm_budget_bytes) {
    int victim = -1;
    for (size_t p = 0; p < S->pool.size(); p++)
      if (!S->pool[p].busy && (victim < 0 || S->pool[p].last < S->pool[victim].last)) victim = (int)p;
    if (victim < 0) break;
    Pooled &v = S->pool[victim];
    if (v.s) fishgpu_solver_destroy(v.s);
    if (v.g) fishgpu_group_destroy(v.g);
    S->used -= v.bytes;
    S->pool.erase(S->pool.begin() + victim);
    S->evicted++;
  }
  return S->used + b <= S->o.hbm_budget_bytes;
}

// Picks queued work that can start now: the first request (in queue order)
// whose size has an idle pooled entry or room in the budget; a 2D request
// takes along the later queued 2D requests of its size (batch_max in all).
// Removes the picked requests from the queue; false if nothing can start.
static bool pick(fishgpu_server_s *S, Job *job) {
  for (size_t qi = 0; qi < S->queue.size(); qi++) {
    Req &r = S->reqs[S->queue[qi]];
    Job j;
    j.dim = r.dim;
    j.n = r.n;
    std::vector<size_t> at{qi};
    if (r.dim == 2 && S->o.batch_max > 1 && S->o.precision == FISHGPU_MIXED) {  // groups: the mixed form
      for (size_t qk = qi + 1; qk < S->queue.size() && (int)at.size() < S->o.batch_max; qk++) {
        const Req &o = S->reqs[S->queue[qk]];
        if (o.dim == 2 && o.n == r.n) at.push_back(qk);
        else if (S->o.fifo) break;  // strict order: only the run of equal requests behind this one
      }
      int c = 1;
      while (c < (int)at.size()) c *= 2;
      j.count = c < S->o.batch_max ? c : S->o.batch_max;
    }
    // an idle pooled entry of this size and count, else room for a new one;
    // a group that does not fit is tried at half the count (down to one,
    // then the request's own solver, whose size admission checked)
    bool ok = false;
    while (!ok) {
      for (size_t p = 0; p < S->pool.size() && !ok; p++) {
        const Pooled &e = S->pool[p];
        if (!e.busy && e.dim == j.dim && e.n == j.n && e.count == j.count) {
          j.slot = (int)p;
          ok = true;
        }
      }
      if (!ok) {
        const long long b = entry_bytes(S->o, j.dim, j.n, j.count);
        if (b >= 0 && make_room(S, b)) {
          j.need = b;
          S->used += b;  // reserved until the entry exists
          ok = true;
        }
      }
      if (ok || j.count == 0) break;
      j.count = j.count > 1 ? j.count / 2 : 0;
    }
    if (ok && (int)at.size() > (j.count > 0 ? j.count : 1)) at.resize(j.count > 0 ? j.count : 1);
    if (ok) {
      for (size_t t = at.size(); t-- > 0;) {
        j.ids.insert(j.ids.begin(), S->queue[at[t]]);
        S->queue.erase(S->queue.begin() + at[t]);
      }
      *job = std::move(j);
      return true;
    }
    if (qi == 0 && S->o.fifo) break;  // strict order: wait for room for the head
  }
  return false;
}

static void worker(fishgpu_server_s *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  while (true) {
    Job job;
    bool got = false;
    S->cv_work.wait(lk, [&] { return S->stop || (!S->queue.empty() && (got = pick(S, &job))); });
    if (S->stop && !got) return;
    const size_t k = job.ids.size();
    std::vector<const double *> fs(k);
    std::vector<double *> us(k);
    for (size_t q = 0; q < k; q++) {
      Req &r = S->reqs[job.ids[q]];
      r.status = -2;
      r.t_start = clk::now();
      fs[q] = r.f;
      us[q] = r.u;
    }
    fishgpu_solver *sol = nullptr;
    fishgpu_group *grp = nullptr;
    int slot = job.slot;
    if (slot >= 0) {
      S->pool[slot].busy = true;
      sol = S->pool[slot].s;
      grp = S->pool[slot].g;
    }
    lk.unlock();
    int rc = FISHGPU_OK;
    std::vector<int> its(k, 0), outer(k, 0);
    std::vector<double> rel(k, 0.0);
    if (job.count > 0) {
      if (!grp) {
        fishgpu_batch_opts bo;
        group_opts(S->o, &bo);
        rc = fishgpu_group_create(&bo, job.n, job.count, &grp);
      }
      if (!rc) rc = fishgpu_group_solve_host(grp, (int)k, fs.data(), us.data(), its.data(), outer.data(), rel.data());
    } else {
      if (!sol) {
        fishgpu_opts o;
        make_opts(S->o, job.dim, job.n, &o);
        rc = fishgpu_solver_create(&o, nullptr, &sol);
      }
      fishgpu_report rep;
      memset(&rep, 0, sizeof(rep));
      if (!rc) rc = fishgpu_solver_solve_host(sol, fs[0], nullptr, us[0], &rep);
      its[0] = rep.its;
      outer[0] = rep.outer_its;
      rel[0] = rep.true_rel_resid;
    }
    lk.lock();
    if (slot < 0) {
      S->used -= job.need;
      if (sol || grp) {
        const long long bytes = sol ? fishgpu_solver_bytes(sol) : fishgpu_group_bytes(grp);
        S->pool.push_back(Pooled{sol, grp, job.dim, job.n, job.count, bytes, false, clk::now()});
        S->used += bytes;
        S->created++;
        slot = (int)S->pool.size() - 1;
      }
    }
    if (slot >= 0) {
      // the pool may have moved: find this entry again
      for (auto &e : S->pool)
        if ((sol && e.s == sol) || (grp && e.g == grp)) {
          e.busy = false;
          e.last = clk::now();
        }
    }
    if (job.count > 0) {
      S->group_solves++;
      S->grouped += (long long)k;
    }
    for (size_t q = 0; q < k; q++) {
      Req &rr = S->reqs[job.ids[q]];
      rr.t_end = clk::now();
      rr.status = rc;
      rr.its = its[q];
      rr.outer = outer[q];
      rr.relres = rel[q];
      S->completed++;
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}

extern "C" int fishgpu_server_opts_default(fishgpu_server_opts *o) {
  if (!o) return FISHGPU_ERR_ARG;
  memset(o, 0, sizeof(*o));
  o->hbm_budget_bytes = 120LL << 30;
  o->workers = 8;
  o->rtol = 1e-8;
  o->precision = FISHGPU_MIXED;
  o->fifo = 0;
  o->batch_max = 16;
  return FISHGPU_OK;
}

extern "C" int fishgpu_server_create(const fishgpu_server_opts *o, fishgpu_server **out) {
  if (!o || !out || o->workers < 1 || o->workers > 256 || o->hbm_budget_bytes <= 0 || !(o->rtol > 0) ||
      o->batch_max < 1 || o->batch_max > 4096)
    return FISHGPU_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return FISHGPU_ERR_NODEVICE;
  }
  fishgpu_server *S = new fishgpu_server();
  S->o = *o;
  cudaGetDevice(&S->device);
  for (int w = 0; w < o->workers; w++) S->workers.emplace_back(worker, S);
  *out = S;
  return FISHGPU_OK;
}

extern "C" int fishgpu_server_submit(fishgpu_server *S, int dim, int n, const double *f_host, double *u_host,
                                     long long *ticket) {
  if (!S || !f_host || !u_host || !ticket || dim < 1 || dim > 3 || n < 3 || ((n - 1) & (n - 2)) != 0)
    return FISHGPU_ERR_ARG;
  fishgpu_opts o;
  make_opts(S->o, dim, n, &o);
  const long long b = fishgpu_solver_estimate_bytes(&o);
  if (b < 0 || b > S->o.hbm_budget_bytes) return FISHGPU_ERR_NOMEM;  // can never be admitted
  std::lock_guard<std::mutex> lk(S->mu);
  Req r;
  r.id = S->next_id++;
  r.dim = dim;
  r.n = n;
  r.f = f_host;
  r.u = u_host;
  r.t_submit = clk::now();
  S->reqs[r.id] = r;
  S->queue.push_back(r.id);
  *ticket = r.id;
  S->cv_work.notify_one();
  return FISHGPU_OK;
}

// Waits for `ticket` (timeout_ms < 0: no limit).  Fills the result and forgets
// the request.  Returns FISHGPU_ERR_TIMEOUT if it has not finished in time.
extern "C" int fishgpu_server_wait(fishgpu_server *S, long long ticket, double timeout_ms,
                                   fishgpu_server_result *res) {
  if (!S || !res) return FISHGPU_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return FISHGPU_ERR_ARG;
  auto ready = [&] { return S->reqs[ticket].status >= 0; };
  if (timeout_ms < 0) S->cv_done.wait(lk, ready);
  else if (!S->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready))
    return FISHGPU_ERR_TIMEOUT;
  const Req &r = S->reqs[ticket];
  auto ms = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
  res->status = r.status;
  res->its = r.its;
  res->outer_its = r.outer;
  res->rel_resid = r.relres;
  res->queue_ms = ms(r.t_submit, r.t_start);
  res->service_ms = ms(r.t_start, r.t_end);
  res->latency_ms = ms(r.t_submit, r.t_end);
  S->reqs.erase(ticket);
  return FISHGPU_OK;
}

extern "C" int fishgpu_server_stats(fishgpu_server *S, long long *pooled_bytes, int *pooled_solvers,
                                    long long *created, long long *evicted) {
  if (!S) return FISHGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  if (pooled_bytes) *pooled_bytes = S->used;
  if (pooled_solvers) *pooled_solvers = (int)S->pool.size();
  if (created) *created = S->created;
  if (evicted) *evicted = S->evicted;
  return FISHGPU_OK;
}

extern "C" int fishgpu_server_group_stats(fishgpu_server *S, long long *group_solves, long long *grouped_requests) {
  if (!S) return FISHGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  if (group_solves) *group_solves = S->group_solves;
  if (grouped_requests) *grouped_requests = S->grouped;
  return FISHGPU_OK;
}

extern "C" int fishgpu_server_destroy(fishgpu_server *S) {
  if (!S) return FISHGPU_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->queue.clear();
  }
  S->cv_work.notify_all();
  for (auto &t : S->workers) t.join();
  for (auto &e : S->pool) {
    if (e.s) fishgpu_solver_destroy(e.s);
    if (e.g) fishgpu_group_destroy(e.g);
  }
  delete S;
  return FISHGPU_OK;
}
