// server.cu -- a solve server with continuous batching.
//
// Requests (one Poisson solve each: dim, n nodes per side, f on the host,
// zero Dirichlet data, mixed form to rtol) are admitted as soon as a worker
// slot is free and the device memory of a solver for that size fits in the
// HBM budget.  Solvers (hierarchies, graphs) stay device-resident in a pool
// keyed by (dim, n) and are reused; idle solvers of other sizes are evicted
// least-recently-used first when a new size needs room.  Every worker drives
// its solve on its own stream, so requests that arrive while others run are
// admitted and their kernels overlap on the device.  Latency is measured on
// the host from submission to completion.
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
  fishgpu_solver *s;
  int dim, n;
  long long bytes;
  bool busy;
  clk::time_point last;
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
  long long completed = 0, created = 0, evicted = 0;
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
}

// Picks a queued request that can start now; returns its id (0: none) and the
// pooled solver index (-1: create one after unlocking, bytes reserved).
static long long pick(fishgpu_server_s *S, int *slot, long long *need) {
  for (size_t qi = 0; qi < S->queue.size(); qi++) {
    Req &r = S->reqs[S->queue[qi]];
    for (size_t p = 0; p < S->pool.size(); p++) {
      Pooled &e = S->pool[p];
      if (!e.busy && e.dim == r.dim && e.n == r.n) {
        *slot = (int)p;
        *need = 0;
        const long long id = r.id;
        S->queue.erase(S->queue.begin() + qi);
        return id;
      }
    }
    fishgpu_opts o;
    make_opts(S->o, r.dim, r.n, &o);
    const long long b = fishgpu_solver_estimate_bytes(&o);
    if (b < 0) continue;
    // evict idle solvers of other sizes, least recently used first, while needed
    while (S->used + b > S->o.hbm_budget_bytes) {
      int victim = -1;
      for (size_t p = 0; p < S->pool.size(); p++)
        if (!S->pool[p].busy && (victim < 0 || S->pool[p].last < S->pool[victim].last)) victim = (int)p;
      if (victim < 0) break;
      fishgpu_solver_destroy(S->pool[victim].s);
      S->used -= S->pool[victim].bytes;
      S->pool.erase(S->pool.begin() + victim);
      S->evicted++;
    }
    if (S->used + b <= S->o.hbm_budget_bytes) {
      *slot = -1;
      *need = b;
      S->used += b;  // reserved until the solver exists
      const long long id = r.id;
      S->queue.erase(S->queue.begin() + qi);
      return id;
    }
    if (qi == 0 && S->o.fifo) break;  // strict order: wait for room for the head
  }
  return 0;
}

static void worker(fishgpu_server_s *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  while (true) {
    int slot = -1;
    long long need = 0, id = 0;
    S->cv_work.wait(lk, [&] { return S->stop || (!S->queue.empty() && (id = pick(S, &slot, &need)) != 0); });
    if (S->stop && id == 0) return;
    Req &r = S->reqs[id];
    r.status = -2;
    r.t_start = clk::now();
    const int dim = r.dim, n = r.n;
    const double *f = r.f;
    double *u = r.u;
    fishgpu_solver *sol = nullptr;
    if (slot >= 0) {
      S->pool[slot].busy = true;
      sol = S->pool[slot].s;
    }
    lk.unlock();
    int rc = FISHGPU_OK;
    if (!sol) {
      fishgpu_opts o;
      make_opts(S->o, dim, n, &o);
      rc = fishgpu_solver_create(&o, nullptr, &sol);
    }
    fishgpu_report rep;
    memset(&rep, 0, sizeof(rep));
    if (!rc) rc = fishgpu_solver_solve_host(sol, f, nullptr, u, &rep);
    lk.lock();
    if (slot < 0) {
      S->used -= need;
      if (sol) {
        S->pool.push_back(Pooled{sol, dim, n, fishgpu_solver_bytes(sol), false, clk::now()});
        S->used += S->pool.back().bytes;
        S->created++;
        slot = (int)S->pool.size() - 1;
      }
    }
    if (slot >= 0) {
      // the pool may have moved: find this solver again
      for (auto &e : S->pool)
        if (e.s == sol) {
          e.busy = false;
          e.last = clk::now();
        }
    }
    Req &rr = S->reqs[id];
    rr.t_end = clk::now();
    rr.status = rc;
    rr.its = rep.its;
    rr.outer = rep.outer_its;
    rr.relres = rep.true_rel_resid;
    S->completed++;
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
  return FISHGPU_OK;
}

extern "C" int fishgpu_server_create(const fishgpu_server_opts *o, fishgpu_server **out) {
  if (!o || !out || o->workers < 1 || o->workers > 256 || o->hbm_budget_bytes <= 0 || !(o->rtol > 0))
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

extern "C" int fishgpu_server_destroy(fishgpu_server *S) {
  if (!S) return FISHGPU_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->queue.clear();
  }
  S->cv_work.notify_all();
  for (auto &t : S->workers) t.join();
  for (auto &e : S->pool) fishgpu_solver_destroy(e.s);
  delete S;
  return FISHGPU_OK;
}
