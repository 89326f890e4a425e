// Serving engine: a request loop for streams of single points.
//
// The reference computes one single point at a time: each
// ClusterAnion::EnergyFromConfiguration call (src/ClusterAnion.cpp:192-290)
// builds the site tables, samples V(r) and diagonalises, and only the next
// call may start; successive points of one stream warm-start from the last
// eigenvectors (istartvec = 0, src/ClusterAnion.cpp:291).  Here:
//   - pg_engine_submit copies a request into a FIFO queue and returns;
//   - `slots` worker threads, each with its own non-blocking stream, solve
//     workspace and buffers (grow-only, so a warm worker does not allocate),
//     take the queue head when the device-memory footprint of the admitted
//     solves plus the head's stays within the budget (head-of-line order:
//     a large request is not starved by smaller ones behind it);
//   - warm start: converged eigenvectors are kept on the device per
//     (key, grid), as many states as any solve of that pair produced; a
//     request starts from the cached vectors (startvec 0), its own start
//     vectors filling any further columns;
//   - matvec batching: mixed-form H*X products of solves in flight on the same
//     grid go to one batcher thread, which merges up to 16 of them into one
//     tensor-core launch per axis (the job table of k_hx_tc).  Ordering between
//     streams is by events only -- the worker records `ready` after the
//     producer of X, the batcher's stream waits on all of them, launches, and
//     records each worker's `done`, which the worker's stream waits on -- so no
//     host synchronisation enters the product.  The batcher launches when every
//     solve in flight on that grid has a product waiting, or when the oldest
//     one has waited batch_window_us.
// Every column of a merged launch is computed exactly as in a launch of its
// own (tiles never mix columns of two solves), so a solve's result does not
// depend on its partners.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "pg_solve.cuh"

namespace {

using Clock = std::chrono::steady_clock;

double seconds_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

struct GridKey {
  int n[3];
  double L[3];
  bool operator<(const GridKey& o) const {
    return std::tie(n[0], n[1], n[2], L[0], L[1], L[2]) < std::tie(o.n[0], o.n[1], o.n[2], o.L[0], o.L[1], o.L[2]);
  }
};

struct Job {
  long id = 0;
  pg_request r{};
  std::vector<double> waters, ions;  // owned copies of the request's host data
  double footprint = 0;
  Clock::time_point t_submit;
};

// One H*X product waiting for the batcher.
struct Ticket {
  const pg_grid* g;
  const double* v;
  const double* x;
  double* y;
  int nvec;
  cudaEvent_t ready, done;
  Clock::time_point t;
  pg_status status = PG_OK;
  std::string err;
  bool finished = false;
};

struct CacheEntry {
  pg::DevBuf<double> vecs;
  int nroots = 0;
};

}  // namespace

struct pg_engine {
  pg_engine_config cfg{};
  int device = 0;
  double budget = 0;

  // queue, admission and results
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<std::unique_ptr<Job>> queue;
  std::map<long, pg_result> done;
  std::deque<long> done_order;
  std::set<long> outstanding;  // submitted, result not yet handed over
  long next_id = 1;
  // device bytes counted against the budget: per worker, the larger of what
  // it keeps between solves and the footprint of the solve it runs (held),
  // plus the warm-start cache (cache_bytes, under cm)
  std::vector<double> held;
  double in_use = 0;  // sum of held
  double cache_bytes = 0;
  int in_flight = 0;
  bool stopping = false;
  pg_engine_stats stats{};
  std::vector<std::thread> workers;

  // batcher
  std::mutex bm;
  std::condition_variable bcv, tcv;
  std::deque<Ticket*> pending;
  std::map<const pg_grid*, int> active;  // solves in flight per grid
  bool bstop = false;
  std::thread batcher;

  // grids and warm-start vectors shared by the workers
  std::mutex gm;
  std::map<GridKey, pg_grid*> grids;
  std::mutex cm;
  std::map<std::pair<long, GridKey>, std::unique_ptr<CacheEntry>> cache;

  pg_status grid_for(const pg_request& r, pg_grid** out);
  double cached() {
    std::lock_guard<std::mutex> l(cm);
    return cache_bytes;
  }
  void worker_main(int slot);
  void batcher_main();
  pg_status batched_hx(const pg_grid* g, const double* v, const double* x, double* y, int nvec, cudaStream_t st,
                       cudaEvent_t ready, cudaEvent_t done);
  void run_job(Job& job, cudaStream_t st, pg::SolveWorkspace* ws, pg::DevBuf<double>& v, pg::DevBuf<double>& evecs,
               cudaEvent_t ready, cudaEvent_t done_ev, pg_result& res);
};

extern "C" double pg_request_footprint(const pg_request* r) {
  if (!r) return 0;
  const double N = (double)r->n[0] * r->n[1] * r->n[2];
  const double ms = r->params.maxsub, nr = r->params.nroots;
  const double work = r->params.corrflag == 2 ? 2 * nr + 1 : 2 * nr;  // pg_davidson_work_size
  const double pc = r->params.corrflag == 3 ? 7 * nr : 0;            // preconditioner blocks (2 x 2nr work, 3nr)
  const double twins = r->params.precision == PG_MIXED ? 2 * ms : 0;  // double-float twins of the basis and products
  // basis + products, work array, diagonal, potential, eigenvectors
  return 8.0 * (N * (2 * ms + twins + work + 1 + 1 + nr + pc) + 2 * ms * ms + 11 * ms);
}

pg_status pg_engine::grid_for(const pg_request& r, pg_grid** out) {
  GridKey k;
  for (int a = 0; a < 3; ++a) {
    k.n[a] = r.n[a];
    k.L[a] = r.L[a];
  }
  std::lock_guard<std::mutex> l(gm);
  auto it = grids.find(k);
  if (it != grids.end()) {
    *out = it->second;
    return PG_OK;
  }
  pg_grid* g = nullptr;
  PG_TRY(pg_grid_create(r.n, r.L, &g));
  grids[k] = g;
  *out = g;
  return PG_OK;
}

pg_status pg_engine::batched_hx(const pg_grid* g, const double* v, const double* x, double* y, int nvec,
                                cudaStream_t st, cudaEvent_t ready, cudaEvent_t done_ev) {
  Ticket t{g, v, x, y, nvec, ready, done_ev, Clock::now()};
  PG_CUDA_TRY(cudaEventRecord(ready, st));
  {
    std::unique_lock<std::mutex> l(bm);
    pending.push_back(&t);
    bcv.notify_all();
    tcv.wait(l, [&] { return t.finished; });
  }
  if (t.status != PG_OK) {
    pg::set_error("%s", t.err.c_str());
    return t.status;
  }
  PG_CUDA_TRY(cudaStreamWaitEvent(st, done_ev, 0));
  return PG_OK;
}

void pg_engine::batcher_main() {
  cudaSetDevice(device);
  cudaStream_t bs = nullptr;
  const cudaError_t se = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
  const auto window = std::chrono::microseconds(std::max(0, cfg.batch_window_us));
  std::unique_lock<std::mutex> l(bm);
  for (;;) {
    if (pending.empty()) {
      if (bstop) break;
      bcv.wait(l);
      continue;
    }
    Ticket* head = pending.front();
    const pg_grid* g = head->g;
    int have = 0;
    for (Ticket* t : pending) have += t->g == g;
    const int want = std::min(active.count(g) ? active[g] : 1, pg::kMaxBatchJobs);
    const auto deadline = head->t + window;
    if (have < want && Clock::now() < deadline) {
      bcv.wait_until(l, deadline);
      continue;
    }
    std::vector<Ticket*> b;
    for (auto it = pending.begin(); it != pending.end() && (int)b.size() < pg::kMaxBatchJobs;) {
      if ((*it)->g == g) {
        b.push_back(*it);
        it = pending.erase(it);
      } else {
        ++it;
      }
    }
    l.unlock();
    const int nj = (int)b.size();
    std::vector<const double*> vs(nj), xs(nj);
    std::vector<double*> ys(nj);
    std::vector<int> nv(nj);
    pg_status s = PG_OK;
    std::string err;
    if (se != cudaSuccess) {
      s = PG_CUDA;
      err = std::string("batcher stream: ") + cudaGetErrorString(se);
    }
    for (int j = 0; j < nj && s == PG_OK; ++j) {
      vs[j] = b[j]->v;
      xs[j] = b[j]->x;
      ys[j] = b[j]->y;
      nv[j] = b[j]->nvec;
      const cudaError_t e = cudaStreamWaitEvent(bs, b[j]->ready, 0);
      if (e != cudaSuccess) {
        s = PG_CUDA;
        err = std::string("batcher wait: ") + cudaGetErrorString(e);
      }
    }
    if (s == PG_OK) {
      s = pg::hx_mixed_batch(g, vs.data(), xs.data(), ys.data(), nv.data(), nj, bs, true);
      if (s != PG_OK) err = pg::last_error();
    }
    // record every done event, also after a failure, so no stream waits on a stale one
    for (int j = 0; j < nj; ++j) {
      const cudaError_t e = cudaEventRecord(b[j]->done, bs);
      if (e != cudaSuccess && s == PG_OK) {
        s = PG_CUDA;
        err = std::string("batcher record: ") + cudaGetErrorString(e);
      }
    }
    {
      std::lock_guard<std::mutex> sl(m);
      stats.batches += 1;
      stats.batched_products += nj;
    }
    l.lock();
    for (Ticket* t : b) {
      t->status = s;
      t->err = err;
      t->finished = true;
    }
    tcv.notify_all();
  }
  l.unlock();
  if (bs) cudaStreamDestroy(bs);
}

void pg_engine::run_job(Job& job, cudaStream_t st, pg::SolveWorkspace* ws, pg::DevBuf<double>& v,
                        pg::DevBuf<double>& evecs, cudaEvent_t ready, cudaEvent_t done_ev, pg_result& res) {
  const pg_request& r = job.r;
  pg_solve_params p = r.params;
  res.nroots = p.nroots;
  auto fail = [&](pg_status s) {
    res.status = s;
    snprintf(res.error, sizeof(res.error), "%s", pg::last_error());
  };
  pg_grid* g = nullptr;
  pg_status s = grid_for(r, &g);
  if (s != PG_OK) return fail(s);
  const long N = g->N;
  if ((s = v.ensure(N)) != PG_OK || (s = evecs.ensure((size_t)N * p.nroots)) != PG_OK) return fail(s);
  s = pg::cluster_potential(g, r.nw, job.waters.data(), r.nions, job.ions.data(), v.p, st);
  if (s != PG_OK) return fail(s);

  GridKey gk;
  for (int a = 0; a < 3; ++a) {
    gk.n[a] = r.n[a];
    gk.L[a] = r.L[a];
  }
  const bool use_cache = cfg.warm_start && r.key >= 0;
  if (use_cache) {
    std::lock_guard<std::mutex> l(cm);
    auto it = cache.find({r.key, gk});
    if (it != cache.end() && it->second->nroots > 0) {
      const int k = std::min(it->second->nroots, p.nroots);
      // fewer cached vectors than states: the request's own start vectors
      // fill the columns the cache does not cover
      if (k < p.nroots && (s = pg::start_vectors(g, p.nroots, p.startvec, evecs.p, st)) != PG_OK) return fail(s);
      // copy under the lock and wait for it: the entry may be rewritten next
      if (cudaMemcpyAsync(evecs.p, it->second->vecs.p, sizeof(double) * N * k, cudaMemcpyDeviceToDevice, st) !=
              cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) {
        pg::set_error("warm-start copy failed: %s", cudaGetErrorString(cudaGetLastError()));
        return fail(PG_CUDA);
      }
      p.startvec = 0;
      res.warm_started = 1;
    }
  }

  const bool batch = cfg.batch_matvecs && p.precision == PG_MIXED;
  {
    std::lock_guard<std::mutex> l(bm);
    active[g] += 1;
  }
  s = pg::solve_with(
      g, v.p, &p, res.evals, evecs.p, &res.stats, st,
      [&](const double* x, double* y, int nvec) {
        if (batch) return batched_hx(g, v.p, x, y, nvec, st, ready, done_ev);
        return pg::hx(g, v.p, x, y, nvec, p.precision, st, true);
      },
      ws);
  {
    std::lock_guard<std::mutex> l(bm);
    if (--active[g] == 0) active.erase(g);
    bcv.notify_all();
  }
  if (s != PG_OK) {
    fail(s);
    if (s != PG_NOT_CONVERGED) return;
  }
  if (s == PG_OK && use_cache) {
    // keep the most states any solve of this key and grid produced: a solve
    // with fewer states refreshes the leading vectors only
    std::lock_guard<std::mutex> l(cm);
    auto& e = cache[{r.key, gk}];
    if (!e) e.reset(new CacheEntry());
    const int keep = std::max(e->nroots, p.nroots);
    pg_status cs = PG_OK;
    if (e->vecs.n < (size_t)N * keep) {
      pg::DevBuf<double> grown;
      cs = grown.alloc((size_t)N * keep);
      if (cs == PG_OK && e->nroots > 0 &&
          cudaMemcpyAsync(grown.p, e->vecs.p, sizeof(double) * N * e->nroots, cudaMemcpyDeviceToDevice, st) !=
              cudaSuccess)
        cs = PG_CUDA;
      if (cs == PG_OK) {
        cache_bytes += 8.0 * ((double)grown.n - (double)e->vecs.n);
        std::swap(grown.p, e->vecs.p), std::swap(grown.n, e->vecs.n);
      }
      if (cs == PG_OK && cudaStreamSynchronize(st) != cudaSuccess) cs = PG_CUDA;  // before `grown` frees the old one
    }
    if (cs == PG_OK &&
        (cudaMemcpyAsync(e->vecs.p, evecs.p, sizeof(double) * N * p.nroots, cudaMemcpyDeviceToDevice, st) !=
             cudaSuccess ||
         cudaStreamSynchronize(st) != cudaSuccess))
      cs = PG_CUDA;
    if (cs != PG_OK) {
      if (cs == PG_CUDA) pg::set_error("warm-start store failed: %s", cudaGetErrorString(cudaGetLastError()));
      cache_bytes -= 8.0 * (double)e->vecs.n;
      cache.erase({r.key, gk});
      return fail(cs);
    }
    e->nroots = keep;
  }
  if (r.evecs_host) {
    if (cudaMemcpyAsync(r.evecs_host, evecs.p, sizeof(double) * N * p.nroots, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      pg::set_error("eigenvector copy failed: %s", cudaGetErrorString(cudaGetLastError()));
      return fail(PG_CUDA);
    }
  }
}

void pg_engine::worker_main(int slot) {
  cudaSetDevice(device);
  cudaStream_t st = nullptr;
  cudaEvent_t ready = nullptr, done_ev = nullptr;
  cudaError_t init = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (init == cudaSuccess) init = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
  if (init == cudaSuccess) init = cudaEventCreateWithFlags(&done_ev, cudaEventDisableTiming);
  pg::SolveWorkspace* ws = pg::workspace_create();
  {
    pg::DevBuf<double> v, evecs;
    for (;;) {
      std::unique_ptr<Job> job;
      {
        std::unique_lock<std::mutex> l(m);
        // the head runs on this worker's retained buffers (grown to its
        // footprint): admitted when the budget holds with this worker's share
        // at max(held, footprint); with nothing in flight it runs regardless
        cv_work.wait(l, [&] {
          if (stopping) return true;
          if (queue.empty()) return false;
          const double f = queue.front()->footprint;
          return in_flight == 0 || in_use - held[slot] + std::max(held[slot], f) + cached() <= budget;
        });
        if (stopping) break;
        job = std::move(queue.front());
        queue.pop_front();
        const double h = std::max(held[slot], job->footprint);
        in_use += h - held[slot];
        held[slot] = h;
        in_flight += 1;
        stats.peak_in_flight = std::max(stats.peak_in_flight, in_flight);
        stats.peak_bytes = std::max(stats.peak_bytes, in_use + cached());
      }
      const auto t_start = Clock::now();
      pg_result res;
      memset(&res, 0, sizeof(res));
      res.id = job->id;
      res.status = PG_OK;
      if (init != cudaSuccess) {
        res.status = PG_CUDA;
        snprintf(res.error, sizeof(res.error), "worker stream/event creation failed: %s",
                 cudaGetErrorString(init));
      } else {
        run_job(*job, st, ws, v, evecs, ready, done_ev, res);
      }
      const auto t_end = Clock::now();
      res.queue_seconds = seconds_between(job->t_submit, t_start);
      res.latency_seconds = seconds_between(job->t_submit, t_end);
      // what this worker keeps for its next solve; beyond its share of the
      // budget the buffers are released, so that idle workers cannot hold
      // memory an admitted solve needs
      double keep = pg::workspace_bytes(ws) + 8.0 * (double)(v.n + evecs.n);
      if (keep > budget / (double)cfg.slots) {
        pg::workspace_destroy(ws);
        ws = pg::workspace_create();
        v.release();
        evecs.release();
        keep = 0;
      }
      {
        std::lock_guard<std::mutex> l(m);
        in_use += keep - held[slot];
        held[slot] = keep;
        in_flight -= 1;
        stats.completed += 1;
        if (res.status != PG_OK) stats.failed += 1;
        if (res.warm_started) stats.warm_starts += 1;
        done[res.id] = res;
        done_order.push_back(res.id);
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }
  pg::workspace_destroy(ws);
  if (ready) cudaEventDestroy(ready);
  if (done_ev) cudaEventDestroy(done_ev);
  if (st) cudaStreamDestroy(st);
}

namespace {

bool finite_all(const double* a, long n) {
  for (long i = 0; i < n; ++i)
    if (!std::isfinite(a[i])) return false;
  return true;
}

}  // namespace

extern "C" pg_status pg_engine_create(const pg_engine_config* c, pg_engine** out) {
  PG_ARG(out, "pg_engine_create: null argument");
  *out = nullptr;
  pg_engine_config cfg{};
  cfg.device = -1;
  cfg.slots = 8;
  cfg.memory_budget = 0;
  cfg.batch_matvecs = 1;
  cfg.batch_window_us = 200;
  cfg.warm_start = 1;
  if (c) cfg = *c;
  PG_ARG(cfg.slots > 0 && cfg.slots <= 256, "pg_engine_create: slots must be in 1..256 (got %d)", cfg.slots);
  PG_ARG(cfg.batch_window_us >= 0, "pg_engine_create: negative batch window");
  int dev = cfg.device;
  if (dev < 0) PG_CUDA_TRY(cudaGetDevice(&dev));
  PG_CUDA_TRY(cudaSetDevice(dev));
  double budget = cfg.memory_budget;
  if (budget <= 0) {
    size_t fr = 0, tot = 0;
    PG_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
    budget = 0.8 * (double)fr;
  }
  std::unique_ptr<pg_engine> e(new pg_engine());
  e->cfg = cfg;
  e->device = dev;
  e->budget = budget;
  e->held.assign((size_t)cfg.slots, 0.0);
  try {
    e->batcher = std::thread(&pg_engine::batcher_main, e.get());
    for (int i = 0; i < cfg.slots; ++i) e->workers.emplace_back(&pg_engine::worker_main, e.get(), i);
  } catch (const std::exception& ex) {
    pg::set_error("pg_engine_create: thread start failed: %s", ex.what());
    {
      std::lock_guard<std::mutex> l(e->m);
      e->stopping = true;
    }
    e->cv_work.notify_all();
    for (auto& t : e->workers) t.join();
    {
      std::lock_guard<std::mutex> l(e->bm);
      e->bstop = true;
    }
    e->bcv.notify_all();
    if (e->batcher.joinable()) e->batcher.join();
    return PG_UNSUPPORTED;
  }
  *out = e.release();
  return PG_OK;
}

extern "C" pg_status pg_engine_submit(pg_engine* e, const pg_request* r, long* id) {
  PG_ARG(e && r && id, "pg_engine_submit: null argument");
  const pg_solve_params& p = r->params;
  for (int a = 0; a < 3; ++a) {
    PG_ARG(r->n[a] >= 2 && r->n[a] <= 4096, "pg_engine_submit: grid size %d out of range", r->n[a]);
    PG_ARG(std::isfinite(r->L[a]) && r->L[a] > 0, "pg_engine_submit: box length must be finite and positive");
  }
  PG_ARG(r->nw >= 0 && r->nions >= 0, "pg_engine_submit: negative site count");
  PG_ARG(r->nw == 0 || r->waters, "pg_engine_submit: null water coordinates");
  PG_ARG(r->nions == 0 || r->ions, "pg_engine_submit: null ion list");
  PG_ARG(r->nw == 0 || finite_all(r->waters, 9L * r->nw), "pg_engine_submit: non-finite water coordinate");
  PG_ARG(r->nions == 0 || finite_all(r->ions, 4L * r->nions), "pg_engine_submit: non-finite ion entry");
  PG_ARG(p.nroots > 0 && p.nroots <= 16 && p.maxsub > p.nroots && p.maxsub <= 128 && p.maxiter > 0 && p.ptol > 0,
         "pg_engine_submit: bad solve parameters (nroots %d, maxsub %d, maxiter %d, ptol %d)", p.nroots, p.maxsub,
         p.maxiter, p.ptol);
  PG_ARG(p.precision == PG_FP64 || p.precision == PG_MIXED, "pg_engine_submit: unknown precision");
  PG_ARG(p.startvec == 1 || p.startvec == 2, "pg_engine_submit: startvec must be 1 or 2 (warm start is the engine's)");
  if (p.precision == PG_MIXED)
    for (int a = 0; a < 3; ++a)
      if (r->n[a] > 256) {
        pg::set_error("pg_engine_submit: the mixed form supports n <= 256 per axis (got %d)", r->n[a]);
        return PG_UNSUPPORTED;
      }
  std::unique_ptr<Job> job(new Job());
  job->r = *r;
  job->waters.assign(r->waters ? r->waters : nullptr, r->waters ? r->waters + 9L * r->nw : nullptr);
  job->ions.assign(r->ions ? r->ions : nullptr, r->ions ? r->ions + 4L * r->nions : nullptr);
  job->r.waters = nullptr;
  job->r.ions = nullptr;
  job->footprint = pg_request_footprint(r);
  job->t_submit = Clock::now();
  std::lock_guard<std::mutex> l(e->m);
  if (job->footprint > e->budget) {
    pg::set_error("pg_engine_submit: request needs %.0f bytes, above the engine's budget of %.0f",
                  job->footprint, e->budget);
    return PG_OOM;
  }
  PG_ARG(!e->stopping, "pg_engine_submit: engine is shutting down");
  job->id = e->next_id++;
  *id = job->id;
  e->outstanding.insert(job->id);
  e->stats.submitted += 1;
  e->queue.push_back(std::move(job));
  e->cv_work.notify_all();
  return PG_OK;
}

extern "C" pg_status pg_engine_wait(pg_engine* e, long id, pg_result* out, double timeout_s) {
  PG_ARG(e && out, "pg_engine_wait: null argument");
  std::unique_lock<std::mutex> l(e->m);
  PG_ARG(e->outstanding.count(id), "pg_engine_wait: no outstanding request %ld", id);
  auto ready = [&] { return e->done.count(id) > 0; };
  if (timeout_s < 0) {
    e->cv_done.wait(l, ready);
  } else if (!e->cv_done.wait_for(l, std::chrono::duration<double>(timeout_s), ready)) {
    pg::set_error("pg_engine_wait: request %ld not done within %.3f s", id, timeout_s);
    return PG_DEVICE_TIMEOUT;
  }
  *out = e->done[id];
  e->done.erase(id);
  e->outstanding.erase(id);
  return PG_OK;
}

extern "C" pg_status pg_engine_poll(pg_engine* e, pg_result* out, int max, int* nout) {
  PG_ARG(e && nout && (max <= 0 || out), "pg_engine_poll: null argument");
  std::lock_guard<std::mutex> l(e->m);
  int k = 0;
  while (k < max && !e->done_order.empty()) {
    const long id = e->done_order.front();
    e->done_order.pop_front();
    auto it = e->done.find(id);
    if (it == e->done.end()) continue;  // already handed over by pg_engine_wait
    out[k++] = it->second;
    e->done.erase(it);
    e->outstanding.erase(id);
  }
  *nout = k;
  return PG_OK;
}

extern "C" pg_status pg_engine_get_stats(pg_engine* e, pg_engine_stats* out) {
  PG_ARG(e && out, "pg_engine_get_stats: null argument");
  std::lock_guard<std::mutex> l(e->m);
  *out = e->stats;
  return PG_OK;
}

extern "C" pg_status pg_engine_destroy(pg_engine* e) {
  if (!e) return PG_OK;
  {
    std::lock_guard<std::mutex> l(e->m);
    e->stopping = true;
    e->queue.clear();  // queued requests never start
  }
  e->cv_work.notify_all();
  for (auto& t : e->workers) t.join();
  {
    std::lock_guard<std::mutex> l(e->bm);
    e->bstop = true;
  }
  e->bcv.notify_all();
  if (e->batcher.joinable()) e->batcher.join();
  e->cache.clear();
  for (auto& kv : e->grids) pg_grid_destroy(kv.second);
  delete e;
  return PG_OK;
}
