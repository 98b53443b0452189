// ensemble.cu -- many independent droplet simulations stepped together on one
// GPU (no reference counterpart: main.f runs one case per process).
//
// Each member is a full context (its own fields, multigrid hierarchy, CUDA
// graphs and stream).  A step of the ensemble is one time step of every
// member.  The members' host-side control (the CFL and residual reads inside a
// step) would serialise them on one host thread, so a pool of worker threads
// steps them: worker w owns a fixed subset of members and steps them one
// after the other on their own streams, while the other workers' members run
// on the GPU at the same time.  Members are spread over the workers by
// longest-processing-time-first on a cost per member: a model
// (launch-bound floor + cells) until the autotuner has measured each
// member's step time, then the measurement.  The autotuner also picks the
// number of workers by timing real steps.
//
// Workers take members only between steps, so a failing member (its step
// returns an error code) never leaves kernels of its own in flight while the
// others continue; the ensemble step reports the first failing member.
//
// Batched mode (dsg_ensemble_set_batched): the members form cost-balanced
// groups, and a worker steps whole groups: every member of the group up to
// its pressure solve, the group's pressure solves as one batched solve
// (batch.cu: one launch per multigrid pass over all members of the group,
// under CUDA graphs, on the group's own stream), then every member after its
// solve.  The groups of different workers overlap on the GPU.  Each member's
// results are bit for bit those of its own step.  A member that fails before
// its solve stops the other members of its group before their solves; the
// step reports the first failing member.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "dsg_internal.cuh"

struct dsg_ensemble {
  std::vector<dsg_ctx *> m;
  std::vector<double> cost;       // per-member cost used by the plan
  std::vector<double> member_ms;  // last measured host time of each member's step
  std::vector<int> rc;
  std::vector<dsg_mg_stats> st;
  std::vector<std::vector<int>> plan;  // members of each worker
  std::vector<std::thread> th;
  std::mutex mu;
  std::condition_variable go, done;
  long long gen = 0;  // step generation the workers wait for
  int busy = 0;       // workers still stepping the current generation
  bool stop = false;
  int t = 0;
  int workers = 0;
  int phase = 0;  // what the workers run: 0 whole member steps, 3 whole group steps (batched mode)
  double last_ms = 0.0;
  double phase_ms[3] = {0.0, 0.0, 0.0};  // batched mode: worker time of the last step's phases, summed
  std::string err;
  // batched mode: the members split into groups, each group's pressure solves
  // one batched solve on its own stream
  std::vector<dsg::BatchSolve *> batch;
  std::vector<std::vector<int>> group;  // members of each group
  std::vector<int> group_rc;            // status of each group's batched solve
  std::vector<dsg_mg_stats> ms;         // per member: statistics and status of its solve
  std::vector<int> mg_rc;
  std::vector<int> reached;             // per member: 1 once its step reached the solve
};

namespace {

using Clock = std::chrono::steady_clock;

// Cost model before any measurement: a member's step is launch-bound below a
// few million cells (about 2e6 cells' worth of bandwidth time per step is
// launch latency on this path), bandwidth-bound above.
double model_cost(const dsg_ctx *c) { return (double)(c->nx - 2) * (c->ny - 2) * (c->nz - 2) + 2.0e6; }

// A worker starts at generation gen0 (the ensemble's generation when the pool
// was built): it steps only for generations announced after that.
void worker_main(dsg_ensemble *e, int w, long long gen0) {
  long long seen = gen0;
  for (;;) {
    std::vector<int> mine;
    int t, phase, workers;
    {
      std::unique_lock<std::mutex> lk(e->mu);
      e->go.wait(lk, [&] { return e->stop || e->gen != seen; });
      if (e->stop) return;
      seen = e->gen;
      mine = e->plan[w];
      t = e->t;
      phase = e->phase;
      workers = e->workers;
    }
    if (phase == 3) {
      // batched mode: worker w takes groups w, w + workers, ... through the
      // whole step (its members up to their solves, the group's batched
      // solve, its members after their solves), so the groups of different
      // workers overlap on the GPU like single members do
      double pm[3] = {0.0, 0.0, 0.0};
      for (size_t g = (size_t)w; g < e->batch.size(); g += (size_t)workers) {
        const std::vector<int> &mem = e->group[g];
        const auto t0 = Clock::now();
        bool all = true;
        for (int i : mem) {
          dsg_ctx *c = e->m[i];
          cudaError_t ce = cudaSetDevice(c->device);
          e->rc[i] = ce == cudaSuccess ? dsg::step_pre_solve(c, t) : dsg::cuda_fail(c, ce, "cudaSetDevice");
          e->reached[i] = e->rc[i] == DSG_OK;
          all = all && e->reached[i];
        }
        const auto t1 = Clock::now();
        e->group_rc[g] = DSG_OK;
        if (all) {
          std::vector<int> act(mem.size(), 1), rc(mem.size());
          std::vector<dsg_mg_stats> st(mem.size());
          e->group_rc[g] = dsg::batch_solve(e->batch[g], act, st, rc);
          if (e->group_rc[g]) e->m[mem[0]]->err = dsg_last_error(nullptr);
          for (size_t q = 0; q < mem.size(); q++) {
            e->ms[mem[q]] = st[q];
            e->mg_rc[mem[q]] = rc[q];
          }
        }
        const auto t2 = Clock::now();
        if (all && !e->group_rc[g])
          for (int i : mem) {
            const int mrc = e->mg_rc[i];
            if (mrc && mrc != DSG_E_NOT_CONVERGED) {
              e->rc[i] = mrc;
              continue;
            }
            e->rc[i] = dsg::step_post_solve(e->m[i], t, &e->ms[i], mrc, &e->st[i]);
          }
        const auto t3 = Clock::now();
        pm[0] += std::chrono::duration<double, std::milli>(t1 - t0).count();
        pm[1] += std::chrono::duration<double, std::milli>(t2 - t1).count();
        pm[2] += std::chrono::duration<double, std::milli>(t3 - t2).count();
        const double per = std::chrono::duration<double, std::milli>(t3 - t0).count() / (double)mem.size();
        for (int i : mem) e->member_ms[i] = per;
      }
      {
        std::lock_guard<std::mutex> lk(e->mu);
        for (int q = 0; q < 3; q++) e->phase_ms[q] += pm[q];
      }
      mine.clear();
    }
    for (int i : mine) {
      dsg_ctx *c = e->m[i];
      const auto t0 = Clock::now();
      cudaError_t ce = cudaSetDevice(c->device);
      if (ce != cudaSuccess) {
        e->rc[i] = dsg::cuda_fail(c, ce, "cudaSetDevice");
      } else {
        e->rc[i] = dsg_step(c, t, &e->st[i]);
      }
      e->member_ms[i] = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
    }
    std::lock_guard<std::mutex> lk(e->mu);
    if (--e->busy == 0) e->done.notify_all();
  }
}

void release_batches(dsg_ensemble *e) {
  for (dsg::BatchSolve *b : e->batch) dsg::batch_destroy(b);
  e->batch.clear();
  e->group.clear();
  e->group_rc.clear();
}

void stop_workers(dsg_ensemble *e) {
  {
    std::lock_guard<std::mutex> lk(e->mu);
    e->stop = true;
  }
  e->go.notify_all();
  for (std::thread &t : e->th) t.join();
  e->th.clear();
  e->stop = false;
}

}  // namespace

extern "C" {

int dsg_ensemble_plan(const double *cost, int n, int workers, int *assign) {
  if (!cost || !assign || n < 0 || workers < 1) return dsg::set_error(nullptr, DSG_E_ARG, "bad plan arguments");
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<double> load(workers, 0.0);
  for (int i : order) {
    int best = 0;
    for (int w = 1; w < workers; w++)
      if (load[w] < load[best]) best = w;
    assign[i] = best;
    load[best] += cost[i];
  }
  return DSG_OK;
}

int dsg_ensemble_set_workers(dsg_ensemble *e, int workers) {
  if (!e) return dsg::set_error(nullptr, DSG_E_ARG, "null ensemble");
  const int n = (int)e->m.size();
  if (workers <= 0) {
    const unsigned hw = std::thread::hardware_concurrency();
    workers = (int)(hw ? hw : 8);
  }
  workers = std::max(1, std::min(workers, n));
  stop_workers(e);
  std::vector<int> assign(n);
  int rc = dsg_ensemble_plan(e->cost.data(), n, workers, assign.data());
  if (rc) return rc;
  e->plan.assign(workers, {});
  for (int i = 0; i < n; i++) e->plan[assign[i]].push_back(i);
  for (auto &p : e->plan)  // within a worker the costliest member first
    std::stable_sort(p.begin(), p.end(), [&](int a, int b) { return e->cost[a] > e->cost[b]; });
  e->workers = workers;
  e->busy = 0;
  try {
    for (int w = 0; w < workers; w++) e->th.emplace_back(worker_main, e, w, e->gen);
  } catch (...) {
    stop_workers(e);
    e->workers = 0;
    return dsg::set_error(nullptr, DSG_E_NOMEM, "cannot start %d worker threads", workers);
  }
  return DSG_OK;
}

int dsg_ensemble_create(const dsg_config *cfgs, int n, int workers, dsg_ensemble **out) {
  if (!cfgs || n <= 0 || !out) return dsg::set_error(nullptr, DSG_E_ARG, "bad ensemble arguments");
  *out = nullptr;
  dsg_ensemble *e = new dsg_ensemble();
  for (int i = 0; i < n; i++) {
    dsg_ctx *c = nullptr;
    int rc = dsg_create(&cfgs[i], &c);
    if (!rc) rc = dsg_init_drop(c);
    if (rc) {
      std::string msg = std::string("member ") + std::to_string(i) + ": " + dsg_last_error(c);
      if (c) dsg_destroy(c);
      for (dsg_ctx *x : e->m) dsg_destroy(x);
      delete e;
      return dsg::set_error(nullptr, rc, "%s", msg.c_str());
    }
    e->m.push_back(c);
    e->cost.push_back(model_cost(c));
  }
  e->member_ms.assign(n, 0.0);
  e->rc.assign(n, 0);
  e->st.assign(n, dsg_mg_stats{});
  int rc = dsg_ensemble_set_workers(e, workers);
  if (rc) {
    for (dsg_ctx *x : e->m) dsg_destroy(x);
    delete e;
    return rc;
  }
  *out = e;
  return DSG_OK;
}

void dsg_ensemble_destroy(dsg_ensemble *e) {
  if (!e) return;
  stop_workers(e);
  release_batches(e);
  for (dsg_ctx *c : e->m) dsg_destroy(c);
  delete e;
}

int dsg_ensemble_size(const dsg_ensemble *e) { return e ? (int)e->m.size() : 0; }

int dsg_ensemble_workers(const dsg_ensemble *e) { return e ? e->workers : 0; }

dsg_ctx *dsg_ensemble_member(dsg_ensemble *e, int i) {
  return (e && i >= 0 && i < (int)e->m.size()) ? e->m[i] : nullptr;
}

const char *dsg_ensemble_last_error(const dsg_ensemble *e) { return e ? e->err.c_str() : ""; }

namespace {

// Run `phase` of step t through the worker pool.
void run_phase(dsg_ensemble *e, int t, int phase) {
  {
    std::lock_guard<std::mutex> lk(e->mu);
    e->t = t;
    e->phase = phase;
    e->busy = e->workers;
    e->gen++;
  }
  e->go.notify_all();
  std::unique_lock<std::mutex> lk(e->mu);
  e->done.wait(lk, [&] { return e->busy == 0; });
}

}  // namespace

int dsg_ensemble_step(dsg_ensemble *e, int t, dsg_mg_stats *stats) {
  if (!e || e->workers < 1) return dsg::set_error(nullptr, DSG_E_ARG, "ensemble without workers");
  const auto t0 = Clock::now();
  const int n = (int)e->m.size();
  if (e->batch.empty()) {
    run_phase(e, t, 0);
  } else {
    for (int q = 0; q < 3; q++) e->phase_ms[q] = 0.0;
    run_phase(e, t, 3);
    for (size_t g = 0; g < e->batch.size(); g++)
      if (e->group_rc[g]) {
        e->err = std::string("batched solve: ") + e->m[e->group[g][0]]->err;
        return e->group_rc[g];
      }
  }
  e->last_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
  if (stats)
    for (int i = 0; i < n; i++) stats[i] = e->st[i];
  for (int i = 0; i < n; i++)
    if (e->rc[i]) {
      e->err = std::string("member ") + std::to_string(i) + ": " + e->m[i]->err;
      return e->rc[i];
    }
  e->err.clear();
  return DSG_OK;
}

int dsg_ensemble_set_batched(dsg_ensemble *e, int groups) {
  if (!e) return dsg::set_error(nullptr, DSG_E_ARG, "null ensemble");
  const int n = (int)e->m.size();
  if (groups <= 0) {
    release_batches(e);
    return DSG_OK;
  }
  if (groups > n) groups = n;
  for (int i = 0; i < n; i++) {
    char why[160];
    if (dsg::batch_eligible(e->m[i], why, sizeof why))
      return dsg::set_error(nullptr, DSG_E_ARG, "member %d cannot be batched: %s", i, why);
  }
  for (int i = 0; i < n; i++) {  // no member work in flight while the batches are set up
    cudaError_t ce = cudaStreamSynchronize(e->m[i]->stream);
    if (ce != cudaSuccess) return dsg::cuda_fail(e->m[i], ce, "dsg_ensemble_set_batched");
  }
  release_batches(e);
  // groups balanced by cost, longest processing time first
  std::vector<int> assign(n);
  int rc = dsg_ensemble_plan(e->cost.data(), n, groups, assign.data());
  if (rc) return rc;
  e->group.assign(groups, {});
  for (int i = 0; i < n; i++) e->group[assign[i]].push_back(i);
  for (int g = 0; g < groups; g++) {
    std::vector<dsg_ctx *> mem;
    for (int i : e->group[g]) mem.push_back(e->m[i]);
    dsg::BatchSolve *b = mem.empty() ? nullptr : dsg::batch_create(mem, &rc);
    if (!b) {
      release_batches(e);
      return rc ? rc : DSG_E_ARG;
    }
    e->batch.push_back(b);
  }
  e->group_rc.assign(groups, 0);
  e->ms.assign(n, dsg_mg_stats{});
  e->mg_rc.assign(n, 0);
  e->reached.assign(n, 0);
  return DSG_OK;
}

int dsg_ensemble_batched(const dsg_ensemble *e) { return e ? (int)e->batch.size() : 0; }

int64_t dsg_ensemble_batch_tail_nodes(const dsg_ensemble *e) {
  return e && !e->batch.empty() ? dsg::batch_tail_nodes(e->batch[0]) : 0;
}

int dsg_ensemble_phase_ms(const dsg_ensemble *e, double *out) {
  if (!e || !out) return DSG_E_ARG;
  for (int q = 0; q < 3; q++) out[q] = e->phase_ms[q];
  return DSG_OK;
}

int dsg_ensemble_autotune_tiles(dsg_ensemble *e, int reps, int *slots_tuned) {
  if (!e || e->batch.empty()) return dsg::set_error(nullptr, DSG_E_STATE, "tile autotuning needs the batched mode");
  if (reps < 1) return dsg::set_error(nullptr, DSG_E_ARG, "reps must be positive");
  for (dsg_ctx *c : e->m) {
    cudaError_t ce = cudaStreamSynchronize(c->stream);
    if (ce != cudaSuccess) return dsg::cuda_fail(c, ce, "dsg_ensemble_autotune_tiles");
  }
  int total = 0;
  for (dsg::BatchSolve *b : e->batch) {
    int k = 0;
    int rc = dsg::batch_autotune(b, reps, &k);
    if (rc) return rc;
    total += k;
  }
  if (slots_tuned) *slots_tuned = total;
  return DSG_OK;
}

double dsg_ensemble_last_ms(const dsg_ensemble *e) { return e ? e->last_ms : 0.0; }

int dsg_ensemble_member_ms(const dsg_ensemble *e, double *out) {
  if (!e || !out) return DSG_E_ARG;
  for (size_t i = 0; i < e->member_ms.size(); i++) out[i] = e->member_ms[i];
  return DSG_OK;
}

int dsg_ensemble_autotune(dsg_ensemble *e, int t0, int steps_per_trial, int *t_next, int *best_workers) {
  if (!e || steps_per_trial < 1) return dsg::set_error(nullptr, DSG_E_ARG, "bad autotune arguments");
  const int n = (int)e->m.size();
  int t = t0;
  // one untimed step: graph capture and first-touch costs
  int rc = dsg_ensemble_step(e, t++, nullptr);
  if (rc) return rc;
  // member costs from their measured step times (one worker: no contention)
  rc = dsg_ensemble_set_workers(e, 1);
  if (rc) return rc;
  rc = dsg_ensemble_step(e, t++, nullptr);
  if (rc) return rc;
  for (int i = 0; i < n; i++) e->cost[i] = e->member_ms[i] > 0.0 ? e->member_ms[i] : e->cost[i];
  const unsigned hw = std::thread::hardware_concurrency();
  const int maxw = std::min(n, std::max(8, 2 * (int)(hw ? hw : 8)));
  std::vector<int> cand;  // 1, 2, 4, ... and maxw itself
  for (int w = 1; w < maxw; w *= 2) cand.push_back(w);
  cand.push_back(maxw);
  double best = 1e300;
  int bw = 1;
  for (int w : cand) {
    rc = dsg_ensemble_set_workers(e, w);
    if (rc) return rc;
    double ms = 0.0;
    for (int s = 0; s < steps_per_trial; s++) {
      rc = dsg_ensemble_step(e, t++, nullptr);
      if (rc) return rc;
      ms += e->last_ms;
    }
    ms /= steps_per_trial;
    if (ms < best) {
      best = ms;
      bw = w;
    }
  }
  rc = dsg_ensemble_set_workers(e, bw);
  if (rc) return rc;
  if (t_next) *t_next = t;
  if (best_workers) *best_workers = bw;
  return DSG_OK;
}

}  // extern "C"
