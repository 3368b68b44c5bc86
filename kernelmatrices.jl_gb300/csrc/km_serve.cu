// Serving form: continuous batching of likelihood, factor and solve requests on one GPU.
//
// A scheduler thread admits queued requests to idle executors whenever the request's device
// bytes (km_estimate_bytes) fit in the HBM budget next to everything that is running or
// resident.  Each executor is a host thread driving its own handle (own stream), so admitted
// requests run concurrently and a new one starts as soon as any executor frees up -- there is
// no batch boundary to wait for.  Factors requested with KM_REQ_FACTOR live in handles of their
// own until released; solves on one factor are serialised, solves on different factors run
// side by side.  Admission is first-come first-served; later requests may pass a head request
// that does not fit yet, until that head has waited kBackfillWindowMs.
//
// The reference has no serving layer (it is a library called in-process); every request runs
// the same handle code path as the single-problem entry points, so a request's results are
// the same whether it runs alone or among others.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/kmhodlr.h"

namespace km {
void set_node_cluster_max(km_handle* h, int v);
}

namespace {

using Clock = std::chrono::steady_clock;
constexpr double kBackfillWindowMs = 100.0;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Job {
  uint64_t ticket = 0;
  km_request req{};
  int64_t need = 0;           // admission estimate (bytes)
  Clock::time_point submitted;
  Clock::time_point started;
};

struct Factor {
  km_handle* h = nullptr;
  int64_t n = 0;
  int64_t bytes = 0;
  bool busy = false;
  bool releasing = false;
};

struct Executor {
  km_handle* h = nullptr;
  std::thread th;
  bool busy = false;
  bool has_job = false;
  Job job;
  int64_t held = 0;           // bytes the handle holds while idle
  int64_t reserve = 0;        // bytes reserved while running
};

}  // namespace

struct km_server {
  km_config cfg{};
  km_serve_opts o{};
  int64_t budget = 0;
  std::mutex mu;
  std::condition_variable cv_sched, cv_exec, cv_done;
  std::deque<Job> queue;
  std::vector<std::unique_ptr<Executor>> ex;
  std::unordered_map<int64_t, std::unique_ptr<Factor>> factors;
  int64_t next_factor = 1;
  int64_t resident = 0;
  uint64_t next_ticket = 1;
  std::unordered_map<uint64_t, km_result> done;
  std::unordered_map<uint64_t, bool> pending;  // submitted, not yet collected
  std::vector<double> latency;
  int64_t submitted = 0, completed = 0, failed = 0, rejected = 0, peak = 0;
  bool stop = false;
  bool sched_done = false;  // the scheduler has drained the queue and exited
  std::thread sched;
};

namespace {

int64_t in_use(const km_server* s) {
  int64_t b = s->resident;
  for (const auto& e : s->ex) b += e->busy ? e->reserve : e->held;
  return b;
}

void finish(km_server* s, const Job& j, km_result r, bool rejected = false) {
  const auto now = Clock::now();
  r.queue_ms = ms_between(j.submitted, j.started);
  r.run_ms = rejected ? 0.0 : ms_between(j.started, now);
  if (r.status == KM_OK) {
    ++s->completed;
    s->latency.push_back(ms_between(j.submitted, now));
  } else if (rejected) {
    ++s->rejected;
  } else {
    ++s->failed;
  }
  s->done[j.ticket] = r;
  s->cv_done.notify_all();
}

// likelihood requests: assemble + factorise + (profile) NLL and gradient on an executor's handle
inline bool is_lik(int kind) { return kind == KM_REQ_NLL_GRAD || kind == KM_REQ_PROFILE_NLL_GRAD; }

// runs one admitted job outside the lock; returns the result
km_result execute(km_server* s, Executor* e, Job& j, Factor* f) {
  km_result r{};
  r.factor_id = -1;
  const km_request& q = j.req;
  const km_serve_opts& o = s->o;
  switch (q.kind) {
    case KM_REQ_NLL_GRAD:
    case KM_REQ_PROFILE_NLL_GRAD: {
      int rc = km_assemble(e->h, q.prob.pts, q.prob.n, o.kernel_id, q.prob.params, 3, KM_METHOD_NYSTROM, 0.0, o.rank,
                           o.level_kind, o.level);
      if (rc == KM_OK) rc = km_factorize(e->h);
      if (rc == KM_OK)
        rc = (q.kind == KM_REQ_PROFILE_NLL_GRAD ? km_profile_nll_grad_seeded : km_nll_grad_seeded)(
            e->h, q.prob.y, q.nprobe, q.probe_seed, &r.nll, q.nprobe > 0 ? r.grad : nullptr);
      r.status = rc;
      break;
    }
    case KM_REQ_FACTOR: {
      km_handle* h = nullptr;
      int rc = km_create(&s->cfg, &h);
      if (rc == KM_OK) km::set_node_cluster_max(h, 1);
      if (rc == KM_OK)
        rc = km_assemble(h, q.prob.pts, q.prob.n, o.kernel_id, q.prob.params, 3, KM_METHOD_NYSTROM, 0.0, o.rank,
                         o.level_kind, o.level);
      if (rc == KM_OK) rc = km_factorize(h);
      if (rc == KM_OK) rc = km_logdet(h, &r.logdet);
      r.status = rc;
      if (rc == KM_OK) {
        km_stats st{};
        km_get_stats(h, &st);
        std::lock_guard<std::mutex> lk(s->mu);
        auto fac = std::make_unique<Factor>();
        fac->h = h;
        fac->n = q.prob.n;
        fac->bytes = st.device_bytes;
        r.factor_id = s->next_factor++;
        s->resident += fac->bytes;
        s->factors[r.factor_id] = std::move(fac);
      } else if (h) {
        km_destroy(h);
      }
      break;
    }
    case KM_REQ_SOLVE: {
      r.status = km_solve(f->h, q.b, q.x, q.nrhs);
      r.factor_id = q.factor_id;
      break;
    }
    case KM_REQ_RELEASE: {
      km_destroy(f->h);
      f->h = nullptr;
      r.status = KM_OK;
      r.factor_id = q.factor_id;
      break;
    }
    default:
      r.status = KM_ERR_BAD_ARG;
  }
  return r;
}

void executor_loop(km_server* s, Executor* e) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->cv_exec.wait(lk, [&] { return e->has_job || s->sched_done; });
    if (!e->has_job) return;
    e->has_job = false;
    Job j = e->job;
    Factor* f = nullptr;
    if (j.req.kind == KM_REQ_SOLVE || j.req.kind == KM_REQ_RELEASE) f = s->factors[j.req.factor_id].get();
    lk.unlock();
    km_result r = execute(s, e, j, f);
    int64_t held = e->held;
    if (is_lik(j.req.kind)) {
      km_stats st{};
      km_get_stats(e->h, &st);
      held = st.device_bytes;
    }
    int64_t fbytes = 0;
    if (f && f->h) {
      km_stats st{};
      km_get_stats(f->h, &st);
      fbytes = st.device_bytes;
    }
    lk.lock();
    if (f) {
      if (j.req.kind == KM_REQ_RELEASE) {
        s->resident -= f->bytes;
        s->factors.erase(j.req.factor_id);
      } else {
        s->resident += fbytes - f->bytes;
        f->bytes = fbytes;
        f->busy = false;
      }
    }
    e->held = held;
    e->busy = false;
    e->reserve = 0;
    s->peak = std::max(s->peak, in_use(s));
    finish(s, j, r);
    s->cv_sched.notify_all();
  }
}

// admission estimate of a request given the current state (lock held); -1 => reject now
int64_t estimate(km_server* s, const km_request& q, Factor* f) {
  const km_serve_opts& o = s->o;
  switch (q.kind) {
    case KM_REQ_NLL_GRAD:
    case KM_REQ_PROFILE_NLL_GRAD:
      return km_estimate_bytes(q.prob.n, o.rank, o.level_kind, o.level, q.nprobe + 1, q.nprobe > 0);
    case KM_REQ_FACTOR:
      return km_estimate_bytes(q.prob.n, o.rank, o.level_kind, o.level, 1, 0);
    case KM_REQ_SOLVE: {
      const int64_t full = km_estimate_bytes(f->n, o.rank, o.level_kind, o.level, q.nrhs, 0);
      return std::max<int64_t>(0, full - f->bytes);
    }
    default:
      return 0;
  }
}

void scheduler_loop(km_server* s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    bool progressed = false;
    const auto now = Clock::now();
    bool head_blocked = false;
    for (auto it = s->queue.begin(); it != s->queue.end();) {
      Job& j = *it;
      const km_request& q = j.req;
      Factor* f = nullptr;
      if (q.kind == KM_REQ_SOLVE || q.kind == KM_REQ_RELEASE) {
        auto fi = s->factors.find(q.factor_id);
        if (fi == s->factors.end() || fi->second->releasing) {
          km_result r{};
          r.status = KM_ERR_BAD_ARG;
          r.factor_id = q.factor_id;
          j.started = now;
          finish(s, j, r);
          it = s->queue.erase(it);
          progressed = true;
          continue;
        }
        f = fi->second.get();
        if (f->busy) {  // one request per factor at a time, in submission order
          ++it;
          continue;
        }
      }
      Executor* e = nullptr;
      for (auto& x : s->ex)
        if (!x->busy) {
          e = x.get();
          break;
        }
      if (!e) break;
      const int64_t need = estimate(s, q, f);
      if (need < 0 || need > s->budget) {
        km_result r{};
        r.status = need < 0 ? KM_ERR_BAD_ARG : KM_ERR_OOM;
        j.started = now;
        finish(s, j, r, need >= 0);
        it = s->queue.erase(it);
        progressed = true;
        continue;
      }
      // the executor's idle buffers are reused by an NLL request
      const bool uses_exec_mem = is_lik(q.kind);
      auto fits = [&] {
        const int64_t base = in_use(s) - (uses_exec_mem ? e->held : 0);
        return base + (uses_exec_mem ? std::max(need, e->held) : need) <= s->budget;
      };
      if (!fits()) {
        // give back buffers that idle executors keep between requests
        for (auto& x : s->ex)
          if (!x->busy && x->held > 0 && (x.get() != e || !uses_exec_mem)) {
            km_trim(x->h);
            x->held = 0;
            if (fits()) break;
          }
        if (uses_exec_mem && !fits() && e->held > 0) {
          km_trim(e->h);
          e->held = 0;
        }
      }
      if (!fits()) {
        if (it == s->queue.begin()) head_blocked = true;
        if (head_blocked && ms_between(s->queue.front().submitted, now) > kBackfillWindowMs) break;
        ++it;
        continue;
      }
      // admit
      j.need = need;
      j.started = now;
      if (f) {
        f->busy = true;
        if (q.kind == KM_REQ_RELEASE) f->releasing = true;
      }
      e->busy = true;
      e->reserve = uses_exec_mem ? std::max(need, e->held) : need;
      e->job = j;
      e->has_job = true;
      s->peak = std::max(s->peak, in_use(s));
      it = s->queue.erase(it);
      progressed = true;
      s->cv_exec.notify_all();
    }
    if (s->stop && s->queue.empty()) {
      bool idle = true;
      for (auto& x : s->ex) idle = idle && !x->busy;
      if (idle) {
        s->sched_done = true;
        s->cv_exec.notify_all();
        return;
      }
    }
    if (!progressed) s->cv_sched.wait_for(lk, std::chrono::milliseconds(20));
  }
}

}  // namespace

extern "C" int km_serve_create(const km_config* cfg, const km_serve_opts* o, km_server** out) {
  if (!cfg || !o || !out) return KM_ERR_BAD_ARG;
  *out = nullptr;
  if (o->rank < 2 || o->nworkers < 0 || o->nworkers > 64) return KM_ERR_BAD_ARG;
  if (o->kernel_id != KM_KERNEL_RATQUAD && o->kernel_id != KM_KERNEL_MATERN32) return KM_ERR_BAD_ARG;
  auto s = std::make_unique<km_server>();
  s->cfg = *cfg;
  s->o = *o;
  if (s->o.nworkers == 0) s->o.nworkers = 8;
  if (cudaSetDevice(cfg->device) != cudaSuccess) {
    cudaGetLastError();
    return KM_ERR_CUDA;
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    return KM_ERR_CUDA;
  }
  const double frac = cfg->hbm_budget_fraction > 0.0 ? cfg->hbm_budget_fraction : 0.8;
  s->budget = (int64_t)(frac * (double)total_b);
  for (int w = 0; w < s->o.nworkers; ++w) {
    auto e = std::make_unique<Executor>();
    const int rc = km_create(cfg, &e->h);
    if (rc != KM_OK) {
      for (auto& x : s->ex) km_destroy(x->h);
      return rc;
    }
    km::set_node_cluster_max(e->h, 1);
    s->ex.push_back(std::move(e));
  }
  km_server* raw = s.get();
  for (auto& e : s->ex) e->th = std::thread(executor_loop, raw, e.get());
  s->sched = std::thread(scheduler_loop, raw);
  *out = s.release();
  return KM_OK;
}

extern "C" int km_serve_submit(km_server* s, const km_request* r, uint64_t* ticket) {
  if (!s || !r || !ticket) return KM_ERR_BAD_ARG;
  const km_request& q = *r;
  if (is_lik(q.kind) || q.kind == KM_REQ_FACTOR) {
    if (!q.prob.pts || q.prob.n < 1 || (is_lik(q.kind) && (!q.prob.y || q.nprobe < 0)))
      return KM_ERR_BAD_ARG;
  } else if (q.kind == KM_REQ_SOLVE) {
    if (!q.b || !q.x || q.nrhs < 1) return KM_ERR_BAD_ARG;
  } else if (q.kind != KM_REQ_RELEASE) {
    return KM_ERR_BAD_ARG;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return KM_ERR_STATE;
  Job j;
  j.ticket = s->next_ticket++;
  j.req = q;
  j.submitted = Clock::now();
  s->queue.push_back(j);
  s->pending[j.ticket] = true;
  ++s->submitted;
  *ticket = j.ticket;
  s->cv_sched.notify_all();
  return KM_OK;
}

extern "C" int km_serve_wait(km_server* s, uint64_t ticket, int64_t timeout_ms, km_result* out) {
  if (!s || !out) return KM_ERR_BAD_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (!s->pending.count(ticket)) return KM_ERR_BAD_ARG;
  auto ready = [&] { return s->done.count(ticket) > 0; };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, ready);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    return KM_ERR_TIMEOUT;
  }
  *out = s->done[ticket];
  s->done.erase(ticket);
  s->pending.erase(ticket);
  return KM_OK;
}

extern "C" int km_serve_stats_get(km_server* s, km_serve_stats* out) {
  if (!s || !out) return KM_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->rejected = s->rejected;
  out->resident_factors = (int64_t)s->factors.size();
  out->bytes_in_use = in_use(s);
  out->peak_bytes = s->peak;
  out->budget_bytes = s->budget;
  if (!s->latency.empty()) {
    std::vector<double> v = s->latency;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
      const size_t i = (size_t)std::min<double>((double)v.size() - 1, std::ceil(p * (double)v.size()) - 1);
      return v[i];
    };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    double sum = 0.0;
    for (double x : v) sum += x;
    out->mean_ms = sum / (double)v.size();
  }
  return KM_OK;
}

extern "C" int km_serve_destroy(km_server* s) {
  if (!s) return KM_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_sched.notify_all();
  }
  if (s->sched.joinable()) s->sched.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->cv_exec.notify_all();
  }
  for (auto& e : s->ex)
    if (e->th.joinable()) e->th.join();
  for (auto& e : s->ex) km_destroy(e->h);
  for (auto& f : s->factors)
    if (f.second->h) km_destroy(f.second->h);
  delete s;
  return KM_OK;
}
