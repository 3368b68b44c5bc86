// Batched form: many independent Nystrom likelihood problems on one GPU.
//
// The reference evaluates one dataset per call (nll_objective, src/HODLR/src/maxlikfunctions.jl:
// 29-50: rebuild, symmetricfactorize!, negloglik, stoch_gradient).  Problems of 2^10..2^15
// points leave most of the 152 SMs idle when run one at a time, so the batch runs a pool of
// handles, each with its own stream and host thread, and hands out problems largest first
// (longest-processing-time order), which keeps every stream busy until the tail.  Handles keep
// their device buffers between problems and calls (capacity-based growth), so a steady batch
// allocates nothing after the first pass.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/kmhodlr.h"

namespace km {
void set_node_cluster_max(km_handle* h, int v);
}

struct km_batch {
  km_config cfg{};
  std::vector<km_handle*> workers;
  std::string err;
  std::mutex mu;
};

extern "C" int km_batch_create(const km_config* cfg, int nworkers, km_batch** out) {
  if (!cfg || !out) return KM_ERR_BAD_ARG;
  *out = nullptr;
  if (nworkers <= 0) nworkers = 8;
  if (nworkers > 64) return KM_ERR_BAD_ARG;
  auto* b = new km_batch;
  b->cfg = *cfg;
  for (int w = 0; w < nworkers; ++w) {
    km_handle* h = nullptr;
    const int rc = km_create(cfg, &h);
    if (rc != KM_OK) {
      for (auto* q : b->workers) km_destroy(q);
      delete b;
      return rc;
    }
    km::set_node_cluster_max(h, 1);
    b->workers.push_back(h);
  }
  *out = b;
  return KM_OK;
}

extern "C" int km_batch_destroy(km_batch* b) {
  if (!b) return KM_OK;
  for (auto* h : b->workers) km_destroy(h);
  delete b;
  return KM_OK;
}

extern "C" const char* km_batch_last_error(const km_batch* b) { return b ? b->err.c_str() : "null batch"; }

// one problem on one handle: assemble, factorise, NLL (+ gradient), or their profile forms
static int run_problem(km_handle* h, const km_batch_opts& o, const km_problem& p, uint64_t seed, double* nll,
                       double* grad) {
  int rc = km_assemble(h, p.pts, p.n, o.kernel_id, p.params, 3, KM_METHOD_NYSTROM, 0.0, o.rank, o.level_kind,
                       o.level);
  if (rc != KM_OK) return rc;
  if ((rc = km_factorize(h)) != KM_OK) return rc;
  return (o.profile ? km_profile_nll_grad_seeded : km_nll_grad_seeded)(h, p.y, o.nprobe, seed, nll,
                                                                        o.nprobe > 0 ? grad : nullptr);
}

extern "C" int km_batch_nll_grad(km_batch* b, const km_batch_opts* o, int64_t nprob, const km_problem* probs,
                                 double* nll, double* grad, int* status) {
  if (!b) return KM_ERR_BAD_ARG;
  std::lock_guard<std::mutex> guard(b->mu);  // one batch call at a time per pool
  b->err.clear();
  if (!o || nprob < 0 || (nprob > 0 && (!probs || !nll || !status)) || (o->nprobe > 0 && !grad) || o->nprobe < 0) {
    b->err = "bad batch arguments";
    return KM_ERR_BAD_ARG;
  }
  if (nprob == 0) return KM_OK;
  std::vector<int64_t> order(nprob);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t c) { return probs[a].n > probs[c].n; });
  std::atomic<int64_t> next{0};
  std::mutex emu;
  int64_t first_bad = -1;
  auto work = [&](km_handle* h) {
    for (;;) {
      const int64_t q = next.fetch_add(1);
      if (q >= nprob) return;
      const int64_t i = order[q];
      double g[3] = {0.0, 0.0, 0.0};
      double v = 0.0;
      const int rc = run_problem(h, *o, probs[i], o->probe_seed + (uint64_t)i, &v, g);
      status[i] = rc;
      nll[i] = rc == KM_OK ? v : 0.0;
      if (o->nprobe > 0)
        for (int j = 0; j < 3; ++j) grad[3 * i + j] = rc == KM_OK ? g[j] : 0.0;
      if (rc != KM_OK) {
        std::lock_guard<std::mutex> lk(emu);
        if (first_bad < 0 || i < first_bad) {
          first_bad = i;
          b->err = "problem " + std::to_string(i) + ": " + km_last_error(h);
        }
      }
    }
  };
  const int64_t nw = std::min<int64_t>((int64_t)b->workers.size(), nprob);
  std::vector<std::thread> th;
  for (int64_t w = 1; w < nw; ++w) th.emplace_back(work, b->workers[w]);
  work(b->workers[0]);
  for (auto& t : th) t.join();
  return first_bad < 0 ? KM_OK : status[first_bad];
}
