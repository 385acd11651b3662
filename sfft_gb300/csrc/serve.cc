// serve.cc — continuous-batching sparse-FFT server on one GPU.
//
// Requests of any (n, k, version, precision) arrive through
// sfft_server_submit.  A scheduler thread groups the queued requests by plan
// and launches a batch per plan as soon as that plan's previous batch has
// left its stream, so requests that arrive while other work runs join the
// next batch of their plan, and batches of different plans run concurrently
// on their plans' streams.  Plans (filters, windows, twiddles, workspace)
// stay on the device in a cache; a plan or batch is admitted only while the
// device memory it needs fits the server's budget (idle plans are evicted
// least recently used first; otherwise the request waits).  Every request
// draws its random numbers from its own seed, so its result is the same
// alone and in any mix.  Completion is signalled by a host function queued
// on the plan's stream after the batch, which stamps each request's latency.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/sfft.h"
#include "engine.h"

namespace sfft {
void set_last_error(const char *m);
const int *plan_counters(sfft_plan *plan);
int k_bucket(int k);
sfft_plan *make_plan_tuned(int n, int k, int version, const sfft_options &o, int mode, bool &tuned);
}

namespace {

using Clock = std::chrono::steady_clock;

struct Batch;

struct Request {
  long id = 0;
  int n = 0, k = 0, version = 0, prec = 0, in_type = 0;
  const void *in = nullptr;
  void *staged = nullptr;  // device copy of a host input
  unsigned seed = 0;
  Clock::time_point t_submit, t_done;
  std::atomic<bool> done{false};
  bool failed = false;
  Batch *batch = nullptr;
  int slot = 0;
  std::string error;
};

struct PlanKey {
  int n, k, version, prec;
  bool operator<(const PlanKey &o) const {
    return std::tie(n, k, version, prec) < std::tie(o.n, o.k, o.version, o.prec);
  }
};

struct PlanEntry {
  PlanKey key;
  sfft_plan *plan = nullptr;
  long cap = 0;
  long bytes = 0;
  std::atomic<bool> busy{false};  // a batch is on its stream
  cudaStream_t stream = nullptr;
  long last_used = 0;
  bool tuned = false;
};

struct Server;

struct Batch {
  Server *srv = nullptr;
  PlanEntry *pe = nullptr;
  std::vector<Request *> reqs;
  std::vector<char> taken;  // per slot: its request was collected (and deleted)
  int *d_idx = nullptr;
  void *d_val = nullptr;
  int *d_cnt = nullptr;
  int *d_ctr = nullptr;  // the plan's counters of this batch's slots, copied after it ran
  long bytes = 0, cap = 0;
  int collected = 0;
  size_t val_size = 16;
  std::atomic<bool> complete{false};
  // results moved to host memory to free the device (see spill_batch)
  bool spilled = false;
  std::vector<int> h_cnt, h_err;
  std::vector<std::vector<int>> h_idx;
  std::vector<std::vector<char>> h_val;
};

}  // namespace

struct sfft_server {
  int device = 0, max_batch = 32, k_round = 0, tune_invalid = 0, v2_voted = 0;
  long budget = 0, held = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> queue;
  std::unordered_map<long, Request *> reqs;
  std::map<PlanKey, PlanEntry *> plans;
  std::list<Batch *> batches;  // launched and not yet fully collected, oldest first
  long next_id = 1, tick = 0;
  bool stop = false;
  std::thread worker;
  // statistics
  long n_batches = 0, n_evicted = 0, n_plans = 0, n_deferred = 0, n_spilled = 0;
};

namespace {

struct Server : sfft_server {};

// Runs on a CUDA driver thread after the batch: no CUDA calls and no
// server lock (plan construction may hold it); flags are atomic and the
// waiters poll with a timeout.
// The batch may be collected and deleted as soon as its last request is
// marked done, so everything that touches the batch or its plan comes
// first, and the requests are marked from a local copy of the list.
void host_done(void *arg) {
  Batch *b = (Batch *)arg;
  sfft_server *s = (sfft_server *)b->srv;
  const auto now = Clock::now();
  const std::vector<Request *> reqs = b->reqs;
  b->complete.store(true, std::memory_order_release);
  b->pe->busy.store(false, std::memory_order_release);
  for (Request *r : reqs) {  // a marked request may be collected at once
    r->t_done = now;
    r->done.store(true, std::memory_order_release);
  }
  s->cv_done.notify_all();  // the server outlives its callbacks (destroy synchronises the device)
  s->cv_work.notify_all();
}

int round_k(int k, int mode) {
  if (!mode || k <= 8) return k;
  if (mode == 2) {
    int b = 8;
    while (b < k) b *= 2;
    return b;
  }
  // smallest value of the grid ceil(8 * 2^(j/4)) that is >= k
  for (int j = 0;; j++) {
    const int v = (int)std::ceil(8.0 * std::pow(2.0, j / 4.0));
    if (v >= k) return v;
  }
}

long device_free() {
  size_t f = 0, t = 0;
  if (cudaMemGetInfo(&f, &t) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (long)f;
}

void free_batch_device(Batch *b) {
  cudaFree(b->d_idx);
  cudaFree(b->d_val);
  cudaFree(b->d_cnt);
  cudaFree(b->d_ctr);
  b->d_idx = nullptr;
  b->d_val = nullptr;
  b->d_cnt = nullptr;
  b->d_ctr = nullptr;
  for (size_t i = 0; i < b->reqs.size(); i++)
    if (!b->taken[i] && b->reqs[i]->staged) {
      cudaFree(b->reqs[i]->staged);
      b->reqs[i]->staged = nullptr;
    }
}

// Moves a finished batch's uncollected results to host memory and frees its
// device memory.  Results are held until their requests are waited for, in
// any order; without spilling, a client that waits for an early request
// while later requests' results fill the budget would never see the early
// one admitted.
bool spill_batch(sfft_server *s, Batch *b) {
  cudaSetDevice(s->device);
  const int m = (int)b->reqs.size();
  b->h_cnt.assign(m, 0);
  b->h_idx.resize(m);
  b->h_val.resize(m);
  std::vector<int> ctr((size_t)m * sfft::CNT_STRIDE);
  if (cudaMemcpy(b->h_cnt.data(), b->d_cnt, sizeof(int) * m, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(ctr.data(), b->d_ctr, sizeof(int) * ctr.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  b->h_err.assign(m, 0);
  for (int i = 0; i < m; i++) b->h_err[i] = ctr[(size_t)i * sfft::CNT_STRIDE + sfft::CNT_ERR];
  for (int i = 0; i < m; i++) {
    if (b->taken[i]) continue;
    const long c = std::max(0L, std::min((long)b->h_cnt[i], b->cap));
    b->h_idx[i].resize(c);
    b->h_val[i].resize(c * b->val_size);
    if (c && (cudaMemcpy(b->h_idx[i].data(), b->d_idx + (size_t)i * b->cap, sizeof(int) * c,
                         cudaMemcpyDeviceToHost) != cudaSuccess ||
              cudaMemcpy(b->h_val[i].data(), (char *)b->d_val + b->val_size * (size_t)i * b->cap,
                         b->val_size * c, cudaMemcpyDeviceToHost) != cudaSuccess)) {
      cudaGetLastError();
      return false;
    }
  }
  free_batch_device(b);
  b->spilled = true;
  s->held -= b->bytes;
  b->bytes = 0;
  s->n_spilled++;
  return true;
}

// Makes `need` more bytes fit the budget: first moves finished batches'
// results to host memory (oldest first; cheap to undo), then evicts idle
// plans (least recently used first, never `keep`; rebuilding a large plan
// takes seconds).
bool make_room(sfft_server *s, long need, const PlanEntry *keep = nullptr) {
  while (s->held + need > s->budget) {
    Batch *sp = nullptr;
    for (Batch *b : s->batches)
      if (!b->spilled && b->complete.load(std::memory_order_acquire)) {
        sp = b;
        break;
      }
    if (sp && spill_batch(s, sp)) continue;
    PlanEntry *victim = nullptr;
    for (auto &kv : s->plans)
      if (kv.second != keep && !kv.second->busy.load() && (!victim || kv.second->last_used < victim->last_used))
        victim = kv.second;
    if (!victim) return false;
    s->held -= victim->bytes;
    sfft_free_plan(victim->plan);
    s->plans.erase(victim->key);
    delete victim;
    s->n_evicted++;
  }
  return true;
}

// Device bytes of a plan with `slots` batch slots, from its shape.
long estimate_bytes(const PlanKey &key, int slots, int tune) {
  long f[11];
  int m = -1;
  sfft_params prm;
  if (key.version < 2 && tune == 2 && sfft_tuned_params(key.n, key.k, key.version, &prm) >= 0)
    m = sfft_describe_plan_params(key.n, key.k, (enum sfft_version)key.version, &prm, f, 11);
  if (m < 0) m = sfft_describe_plan(key.n, key.k, (enum sfft_version)key.version, f, 11);
  if (m < 0 && key.version < 2 && tune && sfft_tuned_params(key.n, key.k, key.version, &prm) >= 0)
    m = sfft_describe_plan_params(key.n, key.k, (enum sfft_version)key.version, &prm, f, 11);
  const long cs = key.prec == SFFT_PREC_FP64 ? 16 : 8;
  if (m < 0) return 4L * key.n * 16 * slots;
  if (key.version < 2) {
    const long xs = f[10], W = f[3], L = f[5] + f[7], num = f[1];
    const long out = std::min(W, f[4] * num) * (key.n / std::max(W, 1L)) + 8L * num * key.n / f[0];
    const long per = xs * (cs + 8) + 4L * key.n + L * num * 4 + W * 8 + out * (cs + 4) + 4096;
    const long cst = (f[8] + f[9]) * cs + 2L * key.n / f[0] * 32 + (f[0] + f[2] + W) * cs;
    return cst + per * slots;
  }
  const long W = f[0], B1 = f[1], B2 = f[3];
  const long per = 32 * (W + B1 + B2) + 16 * 2 * (f[4] + 2) + 64 * (W + B1 + B2 + 8L * key.k) * 4;
  return (f[2] + f[4]) * 16 + 16L * 3 * key.n / B1 + 16L * 3 * key.n / B2 + per * slots;
}

PlanEntry *get_plan(sfft_server *s, const PlanKey &key, std::string &err) {
  auto it = s->plans.find(key);
  if (it != s->plans.end()) {
    it->second->last_used = ++s->tick;  // most recently used
    return it->second;
  }
  const long need = estimate_bytes(key, s->max_batch, s->tune_invalid);
  if (need > s->budget) {
    err = "request needs more device memory than the server's budget";
    return nullptr;
  }
  if (!make_room(s, need)) return (PlanEntry *)-1;  // defer
  sfft_options o{key.prec, s->device, s->max_batch};
  bool tuned = false;
  sfft_plan *p = sfft::make_plan_tuned(key.n, key.k, key.version, o, s->tune_invalid, tuned);
  if (p && s->v2_voted && key.version == SFFT_VERSION_2 && sfft_plan_v2_voted(p, 1) != 0) {
    sfft_free_plan(p);
    p = nullptr;
  }
  if (!p) {
    err = sfft_last_error();
    return nullptr;
  }
  PlanEntry *pe = new PlanEntry();
  pe->key = key;
  pe->plan = p;
  pe->cap = sfft_output_capacity(p);
  pe->bytes = sfft_plan_footprint(p);  // what the plan holds (the estimate only admitted it)
  pe->tuned = tuned;
  pe->stream = (cudaStream_t)sfft_plan_stream(p);
  s->plans[key] = pe;
  s->held += pe->bytes;
  s->n_plans++;
  return pe;
}

void fail(sfft_server *s, Request *r, const std::string &e) {
  r->failed = true;
  r->error = e;
  r->t_done = Clock::now();
  r->done.store(true, std::memory_order_release);
  s->cv_done.notify_all();
}

// One scheduling pass under the lock: launch a batch for every plan that
// has queued requests and an idle stream.
void schedule(sfft_server *s) {
  std::map<std::pair<PlanKey, int>, std::vector<Request *>> groups;  // plan and input type
  for (Request *r : s->queue) groups[{PlanKey{r->n, r->k, r->version, r->prec}, r->in_type}].push_back(r);
  std::deque<Request *> keep;
  for (auto &g : groups) {
    std::string err;
    const PlanKey key = g.first.first;
    PlanEntry *pe = get_plan(s, key, err);
    if (pe == (PlanEntry *)-1) {  // no room yet: wait for batches to finish
      s->n_deferred++;
      for (Request *r : g.second) keep.push_back(r);
      continue;
    }
    if (!pe) {
      for (Request *r : g.second) fail(s, r, err);
      continue;
    }
    if (pe->busy.load(std::memory_order_acquire)) {
      for (Request *r : g.second) keep.push_back(r);
      continue;
    }
    const int m = std::min((int)g.second.size(), s->max_batch);
    Batch *b = new Batch();
    b->srv = (Server *)s;
    b->pe = pe;
    b->val_size = (key.version < 2 && key.prec == SFFT_PREC_FP32) ? 8 : 16;
    b->cap = pe->cap;
    b->reqs.assign(g.second.begin(), g.second.begin() + m);
    b->taken.assign(m, 0);
    for (int i = m; i < (int)g.second.size(); i++) keep.push_back(g.second[i]);
    const long obytes = (long)m * pe->cap * (4 + (long)b->val_size) + 4L * m + 4L * m * sfft::CNT_STRIDE;
    long sbytes = 0;
    for (Request *r : b->reqs)
      if (!r->staged && r->in_type >= 100) sbytes += (long)r->n * ((r->in_type - 100) == SFFT_IN_C64 ? 8 : 16);
    if (pe->bytes + obytes + sbytes > s->budget) {  // would never fit
      for (Request *r : b->reqs) fail(s, r, "batch and plan need more device memory than the server's budget");
      delete b;
      continue;
    }
    if (!make_room(s, obytes + sbytes, pe)) {  // the batch's own plan stays
      for (Request *r : b->reqs) keep.push_back(r);
      delete b;
      s->n_deferred++;
      continue;
    }
    b->bytes = obytes + sbytes;
    s->held += b->bytes;
    cudaStream_t st = pe->stream;  // everything of this batch is ordered on the plan's stream
    bool ok = cudaMallocAsync((void **)&b->d_idx, sizeof(int) * (size_t)m * pe->cap, st) == cudaSuccess &&
              cudaMallocAsync(&b->d_val, b->val_size * (size_t)m * pe->cap, st) == cudaSuccess &&
              cudaMallocAsync((void **)&b->d_cnt, sizeof(int) * m, st) == cudaSuccess &&
              cudaMallocAsync((void **)&b->d_ctr, sizeof(int) * m * sfft::CNT_STRIDE, st) == cudaSuccess;
    std::vector<const void *> ins(m);
    std::vector<unsigned> seeds(m);
    int in_type = SFFT_IN_C128;
    for (int i = 0; ok && i < m; i++) {
      Request *r = b->reqs[i];
      r->batch = b;
      r->slot = i;
      seeds[i] = r->seed;
      const int it = r->in_type >= 100 ? r->in_type - 100 : r->in_type;
      in_type = it;
      if (r->in_type >= 100) {  // host input: stage it
        const size_t nb = (size_t)r->n * (it == SFFT_IN_C64 ? 8 : 16);
        ok = cudaMallocAsync(&r->staged, nb, st) == cudaSuccess &&
             cudaMemcpyAsync(r->staged, r->in, nb, cudaMemcpyHostToDevice, st) == cudaSuccess;
        ins[i] = r->staged;
      } else {
        ins[i] = r->in;
      }
    }
    pe->busy.store(true, std::memory_order_release);
    pe->last_used = ++s->tick;
    if (ok)
      ok = sfft_exec_batch_ex(pe->plan, m, ins.data(), in_type, seeds.data(), b->d_idx, b->d_val, b->d_cnt,
                              pe->cap, st) == 0;
    // the slots' counters (error bits) belong to this batch once it ran
    if (ok)
      ok = cudaMemcpyAsync(b->d_ctr, sfft::plan_counters(pe->plan), sizeof(int) * m * sfft::CNT_STRIDE,
                           cudaMemcpyDeviceToDevice, st) == cudaSuccess;
    if (ok) ok = cudaLaunchHostFunc(st, host_done, b) == cudaSuccess;
    if (ok) s->batches.push_back(b);
    if (!ok) {
      cudaGetLastError();
      const std::string e = std::string("batch launch failed: ") + sfft_last_error();
      pe->busy.store(false, std::memory_order_release);
      for (Request *r : b->reqs) fail(s, r, e);
      s->held -= b->bytes;
      delete b;
      continue;
    }
    s->n_batches++;
  }
  s->queue.swap(keep);
}

void worker_main(sfft_server *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    if (!s->queue.empty()) schedule(s);
    s->cv_work.wait_for(lk, std::chrono::microseconds(200));
  }
}

}  // namespace

extern "C" {

sfft_server *sfft_server_create(const sfft_server_options *opt) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    sfft::set_last_error("no CUDA device: the GB300 sFFT engine has no CPU path");
    return nullptr;
  }
  sfft_server *s = new sfft_server();
  if (opt) {
    if (opt->device >= 0) s->device = opt->device;
    if (opt->max_batch > 0) s->max_batch = opt->max_batch;
    s->budget = opt->hbm_budget_bytes;
    s->k_round = opt->k_round;
    s->tune_invalid = opt->tune_invalid;
    s->v2_voted = opt->v2_voted;
  }
  cudaSetDevice(s->device);
  if (s->budget <= 0) s->budget = (long)(0.8 * device_free());
  s->worker = std::thread(worker_main, s);
  return s;
}

void sfft_server_destroy(sfft_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->worker.join();
  cudaSetDevice(s->device);
  cudaDeviceSynchronize();
  for (Batch *b : s->batches) {  // uncollected results
    if (!b->spilled) free_batch_device(b);
    delete b;
  }
  for (auto &kv : s->plans) {
    sfft_free_plan(kv.second->plan);
    delete kv.second;
  }
  for (auto &kv : s->reqs) delete kv.second;
  delete s;
}

long sfft_server_submit(sfft_server *s, int n, int k, enum sfft_version version, int precision, const void *in,
                        int in_type, unsigned seed) {
  if (!s || !in || n < 16 || (n & (n - 1)) || k < 1) {
    sfft::set_last_error("invalid request");
    return -1;
  }
  cudaPointerAttributes a;
  bool dev = cudaPointerGetAttributes(&a, in) == cudaSuccess &&
             (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged);
  cudaGetLastError();
  Request *r = new Request();
  r->n = n;
  r->k = s->tune_invalid == 2 && version != SFFT_VERSION_3 ? sfft::k_bucket(k) : round_k(k, s->k_round);
  if (s->tune_invalid && version == SFFT_VERSION_3 && r->k < 8) r->k = 8;
  r->version = (int)version;
  r->prec = version == SFFT_VERSION_3 ? SFFT_PREC_FP64 : precision;
  r->in = in;
  r->in_type = dev ? in_type : in_type + 100;  // +100 marks a host input to stage
  r->seed = seed;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> g(s->mu);
    r->id = s->next_id++;
    s->reqs[r->id] = r;
    s->queue.push_back(r);
  }
  s->cv_work.notify_all();
  return r->id;
}

long sfft_server_wait(sfft_server *s, long id, int *out_idx, complex_t *out_val, long cap, double *latency_ms) {
  return sfft_server_wait_for(s, id, out_idx, out_val, cap, latency_ms, -1.0);
}

long sfft_server_wait_for(sfft_server *s, long id, int *out_idx, complex_t *out_val, long cap, double *latency_ms,
                          double timeout_ms) {
  if (!s) return -1;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) {
    sfft::set_last_error("unknown request");
    return -1;
  }
  Request *r = it->second;
  const auto deadline = Clock::now() + std::chrono::microseconds((long)(1000.0 * std::max(0.0, timeout_ms)));
  while (!r->done.load(std::memory_order_acquire)) {
    if (timeout_ms >= 0 && Clock::now() >= deadline) {
      sfft::set_last_error("timed out waiting for the request (it stays queued)");
      return -2;
    }
    s->cv_done.wait_for(lk, std::chrono::microseconds(500));
  }
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  long result = -1;
  if (r->failed) {
    sfft::set_last_error(r->error.c_str());
  } else {
    Batch *b = r->batch;
    cudaSetDevice(s->device);
    int cnt = 0, err = 0;
    bool ok = true;
    if (b->spilled) {
      cnt = (int)b->h_idx[r->slot].size();
      err = b->h_err[r->slot];
    } else {
      ok = cudaMemcpy(&cnt, b->d_cnt + r->slot, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess &&
           cudaMemcpy(&err, b->d_ctr + (size_t)r->slot * sfft::CNT_STRIDE + sfft::CNT_ERR, sizeof(int),
                      cudaMemcpyDeviceToHost) == cudaSuccess;
    }
    if (ok && err) {  // the transform itself flagged this signal
      char msg[160];
      std::snprintf(msg, sizeof msg,
                    "device reported error bits 0x%x (1 hit list, 2 output, 4 v3 no fixpoint, 8 v3 capacity)", err);
      sfft::set_last_error(msg);
      ok = false;
    }
    if (ok && (out_idx || out_val) && cnt > cap) {  // no buffers: only the count is asked for
      sfft::set_last_error("output capacity too small");
      ok = false;
    }
    if (ok && out_idx) {
      if (b->spilled)
        std::memcpy(out_idx, b->h_idx[r->slot].data(), sizeof(int) * (size_t)cnt);
      else
        ok = cudaMemcpy(out_idx, b->d_idx + (size_t)r->slot * b->cap, sizeof(int) * cnt, cudaMemcpyDefault) ==
             cudaSuccess;
    }
    if (ok && out_val) {
      std::vector<char> tmp;
      const char *src = nullptr;
      if (b->spilled) {
        src = b->h_val[r->slot].data();
      } else {
        tmp.resize(b->val_size * (size_t)cnt);
        ok = cudaMemcpy(tmp.data(), (char *)b->d_val + b->val_size * (size_t)r->slot * b->cap,
                        b->val_size * (size_t)cnt, cudaMemcpyDeviceToHost) == cudaSuccess;
        src = tmp.data();
      }
      if (ok && b->val_size == 16) {
        std::memcpy(out_val, src, 16 * (size_t)cnt);
      } else if (ok) {
        const float *f = (const float *)src;
        double *o = (double *)out_val;
        for (size_t i = 0; i < 2 * (size_t)cnt; i++) o[i] = f[i];
      }
    }
    if (ok) result = cnt;
    if (r->staged) {  // the batch is complete: its staged input is no longer read
      cudaFree(r->staged);
      r->staged = nullptr;
    }
    b->taken[r->slot] = 1;  // r is deleted below: the batch must not touch it again
    if (b->spilled) {
      std::vector<int>().swap(b->h_idx[r->slot]);
      std::vector<char>().swap(b->h_val[r->slot]);
    }
    // the batch's memory goes once all its requests are collected
    if (++b->collected == (int)b->reqs.size()) {
      if (!b->spilled) free_batch_device(b);  // every slot is taken: no request is touched
      s->held -= b->bytes;
      s->batches.remove(b);
      delete b;
    }
  }
  s->reqs.erase(it);
  delete r;
  lk.unlock();
  s->cv_work.notify_all();
  return result;
}

long sfft_server_count(sfft_server *s, long id, double timeout_ms) {
  if (!s) return -1;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) {
    sfft::set_last_error("unknown request");
    return -1;
  }
  Request *r = it->second;
  const auto deadline = Clock::now() + std::chrono::microseconds((long)(1000.0 * std::max(0.0, timeout_ms)));
  while (!r->done.load(std::memory_order_acquire)) {
    if (timeout_ms >= 0 && Clock::now() >= deadline) {
      sfft::set_last_error("timed out waiting for the request (it stays queued)");
      return -2;
    }
    s->cv_done.wait_for(lk, std::chrono::microseconds(500));
  }
  if (r->failed) {
    sfft::set_last_error(r->error.c_str());
    return -1;
  }
  Batch *b = r->batch;
  if (b->spilled) return (long)b->h_idx[r->slot].size();
  cudaSetDevice(s->device);
  int cnt = 0;
  if (cudaMemcpy(&cnt, b->d_cnt + r->slot, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    sfft::set_last_error("count read failed");
    return -1;
  }
  return cnt;
}

long sfft_server_plan_bytes(int n, int k, enum sfft_version version, int precision, int max_batch) {
  if (n < 16 || (n & (n - 1)) || k < 1 || max_batch < 1) return -1;
  const int prec = version == SFFT_VERSION_3 ? SFFT_PREC_FP64 : precision;
  return estimate_bytes(PlanKey{n, k, (int)version, prec}, max_batch, 0);
}

int sfft_server_stats(sfft_server *s, long *stats, int nstats) {
  if (!s || !stats) return -1;
  std::lock_guard<std::mutex> g(s->mu);
  const long v[] = {s->n_batches, s->n_plans, s->n_evicted, s->n_deferred, (long)s->plans.size(), s->held,
                    s->budget, (long)s->queue.size(), s->n_spilled};
  const int m = std::min(nstats, (int)(sizeof v / sizeof v[0]));
  for (int i = 0; i < m; i++) stats[i] = v[i];
  return m;
}

}  // extern "C"

