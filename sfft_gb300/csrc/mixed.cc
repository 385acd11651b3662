// mixed.cc — sfft_exec_many for signals of different (n, k, version,
// precision), executed as one CUDA graph.
//
// sfft_mixed_create groups the signals by plan.  The first sfft_mixed_exec
// runs every group's batched pipeline directly (which also sets kernel
// attributes and sizes the workspaces) and then captures the same work into
// one graph: each group is a branch forked from a master stream onto its
// plan's stream and joined back, so groups run concurrently.  Every later
// call writes fresh draws (from per-signal seeds, or glibc's streams) and
// input pointers into page-locked staging that the graph's copy nodes read,
// and launches the graph once.  Results land in a device arena with a fixed
// place per signal.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/sfft.h"

#include "engine.h"

namespace sfft {
void set_last_error(const char *m);
bool plan_staged_view(sfft_plan *plan, int num, int in_type, int *out_idx, void *out_val, int *out_count, long stride,
                      V12Dev *d);
bool plan_persist_prepare(sfft_plan *plan, int num, cudaStream_t s);
const int *plan_counters(sfft_plan *plan);
bool plan_enable_staging(sfft_plan *plan, int slots);
bool plan_stage(sfft_plan *plan, int num, const void *const *in, const unsigned *seeds);
bool plan_launch_staged(sfft_plan *plan, int num, int in_type, int *out_idx, void *out_val, int *out_count,
                        long stride, cudaStream_t s);
int k_bucket(int k);
sfft_plan *make_plan_tuned(int n, int k, int version, const sfft_options &o, int mode, bool &tuned);
}  // namespace sfft

namespace {
struct Group {
  int n, k, version, prec;
  sfft_plan *plan = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t join = nullptr;
  std::vector<int> members;  // signal indices, in slot order
  long cap = 0, idx_off = 0, cnt_off = 0;
  size_t vsize = 16, val_off = 0;
  bool tuned = false;
  bool persist = false;  // run by the persistent executor
};
}  // namespace

struct sfft_mixed {
  int device = 0, num = 0, in_type = 0;
  std::vector<Group> groups;
  std::vector<int> sig_group, sig_slot;
  int *d_idx = nullptr, *d_cnt = nullptr;
  unsigned char *d_val = nullptr;
  cudaStream_t master = nullptr;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // persistent executor (sfft_mixed_set_persistent)
  bool persistent = false;
  sfft::PersistProg prog{};
  sfft::PersistGroup *d_groups = nullptr;
  sfft::PersistItem *d_items = nullptr;
  int *d_state = nullptr;
  int persist_groups = 0;
  std::mutex mu;
};

namespace {

bool ok(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  cudaGetLastError();
  sfft::set_last_error((std::string(what) + ": " + cudaGetErrorString(e)).c_str());
  return false;
}

bool stage_all(sfft_mixed *m, const void *const *in, const unsigned *seeds) {
  for (Group &g : m->groups) {
    std::vector<const void *> gin(g.members.size());
    std::vector<unsigned> gseed(g.members.size());
    for (size_t i = 0; i < g.members.size(); i++) {
      gin[i] = in[g.members[i]];
      if (seeds) gseed[i] = seeds[g.members[i]];
    }
    if (!sfft::plan_stage(g.plan, (int)g.members.size(), gin.data(), seeds ? gseed.data() : nullptr)) {
      sfft::set_last_error("staging failed");
      return false;
    }
  }
  return true;
}

// Forks every group the persistent executor does not run from `master` onto
// its plan's stream and joins back; the executor's groups run as one kernel
// on `master`.
bool launch_all(sfft_mixed *m) {
  if (!ok(cudaEventRecord(m->fork, m->master), "fork")) return false;
  if (m->persistent && m->persist_groups) {
    for (Group &g : m->groups)
      if (g.persist && !sfft::plan_persist_prepare(g.plan, (int)g.members.size(), m->master)) {
        sfft::set_last_error("persistent executor: staging upload failed");
        return false;
      }
    if (!ok(sfft::persist_run(m->prog, m->master), "persistent executor")) return false;
  }
  for (Group &g : m->groups) {
    if (g.persist) continue;
    if (!ok(cudaStreamWaitEvent(g.stream, m->fork, 0), "fork wait")) return false;
    if (!sfft::plan_launch_staged(g.plan, (int)g.members.size(), m->in_type, m->d_idx + g.idx_off,
                                  m->d_val + g.val_off, m->d_cnt + g.cnt_off, g.cap, g.stream))
      return false;
    if (!ok(cudaEventRecord(g.join, g.stream), "join") || !ok(cudaStreamWaitEvent(m->master, g.join, 0), "join wait"))
      return false;
  }
  return true;
}

}  // namespace

extern "C" {

sfft_mixed *sfft_mixed_create(int num, const int *n, const int *k, const int *version, const int *precision,
                              int in_type, int tune, int device) {
  if (num < 1 || !n || !k || !version) {
    sfft::set_last_error("invalid arguments");
    return nullptr;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    sfft::set_last_error("no CUDA device: the GB300 sFFT engine has no CPU path");
    return nullptr;
  }
  sfft_mixed *m = new sfft_mixed();
  m->num = num;
  m->in_type = in_type;
  if (device >= 0) cudaSetDevice(device);
  cudaGetDevice(&m->device);
  std::map<std::tuple<int, int, int, int>, int> index;
  m->sig_group.resize(num);
  m->sig_slot.resize(num);
  for (int i = 0; i < num; i++) {
    const int v = version[i], pr = (v == SFFT_VERSION_3 || !precision) ? SFFT_PREC_FP64 : precision[i];
    // mode 2: one plan per (n, k bucket)
    const int kk = tune == 2 && v != SFFT_VERSION_3 ? sfft::k_bucket(k[i]) : k[i];
    auto key = std::make_tuple(n[i], kk, v, pr);
    auto it = index.find(key);
    int gi;
    if (it == index.end()) {
      gi = (int)m->groups.size();
      index[key] = gi;
      Group g;
      g.n = n[i];
      g.k = kk;
      g.version = v;
      g.prec = pr;
      m->groups.push_back(g);
    } else {
      gi = it->second;
    }
    m->sig_group[i] = gi;
    m->sig_slot[i] = (int)m->groups[gi].members.size();
    m->groups[gi].members.push_back(i);
  }
  long idx_total = 0, cnt_total = 0;
  size_t val_total = 0;
  bool good = true;
  for (Group &g : m->groups) {
    const int cnt = (int)g.members.size();
    sfft_options o{g.prec, m->device, cnt};
    g.plan = sfft::make_plan_tuned(g.n, g.k, g.version, o, tune, g.tuned);
    if (!g.plan || !sfft::plan_enable_staging(g.plan, cnt)) {
      good = false;
      break;
    }
    g.stream = (cudaStream_t)sfft_plan_stream(g.plan);
    g.cap = sfft_output_capacity(g.plan);
    g.vsize = (g.version < 2 && g.prec == SFFT_PREC_FP32) ? 8 : 16;
    g.idx_off = idx_total;
    g.val_off = val_total;
    g.cnt_off = cnt_total;
    cnt_total += cnt;
    idx_total += (long)cnt * g.cap;
    val_total += g.vsize * (size_t)cnt * g.cap;
    good = good && ok(cudaEventCreateWithFlags(&g.join, cudaEventDisableTiming), "event");
  }
  good = good && ok(cudaMalloc((void **)&m->d_idx, sizeof(int) * std::max(1L, idx_total)), "arena") &&
         ok(cudaMalloc((void **)&m->d_val, std::max<size_t>(16, val_total)), "arena") &&
         ok(cudaMalloc((void **)&m->d_cnt, sizeof(int) * num), "arena") &&
         ok(cudaStreamCreateWithFlags(&m->master, cudaStreamNonBlocking), "stream") &&
         ok(cudaEventCreateWithFlags(&m->fork, cudaEventDisableTiming), "event");
  if (!good) {
    sfft_mixed_destroy(m);
    return nullptr;
  }
  return m;
}

int sfft_mixed_exec(sfft_mixed *m, const void *const *in, const unsigned *seeds) {
  if (!m || !in) {
    sfft::set_last_error("invalid arguments");
    return -1;
  }
  std::lock_guard<std::mutex> lk(m->mu);
  cudaSetDevice(m->device);
  // the previous replay has read the staging once its stream drained
  if (!ok(cudaStreamSynchronize(m->master), "sync")) return -1;
  if (!stage_all(m, in, seeds)) return -1;
  if (m->exec) return ok(cudaGraphLaunch(m->exec, m->master), "graph launch") ? 0 : -1;
  // first call: run directly (its results are this call's), then capture
  if (!launch_all(m) || !ok(cudaStreamSynchronize(m->master), "sync")) return -1;
  if (!ok(cudaStreamBeginCapture(m->master, cudaStreamCaptureModeThreadLocal), "capture")) return -1;
  const long counted = sfft_kernel_launches();
  const bool launched = launch_all(m);
  // captured launches run when the graph is replayed; this call launched
  // only the direct ones
  sfft::note_launches(counted - sfft_kernel_launches());
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(m->master, &g);
  if (!launched || !ok(e, "end capture")) {
    if (g) cudaGraphDestroy(g);
    return -1;
  }
  m->graph = g;
  if (!ok(cudaGraphInstantiate(&m->exec, m->graph, 0), "instantiate")) return -1;
  return 0;
}

int sfft_mixed_sync(sfft_mixed *m) {
  if (!m) return -1;
  std::lock_guard<std::mutex> lk(m->mu);
  if (!ok(cudaStreamSynchronize(m->master), "sync")) return -1;
  // error bits the kernels set for any signal (hit-list overflow, a wait
  // of the persistent executor that ran out, ...)
  for (const Group &g : m->groups) {
    const int cnt = (int)g.members.size();
    std::vector<int> c((size_t)sfft::CNT_STRIDE * cnt);
    if (!ok(cudaMemcpy(c.data(), sfft::plan_counters(g.plan), sizeof(int) * c.size(), cudaMemcpyDeviceToHost),
            "counters"))
      return -1;
    for (int i = 0; i < cnt; i++) {
      const int e = c[(size_t)i * sfft::CNT_STRIDE + sfft::CNT_ERR];
      if (e) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "device reported error bits 0x%x on signal %d", e, g.members[i]);
        sfft::set_last_error(buf);
        return -1;
      }
    }
  }
  return 0;
}

int sfft_mixed_set_persistent(sfft_mixed *m, int on) {
  if (!m) {
    sfft::set_last_error("invalid arguments");
    return -1;
  }
  std::lock_guard<std::mutex> lk(m->mu);
  if (m->exec || m->persistent) {
    sfft::set_last_error("the persistent executor is chosen before the first execution");
    return -1;
  }
  if (!on) return 0;
  cudaSetDevice(m->device);
  std::vector<sfft::PersistGroup> pg;
  int slots = 0;
  for (Group &g : m->groups) {
    sfft::PersistGroup p{};
    const int cnt = (int)g.members.size();
    if (!sfft::plan_staged_view(g.plan, cnt, m->in_type, m->d_idx + g.idx_off, m->d_val + g.val_off,
                                m->d_cnt + g.cnt_off, g.cap, &p.d) ||
        !sfft::persist_eligible(p.d))
      continue;
    p.gslot0 = slots;
    p.slots = cnt;
    sfft::persist_shape(p);
    slots += cnt;
    g.persist = true;
    pg.push_back(p);
  }
  std::vector<sfft::PersistItem> items;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device) != cudaSuccess || sms <= 0) {
    cudaGetLastError();
    sms = 152;
  }
  sfft::persist_items(pg.data(), (int)pg.size(), items, sms);
  const size_t smem = sfft::persist_smem(pg.data(), (int)pg.size());
  if (smem > 200 * 1024) {  // with the executor's static shared memory, above a CTA's 227 KB
    for (Group &g : m->groups) g.persist = false;
    sfft::set_last_error("persistent executor: a plan needs more shared memory than one CTA has");
    return -1;
  }
  if (!pg.empty() &&
      (!ok(cudaMalloc((void **)&m->d_groups, sizeof(sfft::PersistGroup) * pg.size()), "executor") ||
       !ok(cudaMalloc((void **)&m->d_items, sizeof(sfft::PersistItem) * std::max<size_t>(1, items.size())),
           "executor") ||
       !ok(cudaMalloc((void **)&m->d_state, sizeof(int) * (2 + 4 * (size_t)slots)), "executor") ||
       !ok(cudaMemcpy(m->d_groups, pg.data(), sizeof(sfft::PersistGroup) * pg.size(), cudaMemcpyHostToDevice),
           "executor") ||
       !ok(cudaMemcpy(m->d_items, items.data(), sizeof(sfft::PersistItem) * items.size(), cudaMemcpyHostToDevice),
           "executor")))
    return -1;
  m->prog.groups = m->d_groups;
  m->prog.items = m->d_items;
  m->prog.nitems = (int)items.size();
  m->prog.state = m->d_state;
  m->prog.nslots_total = slots;
  m->prog.smem = smem;
  m->prog.in_type = m->in_type;
  m->persist_groups = (int)pg.size();
  m->persistent = true;
  return 0;
}

int sfft_mixed_result(sfft_mixed *m, int s, const int **idx, const void **val, int *value_bytes, long *cap) {
  if (!m || s < 0 || s >= m->num) {
    sfft::set_last_error("invalid arguments");
    return -1;
  }
  const Group &g = m->groups[m->sig_group[s]];
  const int slot = m->sig_slot[s];
  if (idx) *idx = m->d_idx + g.idx_off + (long)slot * g.cap;
  if (val) *val = m->d_val + g.val_off + g.vsize * (size_t)slot * g.cap;
  if (value_bytes) *value_bytes = (int)g.vsize;
  if (cap) *cap = g.cap;
  int c = 0;
  if (!ok(cudaMemcpy(&c, m->d_cnt + g.cnt_off + slot, sizeof(int), cudaMemcpyDeviceToHost), "count"))
    return -1;
  return c;
}

long sfft_mixed_result_host(sfft_mixed *m, int s, int *idx, void *val, long cap) {
  const int *di = nullptr;
  const void *dv = nullptr;
  int vb = 0;
  long dcap = 0;
  const int c = sfft_mixed_result(m, s, &di, &dv, &vb, &dcap);
  if (c < 0) return -1;
  const long n = std::min<long>(c, cap);
  if (n > 0 && ((idx && !ok(cudaMemcpy(idx, di, sizeof(int) * n, cudaMemcpyDeviceToHost), "copy")) ||
                (val && !ok(cudaMemcpy(val, dv, (size_t)vb * n, cudaMemcpyDeviceToHost), "copy"))))
    return -1;
  return c;
}

int sfft_mixed_groups(const sfft_mixed *m) { return m ? (int)m->groups.size() : -1; }

void *sfft_mixed_stream(const sfft_mixed *m) { return m ? (void *)m->master : nullptr; }

void sfft_mixed_destroy(sfft_mixed *m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->master) cudaStreamSynchronize(m->master);
  if (m->exec) cudaGraphExecDestroy(m->exec);
  if (m->graph) cudaGraphDestroy(m->graph);
  for (Group &g : m->groups) {
    if (g.join) cudaEventDestroy(g.join);
    if (g.plan) sfft_free_plan(g.plan);
  }
  if (m->fork) cudaEventDestroy(m->fork);
  if (m->master) cudaStreamDestroy(m->master);
  cudaFree(m->d_idx);
  cudaFree(m->d_val);
  cudaFree(m->d_cnt);
  cudaFree(m->d_groups);
  cudaFree(m->d_items);
  cudaFree(m->d_state);
  delete m;
}

}  // extern "C"
