// api.cc — the C interface of include/sfft.h on top of the GB300 kernels.
//
// A plan owns device-resident filters, twiddle tables and a workspace for
// `max_batch` signals.  Execution draws the reference's random numbers on
// the host (glibc random()/drand48(), same order as src/computefourier-
// 1.0-2.0.cc:465-474, :62 and src/computefourier-3.0.cc:800-810), uploads
// them, and launches the pipeline on the plan's stream.  No computation of
// the transform happens on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <set>
#include <string>
#include <vector>

#include "../../include/sfft.h"
#include "engine.h"
#include "host_plan.h"

#include <atomic>
#include <deque>

namespace sfft {
static std::atomic<long> g_launches{0};
void note_launches(long n) { g_launches += n; }
void mark(StageEvents *se, cudaStream_t s) {
  if (se && se->recorded < 8) cudaEventRecord(se->ev[se->recorded++], s);
}
}  // namespace sfft

namespace {

thread_local std::string g_err;

void set_err(const std::string &m) { g_err = m; }

bool cuda_ok(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  set_err(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

// A device allocation owned by a plan.
struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  bool ensure(size_t b) {
    if (b <= bytes && p) return true;
    release();
    if (b == 0) b = 16;
    if (cudaMalloc(&p, b) != cudaSuccess) {
      cudaGetLastError();
      set_err("device allocation of " + std::to_string(b) + " bytes failed");
      p = nullptr;
      return false;
    }
    bytes = b;
    return true;
  }
  template <typename T>
  bool upload(const std::vector<T> &v) {
    if (!ensure(sizeof(T) * v.size())) return false;
    return cuda_ok(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice), "upload");
  }
  template <typename T>
  T *as() const {
    return (T *)p;
  }
};

int gcd_ref(int a, int b) { return (a % b == 0) ? b : gcd_ref(b, a % b); }  // src/utils.cc:41-46

int mod_inverse_ref(int a, int n) {  // src/utils.cc:85-101
  int i = n, v = 0, d = 1;
  while (a > 0) {
    int t = i / a, x = a;
    a = i % x;
    i = x;
    x = d;
    d = v - t * x;
    v = x;
  }
  v %= n;
  if (v < 0) v = (v + n) % n;
  return v;
}

int ilog2(long v) {
  int m = 0;
  while ((1L << m) < v) m++;
  return m;
}

std::vector<float> to_f32(const std::vector<double> &v) {
  std::vector<float> o(v.size());
  for (size_t i = 0; i < v.size(); i++) o[i] = (float)v[i];
  return o;
}

}  // namespace

struct PlanImpl {
  int version = 0, n = 0, k = 0, prec = sfft::PREC_FP64, device = 0, max_batch = 16;
  int voted = 0;  // v2: estimate voted candidates only (opt-in, not the reference's output)
  sfft::V12Params p12;
  sfft::V3Params p3;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  // host-buffer pipeline of sfft_exec_many: copies in / out on their own streams
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_comp[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr};
  std::mutex mu;
  // constants
  DBuf taps_a, taps_b, win_a, win_b, win32_a, win32_b, tw_a, tw_b, tw_c;
  int win_half_a = 0, win_half_b = 0;
  // workspace
  int slots = 0;
  DBuf xs, xs32, xs_tmp, comb_buf, comb_tmp, J, score, hits, comb_bits, comb_list, counters, out_idx, out_val;
  DBuf man, man_tmp, g1, g2, perm, est_f, est_v, map_keys, map_vals, map_list;
  DBuf rparams, inputs, dense_ptrs, in_stage, dense_stage, trace, cnt_stash;
  std::vector<unsigned> epoch;
  int hit_cap = 0, out_cap = 0, est_cap = 0, map_cap = 0, table_cap = 0;
  int large_b = 0, large_c = 0;  // FFTs longer than one CTA's shared memory
  int rp_stride = 0;
  std::vector<int> last_rp;  // draws of the last exec (slot 0)
  // page-locked staging for graph replays (draws and input pointers are
  // written here by the host and copied by captured memcpy nodes)
  int *h_rp = nullptr;
  const void **h_in = nullptr;
  int staged_slots = 0;
  // stage timing (sfft_profile): event sets of launches not yet harvested
  bool profiling = false;
  std::vector<sfft::StageEvents *> free_sets;
  std::deque<sfft::StageEvents *> pending;
  double stage_ms[8] = {0};
  long profiled = 0;
  ~PlanImpl() {
    for (auto *e : free_sets) destroy(e);
    for (auto *e : pending) destroy(e);
    if (h_rp) cudaFreeHost(h_rp);
    if (h_in) cudaFreeHost((void *)h_in);
  }
  static void destroy(sfft::StageEvents *e) {
    for (int i = 0; i < 8; i++) cudaEventDestroy(e->ev[i]);
    delete e;
  }
  sfft::StageEvents *take_set() {
    sfft::StageEvents *e;
    if (!free_sets.empty()) {
      e = free_sets.back();
      free_sets.pop_back();
    } else {
      e = new sfft::StageEvents();
      for (int i = 0; i < 8; i++) cudaEventCreate(&e->ev[i]);
    }
    e->recorded = 0;
    return e;
  }
  void harvest() {
    while (!pending.empty()) {
      sfft::StageEvents *e = pending.front();
      pending.pop_front();
      if (e->recorded > 0 && cudaEventSynchronize(e->ev[e->recorded - 1]) == cudaSuccess) {
        for (int i = 0; i + 1 < e->recorded; i++) {
          float ms = 0;
          if (cudaEventElapsedTime(&ms, e->ev[i], e->ev[i + 1]) == cudaSuccess) stage_ms[i] += ms;
        }
        profiled++;
      }
      free_sets.push_back(e);
    }
  }
};

namespace {

int L12(const PlanImpl &P) { return P.p12.loops_loc + P.p12.loops_est; }

// Bucket layout of a v1/v2 plan's x_samp (V12Dev::xs_perm): grouped by comb
// residue for plain v2 (FP32 or FP64) whose comb width W is a multiple of
// both n / B and that has at least 32 candidates per residue; natural (0)
// otherwise.
int xs_perm_of(const PlanImpl &P) {
  const auto &p = P.p12;
  if (P.version != 1 || P.voted || P.large_b || p.W_Comb <= 0) return 0;
  const long ql = P.n / p.B_loc, qe = P.n / p.B_est, R = P.n / p.W_Comb;
  if (p.W_Comb % ql || p.W_Comb % qe || R < 32) return 0;
  return ilog2(std::min<long>(R, 256));
}

// Position of bucket b of a loop of B buckets in the grouped layout.
long xs_position(long b, long B, int lg) {
  if (!lg) return b;
  const int lt = ilog2(B) - lg;
  return ((b & ((1L << lt) - 1)) << lg) | (b >> lt);
}

// ------------------------------------------------------------- constants --

bool upload_twiddles(DBuf &b, long N, int prec) {
  const std::vector<double> &tw = sfft::fft_twiddles(N);
  std::vector<double> t(tw.begin(), tw.begin() + 2 * N);
  if (prec == sfft::PREC_FP64) return b.upload(t);
  return b.upload(to_f32(t));
}

// Plan-time FFTs of power-of-two length n >= 2^15 on the plan's device.
// The global-memory Stockham stages perform exactly host_fft's operations
// (the backward transform conjugates on the host around a forward one), so
// the filters built this way are bit-identical to the host's; on any CUDA
// failure the host FFT runs instead.
bool device_fft(long n, double *data, int sign, void *ctx) {
  if (n < (1L << 15) || (n & (n - 1))) return false;
  const int dev = *(const int *)ctx;
  if (cudaSetDevice(dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const std::vector<double> &tw = sfft::fft_twiddles(n);
  const size_t bytes = sizeof(double) * 2 * (size_t)n;
  void *a = nullptr, *b = nullptr, *t = nullptr;
  cudaStream_t s = nullptr;
  auto conj = [&] {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) data[2 * i + 1] = -data[2 * i + 1];
  };
  bool good = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&a, bytes) == cudaSuccess && cudaMalloc(&b, bytes) == cudaSuccess &&
              cudaMalloc(&t, bytes) == cudaSuccess;
  if (good) {
    std::vector<double> out(2 * (size_t)n);  // data stays intact until success
    if (sign > 0) conj();
    good = cudaMemcpyAsync(a, data, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess &&
           cudaMemcpyAsync(t, tw.data(), bytes, cudaMemcpyHostToDevice, s) == cudaSuccess &&
           sfft::global_fft_c128(a, b, (int)n, 1, n, n, 1, t, s) == cudaSuccess &&
           cudaMemcpyAsync(out.data(), a, bytes, cudaMemcpyDeviceToHost, s) == cudaSuccess;
    good = cudaStreamSynchronize(s) == cudaSuccess && good;
    if (good) std::memcpy(data, out.data(), bytes);
    if (sign > 0) conj();
  }
  cudaGetLastError();
  if (a) cudaFree(a);
  if (b) cudaFree(b);
  if (t) cudaFree(t);
  if (s) cudaStreamDestroy(s);
  return good;
}

// Estimation window of a v1/v2 filter: the q = n/B entries of filter.freq
// that src/computefourier-1.0-2.0.cc:370-385 can index, win[m] =
// freq[(n - d) % n] with d = m - (q-1)/2.
bool upload_v12_window(DBuf &b, const std::vector<double> &freq, int n, int q, int prec) {
  if (prec == sfft::PREC_FP64) {
    std::vector<double> w(4 * (size_t)q);
    for (int m = 0; m < q; m++) {
      const long d = m - (q - 1) / 2;
      const long idx = ((long)n - d) % n;
      const double c = freq[2 * idx], dd = freq[2 * idx + 1];
      w[4 * m] = c;
      w[4 * m + 1] = dd;
      w[4 * m + 2] = c * c + dd * dd;  // same rounding as the reference's hadd
      w[4 * m + 3] = 0.0;
    }
    return b.upload(w);
  }
  std::vector<float> w(2 * (size_t)q);
  for (int m = 0; m < q; m++) {
    const long d = m - (q - 1) / 2;
    const long idx = ((long)n - d) % n;
    const double c = freq[2 * idx], dd = freq[2 * idx + 1];
    const double den = c * c + dd * dd;
    w[2 * m] = (float)(c / den);
    w[2 * m + 1] = (float)(dd / den);
  }
  return b.upload(w);
}

// v3 window: freq[(m - half) mod n] for m in [0, 2*half].
bool upload_v3_window(DBuf &b, const std::vector<double> &freq, int n, int half) {
  std::vector<double> w(2 * (size_t)(2 * half + 1));
  for (int m = 0; m <= 2 * half; m++) {
    const long idx = (((long)m - half) % n + n) % n;
    w[2 * m] = freq[2 * idx];
    w[2 * m + 1] = freq[2 * idx + 1];
  }
  return b.upload(w);
}

bool upload_taps(DBuf &b, const std::vector<double> &t, int prec) {
  if (prec == sfft::PREC_FP64) return b.upload(t);
  return b.upload(to_f32(t));
}

// ------------------------------------------------------------- workspace --

bool ensure_slots(PlanImpl &P, int want) {
  if (want <= P.slots) return true;
  const size_t S = (size_t)want;
  const size_t cs = P.prec == sfft::PREC_FP64 ? 16 : 8;
  if (!P.counters.ensure(sizeof(int) * sfft::CNT_STRIDE * S)) return false;
  if (!P.inputs.ensure(sizeof(void *) * S) || !P.dense_ptrs.ensure(sizeof(void *) * S)) return false;
  if (P.version < 2) {
    const auto &p = P.p12;
    const int L = L12(P);
    P.rp_stride = 2 * L + p.Comb_loops + 1;
    const int q = P.n / p.B_loc;
    P.hit_cap = P.version == 0
                    ? (int)std::min<long>((long)P.n, ((long)p.loops_loc * p.B_thresh * q) / p.loops_thresh + 1)
                    : 1;
    const long comb_max = std::min<long>((long)p.W_Comb, (long)p.Comb_loops * p.B_thresh);
    P.out_cap = P.version == 0 ? P.hit_cap : (int)(comb_max * (P.n / p.W_Comb));
    if (P.voted) {
      // voted v2: a candidate needs `thresh` votes; at most min(comb
      // candidates, loc_loops * 2k * n/B / thresh) can reach it.  Besides
      // the k tones, a comb candidate that is no tone lies in one of the 2k
      // selected buckets of a location loop with probability 2k / B, so
      // about (comb candidates) * P[Binomial(loops, 2k / B) >= thresh] pass
      // by chance -- a handful with the reference's constants, a large
      // share when the constants make B small against 2k.  The list holds
      // four times that expectation plus 8 * 2k (at least 65536); a longer
      // one sets ERR_HIT_OVERFLOW and the execution reports an error
      // (nothing is dropped silently).
      const long vote_max = ((long)p.loops_loc * p.B_thresh * q) / p.loops_thresh + 1;
      const double pv = std::min(1.0, (double)p.B_thresh / p.B_loc);
      double tail = 0.0;
      for (int v = p.loops_thresh; v <= p.loops_loc; v++) {
        double c = 1.0;  // binomial coefficient C(loops_loc, v)
        for (int t = 0; t < v; t++) c = c * (p.loops_loc - t) / (t + 1);
        tail += c * std::pow(pv, v) * std::pow(1.0 - pv, p.loops_loc - v);
      }
      const double expect = tail * (double)P.out_cap;
      const long want = std::max<long>(65536, (long)std::min(4.0 * expect, 4e9) + 8L * p.B_thresh);
      P.hit_cap = (int)std::min<long>(std::min<long>((long)P.out_cap, vote_max), want);
      P.out_cap = P.hit_cap;
    }
    if (P.prec == sfft::PREC_FP64 && !P.xs32.ensure(8 * p.x_samp_size * S)) return false;
    if (P.large_b && !P.xs_tmp.ensure(cs * p.x_samp_size * S)) return false;
    if (P.large_c && (!P.comb_buf.ensure(cs * (size_t)p.Comb_loops * p.W_Comb * S) ||
                      !P.comb_tmp.ensure(cs * (size_t)p.Comb_loops * p.W_Comb * S)))
      return false;
    if (!P.xs.ensure(cs * p.x_samp_size * S) || !P.J.ensure(sizeof(int) * L * p.B_thresh * S) ||
        !P.hits.ensure(sizeof(int) * P.hit_cap * S) ||
        !P.comb_bits.ensure(sizeof(unsigned) * ((p.W_Comb + 31) / 32) * S) ||
        !P.comb_list.ensure(sizeof(int) * p.W_Comb * S) || !P.out_idx.ensure(sizeof(int) * P.out_cap * S) ||
        !P.out_val.ensure(cs * P.out_cap * S))
      return false;
    // vote counters persist across execs (epoch-tagged); grow by copy-free realloc
    DBuf fresh;
    if (!fresh.ensure(sizeof(unsigned) * (size_t)P.n * S)) return false;
    if (!cuda_ok(cudaMemset(fresh.p, 0, sizeof(unsigned) * (size_t)P.n * S), "memset")) return false;
    std::swap(P.score.p, fresh.p);
    std::swap(P.score.bytes, fresh.bytes);
    P.epoch.assign(S, 0);
  } else {
    const auto &p = P.p3;
    P.rp_stride = 5;
    P.est_cap = std::max(p.W_Man, std::max(p.B_g1, p.B_g2));
    P.map_cap = 4 * (p.W_Man + p.B_g1 + p.B_g2) + 8 * P.k;
    P.table_cap = 1;
    while (P.table_cap < 2 * P.map_cap) P.table_cap <<= 1;
    P.out_cap = P.map_cap;
    if (!P.perm.ensure(16 * 2 * (size_t)(p.w_g2 + 2) * S)) return false;
    if ((p.W_Man > sfft::v3_max_smem_fft() || sfft::v3_man_split(p.W_Man)) &&
        !P.man_tmp.ensure(64 * (size_t)p.W_Man * S))
      return false;
    if (!P.man.ensure(32 * (size_t)p.W_Man * S) || !P.g1.ensure(32 * (size_t)p.B_g1 * S) ||
        !P.g2.ensure(32 * (size_t)p.B_g2 * S) || !P.est_f.ensure(sizeof(int) * P.est_cap * S) ||
        !P.est_v.ensure(16 * (size_t)P.est_cap * S) || !P.map_keys.ensure(sizeof(int) * P.table_cap * S) ||
        !P.map_vals.ensure(16 * (size_t)P.table_cap * S) || !P.map_list.ensure(sizeof(int) * P.map_cap * S) ||
        !P.out_idx.ensure(sizeof(int) * P.out_cap * S) || !P.out_val.ensure(16 * (size_t)P.out_cap * S) ||
        !P.trace.ensure(sizeof(double) * 5 * (size_t)P.map_cap))
      return false;
  }
  if (!P.rparams.ensure(sizeof(int) * P.rp_stride * S)) return false;
  P.slots = want;
  return true;
}

// ------------------------------------------------------------------ RNG --

// Source of the reference's random numbers: glibc's global random() /
// drand48() streams (what sfft_exec uses, like the reference), or private
// reentrant copies seeded per transform (random_r / drand48_r with the
// state srandom(seed) / srand48(seed) would give), so that a transform's
// draws do not depend on what else runs.
struct Rng {
  bool seeded = false;
  struct random_data rd;
  char state[128];
  struct drand48_data dd;
  void seed(unsigned s) {
    seeded = true;
    std::memset(&rd, 0, sizeof rd);
    std::memset(state, 0, sizeof state);
    initstate_r(s, state, sizeof state, &rd);
    srand48_r((long)s, &dd);
  }
  long rnd() {
    if (!seeded) return random();
    int32_t r;
    random_r(&rd, &r);
    return r;
  }
  double d48() {
    if (!seeded) return drand48();
    double x;
    drand48_r(&dd, &x);
    return x;
  }
};

// Draws of one transform, in the reference's order.
void draw_params(const PlanImpl &P, int *rp, unsigned epoch, Rng &g) {
  const int n = P.n;
  if (P.version < 2) {
    const int L = L12(P);
    for (int i = 0; i < L; i++) {  // src/computefourier-1.0-2.0.cc:465-474
      int a = 0;
      while (gcd_ref(a, n) != 1) a = (int)(g.rnd() % n);
      rp[i] = a;
      rp[L + i] = mod_inverse_ref(a, n);
    }
    for (int c = 0; c < P.p12.Comb_loops; c++) {  // :62, once per Comb_Filt call
      if (P.version == 1) {
        const int sigma = n / P.p12.W_Comb;
        rp[2 * L + c] = (int)(unsigned)std::floor(g.d48() * sigma);
      } else {
        rp[2 * L + c] = 0;
      }
    }
    rp[2 * L + P.p12.Comb_loops] = (int)epoch;
  } else {  // src/computefourier-3.0.cc:800-810
    int a = 0;
    while (gcd_ref(a, n) != 1) a = (int)(g.rnd() % n);
    rp[0] = a;
    rp[1] = mod_inverse_ref(a, n);
    rp[2] = (int)(g.rnd() % n);
    rp[3] = (int)(unsigned)std::floor(g.d48() * n);
    rp[4] = (int)(unsigned)std::floor(g.d48() * n);
  }
}

void draw_params(const PlanImpl &P, int *rp, unsigned epoch) {
  Rng g;
  draw_params(P, rp, epoch, g);
}

// ---------------------------------------------------------------- launch --

sfft::V12Dev v12_view(PlanImpl &P) {
  sfft::V12Dev d{};
  const auto &p = P.p12;
  d.version = P.version;
  d.prec = P.prec;
  d.n = P.n;
  d.logn = ilog2(P.n);
  d.k = P.k;
  d.num = p.B_thresh;
  d.B_loc = p.B_loc;
  d.B_est = p.B_est;
  d.L_loc = p.loops_loc;
  d.L_est = p.loops_est;
  d.L = L12(P);
  d.thresh = p.loops_thresh;
  d.W = p.W_Comb;
  d.comb_loops = p.Comb_loops;
  d.w_loc = p.w_loc;
  d.w_est = p.w_est;
  d.q_loc = P.n / p.B_loc;
  d.q_est = P.n / p.B_est;
  d.xs_size = p.x_samp_size;
  d.taps_loc = P.taps_a.p;
  d.taps_est = P.taps_b.p;
  d.win_loc = P.win_a.p;
  d.win_est = P.win_b.p;
  d.tw_loc = P.tw_a.p;
  d.tw_est = P.tw_b.p;
  d.tw_comb = P.tw_c.p;
  d.xs = P.xs.p;
  d.xs32 = P.prec == sfft::PREC_FP64 ? P.xs32.p : nullptr;
  d.xs_tmp = P.xs_tmp.p;
  d.comb_buf = P.comb_buf.p;
  d.comb_tmp = P.comb_tmp.p;
  d.large_buckets = P.large_b;
  d.large_comb = P.large_c;
  d.win32_loc = P.win32_a.p;
  d.win32_est = P.win32_b.p;
  d.J = P.J.as<int>();
  d.score = P.score.as<unsigned>();
  d.hits = P.hits.as<int>();
  d.comb_bits = P.comb_bits.as<unsigned>();
  d.comb_list = P.comb_list.as<int>();
  d.counters = P.counters.as<int>();
  d.out_idx = P.out_idx.as<int>();
  d.out_val = P.out_val.p;
  d.out_count = nullptr;
  d.hit_cap = P.hit_cap;
  d.out_cap = P.out_cap;
  d.voted = P.voted;
  d.xs_perm = xs_perm_of(P);

  d.out_stride = P.out_cap;
  d.rparams = P.rparams.as<int>();
  d.rp_stride = P.rp_stride;
  d.inputs = (const void *const *)P.inputs.p;
  return d;
}

sfft::V3Dev v3_view(PlanImpl &P) {
  sfft::V3Dev d{};
  const auto &p = P.p3;
  d.prec = sfft::PREC_FP64;
  d.n = P.n;
  d.logn = ilog2(P.n);
  d.k = P.k;
  d.W = p.W_Man;
  d.B1 = p.B_g1;
  d.B2 = p.B_g2;
  d.w1 = p.w_g1;
  d.w2 = p.w_g2;
  d.q1 = P.n / p.B_g1;
  d.q2 = P.n / p.B_g2;
  d.win1_half = P.win_half_a;
  d.win2_half = P.win_half_b;
  d.taps1 = P.taps_a.p;
  d.taps2 = P.taps_b.p;
  d.win1 = P.win_a.p;
  d.win2 = P.win_b.p;
  d.tw_man = P.tw_c.p;
  d.tw_g1 = P.tw_a.p;
  d.tw_g2 = P.tw_b.p;
  d.man = P.man.p;
  d.man_tmp = P.man_tmp.p;
  d.large_man = p.W_Man > sfft::v3_max_smem_fft();
  d.g1 = P.g1.p;
  d.g2 = P.g2.p;
  d.perm = P.perm.p;
  d.est_f = P.est_f.as<int>();
  d.est_v = P.est_v.p;
  d.map_keys = P.map_keys.as<int>();
  d.map_vals = P.map_vals.p;
  d.map_table = P.map_list.as<int>();
  d.est_cap = P.est_cap;
  d.map_cap = P.map_cap;
  d.table_cap = P.table_cap;
  d.counters = P.counters.as<int>();
  d.out_idx = P.out_idx.as<int>();
  d.out_val = P.out_val.p;
  d.out_count = nullptr;
  d.out_cap = P.out_cap;
  d.out_stride = P.out_cap;
  d.max_passes = 3000;
  d.trace = P.trace.as<double>();
  d.trace_cap = P.map_cap;
  d.rparams = P.rparams.as<int>();
  d.rp_stride = P.rp_stride;
  d.inputs = (const void *const *)P.inputs.p;
  return d;
}

// Where a launch writes its sparse results (default: the plan's buffers).
struct OutTarget {
  int *idx;
  void *val;
  int *count;
  long stride;
};

// Uploads draws and input pointers for `num` slots and runs the pipeline.
template <typename T>
void shift(T *&p, size_t per_slot, int base) {
  if (p) p = (T *)((char *)p + per_slot * (size_t)base);
}

// Moves every per-slot pointer of a view to slot `base` (double-buffered
// pipelines use slots [base, base + num)).
void shift_view(PlanImpl &P, sfft::V12Dev &d, int base, bool own_out) {
  if (!base) return;
  const size_t cs = P.prec == sfft::PREC_FP64 ? 16 : 8;
  shift(d.xs, cs * d.xs_size, base);
  shift(d.xs32, 8 * d.xs_size, base);
  shift(d.xs_tmp, cs * d.xs_size, base);
  shift(d.comb_buf, cs * (size_t)d.comb_loops * d.W, base);
  shift(d.comb_tmp, cs * (size_t)d.comb_loops * d.W, base);
  shift(d.J, sizeof(int) * (size_t)d.L * d.num, base);
  shift(d.score, sizeof(unsigned) * (size_t)d.n, base);
  shift(d.hits, sizeof(int) * (size_t)d.hit_cap, base);
  shift(d.comb_bits, sizeof(unsigned) * (size_t)((d.W + 31) / 32), base);
  shift(d.comb_list, sizeof(int) * (size_t)d.W, base);
  shift(d.counters, sizeof(int) * sfft::CNT_STRIDE, base);
  if (own_out) {
    shift(d.out_idx, sizeof(int) * (size_t)d.out_cap, base);
    shift(d.out_val, cs * (size_t)d.out_cap, base);
  }
  shift(d.rparams, sizeof(int) * (size_t)d.rp_stride, base);
  shift(d.inputs, sizeof(void *), base);
}

void shift_view(PlanImpl &P, sfft::V3Dev &d, int base, bool own_out) {
  if (!base) return;
  shift(d.man, 32 * (size_t)d.W, base);
  if (d.large_man || sfft::v3_man_split(d.W)) shift(d.man_tmp, 64 * (size_t)d.W, base);
  shift(d.g1, 32 * (size_t)d.B1, base);
  shift(d.g2, 32 * (size_t)d.B2, base);
  shift(d.perm, 16 * 2 * (size_t)(d.w2 + 2), base);
  shift(d.est_f, sizeof(int) * (size_t)d.est_cap, base);
  shift(d.est_v, 16 * (size_t)d.est_cap, base);
  shift(d.map_keys, sizeof(int) * (size_t)d.table_cap, base);
  shift(d.map_vals, 16 * (size_t)d.table_cap, base);
  shift(d.map_table, sizeof(int) * (size_t)d.map_cap, base);
  shift(d.counters, sizeof(int) * sfft::CNT_STRIDE, base);
  if (own_out) {
    shift(d.out_idx, sizeof(int) * (size_t)d.out_cap, base);
    shift(d.out_val, 16 * (size_t)d.out_cap, base);
  }
  shift(d.rparams, sizeof(int) * (size_t)d.rp_stride, base);
  shift(d.inputs, sizeof(void *), base);
  d.trace = nullptr;
  (void)P;
}

bool launch(PlanImpl &P, int num, const void *const *in_dev, int in_type, cudaStream_t s,
            const OutTarget *tgt = nullptr, int base = 0, const unsigned *seeds = nullptr) {
  std::vector<int> rp((size_t)P.rp_stride * num);
  for (int i = 0; i < num; i++) {
    unsigned ep = 0;
    if (P.version < 2) {
      const int sl = base + i;
      if (++P.epoch[sl] >= (1u << 24)) {  // wrap: clear this slot's vote counters
        if (!cuda_ok(cudaMemsetAsync(P.score.as<unsigned>() + (size_t)sl * P.n, 0, sizeof(unsigned) * P.n, s),
                     "memset"))
          return false;
        P.epoch[sl] = 1;
      }
      ep = P.epoch[sl];
    }
    Rng g;
    if (seeds) g.seed(seeds[i]);
    draw_params(P, &rp[(size_t)i * P.rp_stride], ep, g);
  }
  if (base == 0) P.last_rp.assign(rp.begin(), rp.begin() + P.rp_stride);
  // pageable sources: the runtime stages them before returning
  if (!cuda_ok(cudaMemcpyAsync(P.rparams.as<int>() + (size_t)base * P.rp_stride, rp.data(), sizeof(int) * rp.size(),
                               cudaMemcpyHostToDevice, s),
               "params upload"))
    return false;
  std::vector<const void *> ptrs(in_dev, in_dev + num);
  if (!cuda_ok(cudaMemcpyAsync((const void **)P.inputs.p + base, ptrs.data(), sizeof(void *) * num,
                               cudaMemcpyHostToDevice, s),
               "pointer upload"))
    return false;
  sfft::StageEvents *se = P.profiling ? P.take_set() : nullptr;
  bool ok;
  if (P.version < 2) {
    sfft::V12Dev d = v12_view(P);
    shift_view(P, d, base, tgt == nullptr);
    d.in_type = in_type;
    if (tgt) {
      d.out_idx = tgt->idx;
      d.out_val = tgt->val;
      d.out_count = tgt->count;
      d.out_stride = tgt->stride;
    }
    ok = cuda_ok(sfft::v12_run(d, num, s, se), "v1/v2 launch");
  } else {
    sfft::V3Dev d = v3_view(P);
    shift_view(P, d, base, tgt == nullptr);
    d.in_type = in_type;
    if (tgt) {
      d.out_idx = tgt->idx;
      d.out_val = tgt->val;
      d.out_count = tgt->count;
      d.out_stride = tgt->stride;
    }
    ok = cuda_ok(sfft::v3_run(d, num, s, se), "v3 launch");
  }
  if (se) P.pending.push_back(se);
  return ok;
}

// Error bits of `num` signals' counters (CNT_STRIDE ints each, host copy).
bool check_counts(const int *cnt, int num) {
  for (int i = 0; i < num; i++) {
    const int e = cnt[(size_t)i * sfft::CNT_STRIDE + sfft::CNT_ERR];
    if (e) {
      char buf[160];
      std::snprintf(buf, sizeof buf, "device reported error bits 0x%x on signal %d (1 hits, 2 output, 4 v3 no fixpoint, 8 v3 capacity, 16 copy wait timed out)",
                    e, i);
      set_err(buf);
      return false;
    }
  }
  return true;
}

bool check_device_errors(PlanImpl &P, int num, int base = 0) {
  std::vector<int> cnt((size_t)sfft::CNT_STRIDE * num);
  if (!cuda_ok(cudaMemcpy(cnt.data(), P.counters.as<int>() + (size_t)base * sfft::CNT_STRIDE, sizeof(int) * cnt.size(),
                          cudaMemcpyDeviceToHost),
               "counters"))
    return false;
  return check_counts(cnt.data(), num);
}

bool is_device_ptr(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

std::mutex g_alloc_mu;
std::set<void *> g_pinned;

PlanImpl *impl(sfft_plan *p) { return p ? (PlanImpl *)p->data : nullptr; }

// Runs `num` (<= slots) transforms whose inputs are host or device
// pointers and writes dense n-point outputs (host or device).
bool exec_dense_chunk(PlanImpl &P, int num, complex_t **in, complex_t **out) {
  cudaStream_t s = P.stream;
  const size_t nb = sizeof(double) * 2 * (size_t)P.n;
  std::vector<const void *> dev_in(num);
  bool need_in_stage = false, need_out_stage = false;
  for (int i = 0; i < num; i++) {
    if (!is_device_ptr(in[i])) need_in_stage = true;
    if (!is_device_ptr(out[i])) need_out_stage = true;
  }
  if (need_in_stage && !P.in_stage.ensure(nb * P.slots)) return false;
  if (need_out_stage && !P.dense_stage.ensure(nb * P.slots)) return false;
  for (int i = 0; i < num; i++) {
    if (is_device_ptr(in[i])) {
      dev_in[i] = in[i];
    } else {
      void *dst = (char *)P.in_stage.p + nb * i;
      if (!cuda_ok(cudaMemcpyAsync(dst, in[i], nb, cudaMemcpyHostToDevice, s), "input copy")) return false;
      dev_in[i] = dst;
    }
  }
  if (!launch(P, num, dev_in.data(), sfft::IN_C128, s)) return false;
  std::vector<void *> dense(num);
  for (int i = 0; i < num; i++) {
    dense[i] = is_device_ptr(out[i]) ? (void *)out[i] : (char *)P.dense_stage.p + nb * i;
    if (!cuda_ok(cudaMemsetAsync(dense[i], 0, nb, s), "output clear")) return false;
  }
  if (!cuda_ok(cudaMemcpyAsync(P.dense_ptrs.p, dense.data(), sizeof(void *) * num, cudaMemcpyHostToDevice, s),
               "pointer upload"))
    return false;
  if (!cuda_ok(sfft::scatter_dense(P.out_idx.as<int>(), P.out_val.p, P.version < 2 ? P.prec : sfft::PREC_FP64,
                                   P.counters.as<int>(), P.out_cap, (void *const *)P.dense_ptrs.p, num, s),
               "scatter"))
    return false;
  for (int i = 0; i < num; i++)
    if (!is_device_ptr(out[i]) &&
        !cuda_ok(cudaMemcpyAsync(out[i], dense[i], nb, cudaMemcpyDeviceToHost, s), "output copy"))
      return false;
  if (!cuda_ok(cudaStreamSynchronize(s), "exec")) return false;
  return check_device_errors(P, num);
}

// sfft_exec_many on host buffers: chunk c's input copies (copy_in), its
// transform (plan stream) and its dense output copies (copy_out) overlap
// with the neighbouring chunks; workspace, input staging and dense staging
// are double-buffered (slot halves [0, chunk) and [chunk, 2 chunk)).  Each
// chunk's counters are stashed on the device (a kernel, no copy engine) and
// read once at the end: a blocking per-chunk read would queue behind the
// large output copies and keep the host from issuing the next input copies,
// serialising the two directions.
bool exec_dense_pipelined(PlanImpl &P, int num, complex_t **in, complex_t **out, int chunk) {
  const size_t nb = sizeof(double) * 2 * (size_t)P.n;
  if (!ensure_slots(P, 2 * chunk)) return false;
  if (!P.in_stage.ensure(nb * 2 * chunk) || !P.dense_stage.ensure(nb * 2 * chunk) ||
      !P.dense_ptrs.ensure(sizeof(void *) * 2 * chunk) ||
      !P.cnt_stash.ensure(sizeof(int) * sfft::CNT_STRIDE * (size_t)num))
    return false;
  cudaStream_t s = P.stream;
  const int nchunks = (num + chunk - 1) / chunk;
  for (int c = 0; c < nchunks; c++) {
    const int half = c & 1, base = half * chunk, i0 = c * chunk, m = std::min(chunk, num - i0);
    char *istage = (char *)P.in_stage.p + nb * base;
    char *ostage = (char *)P.dense_stage.p + nb * base;
    // inputs of chunk c may overwrite this half once chunk c-2's transform has read it
    if (c >= 2 && !cuda_ok(cudaStreamWaitEvent(P.copy_in, P.ev_comp[half], 0), "wait")) return false;
    for (int i = 0; i < m; i++)
      if (!cuda_ok(cudaMemcpyAsync(istage + nb * i, in[i0 + i], nb, cudaMemcpyHostToDevice, P.copy_in), "input copy"))
        return false;
    if (!cuda_ok(cudaEventRecord(P.ev_in[half], P.copy_in), "event")) return false;
    if (!cuda_ok(cudaStreamWaitEvent(s, P.ev_in[half], 0), "wait")) return false;
    // the dense staging of this half is free once chunk c-2's output copies finished
    if (c >= 2 && !cuda_ok(cudaStreamWaitEvent(s, P.ev_out[half], 0), "wait")) return false;
    std::vector<const void *> dev_in(m);
    std::vector<void *> dense(m);
    for (int i = 0; i < m; i++) {
      dev_in[i] = istage + nb * i;
      dense[i] = ostage + nb * i;
    }
    if (!launch(P, m, dev_in.data(), sfft::IN_C128, s, nullptr, base)) return false;
    if (!cuda_ok(cudaMemsetAsync(ostage, 0, nb * m, s), "output clear")) return false;
    if (!cuda_ok(cudaMemcpyAsync((void **)P.dense_ptrs.p + base, dense.data(), sizeof(void *) * m,
                                 cudaMemcpyHostToDevice, s),
                 "pointer upload"))
      return false;
    const size_t cs = (P.version < 2 && P.prec == sfft::PREC_FP32) ? 8 : 16;
    if (!cuda_ok(sfft::scatter_dense(P.out_idx.as<int>() + (size_t)base * P.out_cap,
                                     (char *)P.out_val.p + cs * (size_t)base * P.out_cap,
                                     P.version < 2 ? P.prec : sfft::PREC_FP64,
                                     P.counters.as<int>() + (size_t)base * sfft::CNT_STRIDE, P.out_cap,
                                     (void *const *)P.dense_ptrs.p + base, m, s),
                 "scatter"))
      return false;
    if (!cuda_ok(sfft::copy_ints(P.counters.as<int>() + (size_t)base * sfft::CNT_STRIDE,
                                 P.cnt_stash.as<int>() + (size_t)i0 * sfft::CNT_STRIDE, sfft::CNT_STRIDE * m, s),
                 "counter stash"))
      return false;
    if (!cuda_ok(cudaEventRecord(P.ev_comp[half], s), "event")) return false;
    if (!cuda_ok(cudaStreamWaitEvent(P.copy_out, P.ev_comp[half], 0), "wait")) return false;
    for (int i = 0; i < m; i++)
      if (!cuda_ok(cudaMemcpyAsync(out[i0 + i], ostage + nb * i, nb, cudaMemcpyDeviceToHost, P.copy_out),
                   "output copy"))
        return false;
    if (!cuda_ok(cudaEventRecord(P.ev_out[half], P.copy_out), "event")) return false;
    if (c >= 1) {  // the host runs at most about one chunk ahead of the device
      if (!cuda_ok(cudaEventSynchronize(P.ev_comp[(c - 1) & 1]), "sync")) return false;
    }
  }
  if (!cuda_ok(cudaStreamSynchronize(P.copy_out), "sync") || !cuda_ok(cudaStreamSynchronize(s), "sync")) return false;
  std::vector<int> cnt((size_t)sfft::CNT_STRIDE * num);
  if (!cuda_ok(cudaMemcpy(cnt.data(), P.cnt_stash.p, sizeof(int) * cnt.size(), cudaMemcpyDeviceToHost), "counters"))
    return false;
  return check_counts(cnt.data(), num);
}

// sfft_exec_many with sparse results: like exec_dense_pipelined, chunk c's
// input copies (copy_in) and transform (plan stream) overlap the
// neighbouring chunks; once chunk c-1's transform is done its counts are
// read and exactly that many (index, value) pairs are copied out on
// copy_out.  Values keep the plan's type (complex64 for FP32 v1/v2).
bool exec_sparse_pipelined(PlanImpl &P, int num, const complex_t *const *in, int *out_idx, void *out_val,
                           int *out_count, long out_stride, int chunk) {
  const size_t nb = sizeof(double) * 2 * (size_t)P.n;
  if (!ensure_slots(P, 2 * chunk)) return false;
  if (!P.in_stage.ensure(nb * 2 * chunk)) return false;
  cudaStream_t s = P.stream;
  const size_t cs = (P.version < 2 && P.prec == sfft::PREC_FP32) ? 8 : 16;
  const bool dev_out = is_device_ptr(out_idx);
  const cudaMemcpyKind kind = dev_out ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  const int nchunks = (num + chunk - 1) / chunk;
  std::vector<int> cnt((size_t)sfft::CNT_STRIDE * chunk);
  // results of chunk c (slot half c & 1): wait for its transform, check it,
  // copy its counts and pairs out
  auto drain = [&](int c) -> bool {
    const int half = c & 1, base = half * chunk, i0 = c * chunk, m = std::min(chunk, num - i0);
    if (!cuda_ok(cudaEventSynchronize(P.ev_comp[half]), "sync")) return false;
    if (!cuda_ok(cudaMemcpy(cnt.data(), P.counters.as<int>() + (size_t)base * sfft::CNT_STRIDE,
                            sizeof(int) * sfft::CNT_STRIDE * m, cudaMemcpyDeviceToHost),
                 "counts"))
      return false;
    for (int i = 0; i < m; i++) {
      const int *ci = &cnt[(size_t)i * sfft::CNT_STRIDE];
      if (ci[sfft::CNT_ERR]) return check_device_errors(P, m, base);
      const long c_out = ci[sfft::CNT_OUT];
      if (c_out > out_stride) {
        set_err("out_stride below the result count (" + std::to_string(c_out) + ")");
        return false;
      }
      out_count[i0 + i] = (int)c_out;
      const size_t src = (size_t)(base + i) * P.out_cap, dst = (size_t)(i0 + i) * out_stride;
      if (!cuda_ok(cudaMemcpyAsync(out_idx + dst, P.out_idx.as<int>() + src, sizeof(int) * c_out, kind, P.copy_out),
                   "index copy") ||
          !cuda_ok(cudaMemcpyAsync((char *)out_val + cs * dst, (char *)P.out_val.p + cs * src, cs * c_out, kind,
                                   P.copy_out),
                   "value copy"))
        return false;
    }
    return cuda_ok(cudaEventRecord(P.ev_out[half], P.copy_out), "event");
  };
  for (int c = 0; c < nchunks; c++) {
    const int half = c & 1, base = half * chunk, i0 = c * chunk, m = std::min(chunk, num - i0);
    char *istage = (char *)P.in_stage.p + nb * base;
    // inputs of chunk c may overwrite this half once chunk c-2's transform has read it
    if (c >= 2 && !cuda_ok(cudaStreamWaitEvent(P.copy_in, P.ev_comp[half], 0), "wait")) return false;
    for (int i = 0; i < m; i++)
      if (!cuda_ok(cudaMemcpyAsync(istage + nb * i, in[i0 + i], nb, cudaMemcpyHostToDevice, P.copy_in), "input copy"))
        return false;
    if (!cuda_ok(cudaEventRecord(P.ev_in[half], P.copy_in), "event")) return false;
    if (!cuda_ok(cudaStreamWaitEvent(s, P.ev_in[half], 0), "wait")) return false;
    // this half's sparse outputs are free once chunk c-2's copies finished
    if (c >= 2 && !cuda_ok(cudaStreamWaitEvent(s, P.ev_out[half], 0), "wait")) return false;
    std::vector<const void *> dev_in(m);
    for (int i = 0; i < m; i++) dev_in[i] = istage + nb * i;
    if (!launch(P, m, dev_in.data(), sfft::IN_C128, s, nullptr, base)) return false;
    if (!cuda_ok(cudaEventRecord(P.ev_comp[half], s), "event")) return false;
    if (c >= 1 && !drain(c - 1)) return false;
  }
  if (!drain(nchunks - 1)) return false;
  return cuda_ok(cudaStreamSynchronize(P.copy_out), "sync") && cuda_ok(cudaStreamSynchronize(s), "sync");
}

}  // namespace

namespace sfft {

// For entry points that bring their own workspace: the plan's constants
// and sizes (workspace pointers of the view are the plan's and must be
// replaced by the caller).  Returns false for plans other than v1/v2.
bool plan_v12_constants(sfft_plan *plan, V12Dev *d, int *hit_cap, int *out_cap) {
  PlanImpl *P = impl(plan);
  if (!P || P->version > 1) return false;
  *d = v12_view(*P);
  *hit_cap = P->hit_cap;
  *out_cap = P->out_cap;
  return true;
}

// The random draws of one transform, in the reference's order.
void plan_draw(sfft_plan *plan, int *rp, unsigned epoch) { draw_params(*impl(plan), rp, epoch); }

int plan_device(sfft_plan *plan) { return impl(plan)->device; }

// Device counters of the plan's batch slots (CNT_STRIDE ints per slot),
// rewritten by every execution.
const int *plan_counters(sfft_plan *plan) { return impl(plan)->counters.as<int>(); }

void set_last_error(const char *m) { set_err(m); }

// ----------------------------------------------- graph-capturable launches

bool plan_enable_staging(sfft_plan *plan, int slots) {
  PlanImpl *P = impl(plan);
  if (!P) return false;
  std::lock_guard<std::mutex> g(P->mu);
  cudaSetDevice(P->device);
  if (!ensure_slots(*P, slots)) return false;
  if (P->staged_slots >= slots) return true;
  if (P->h_rp) cudaFreeHost(P->h_rp);
  if (P->h_in) cudaFreeHost((void *)P->h_in);
  P->h_rp = nullptr;
  P->h_in = nullptr;
  if (!cuda_ok(cudaMallocHost((void **)&P->h_rp, sizeof(int) * (size_t)P->rp_stride * slots), "staging") ||
      !cuda_ok(cudaMallocHost((void **)&P->h_in, sizeof(void *) * (size_t)slots), "staging"))
    return false;
  P->staged_slots = slots;
  return true;
}

// Host side of a staged launch: the draws (from per-signal seeds) and the
// input pointers of `num` signals go into the page-locked staging.
bool plan_stage(sfft_plan *plan, int num, const void *const *in, const unsigned *seeds) {
  PlanImpl *P = impl(plan);
  if (!P || num > P->staged_slots) return false;
  std::lock_guard<std::mutex> g(P->mu);
  for (int i = 0; i < num; i++) {
    unsigned ep = 0;
    if (P->version < 2) {
      if (++P->epoch[i] >= (1u << 24)) {
        // counters of this slot must be cleared: done synchronously here,
        // outside any capture (a replay is never in flight at this point)
        if (!cuda_ok(cudaMemset(P->score.as<unsigned>() + (size_t)i * P->n, 0, sizeof(unsigned) * P->n), "memset"))
          return false;
        P->epoch[i] = 1;
      }
      ep = P->epoch[i];
    }
    Rng r;
    if (seeds) r.seed(seeds[i]);
    draw_params(*P, P->h_rp + (size_t)i * P->rp_stride, ep, r);
    P->h_in[i] = in[i];
  }
  return true;
}

// The view of a staged v1/v2 launch of `num` signals writing into the given
// outputs, for the persistent executor (no launch).
bool plan_staged_view(sfft_plan *plan, int num, int in_type, int *out_idx, void *out_val, int *out_count, long stride,
                      V12Dev *d) {
  PlanImpl *P = impl(plan);
  if (!P || P->version > 1 || num > P->staged_slots) return false;
  std::lock_guard<std::mutex> g(P->mu);
  *d = v12_view(*P);
  d->in_type = in_type;
  d->out_idx = out_idx;
  d->out_val = out_val;
  d->out_count = out_count;
  d->out_stride = stride;
  return true;
}

// Per call of the persistent executor, capturable: the staged draws and
// input pointers go to the device, the counters and comb bitmaps of `num`
// slots are cleared (what v12_run does before its first kernel).
bool plan_persist_prepare(sfft_plan *plan, int num, cudaStream_t s) {
  PlanImpl *P = impl(plan);
  if (!P || P->version > 1 || num > P->staged_slots) return false;
  std::lock_guard<std::mutex> g(P->mu);
  const auto &p = P->p12;
  return cuda_ok(cudaMemcpyAsync(P->rparams.p, P->h_rp, sizeof(int) * (size_t)P->rp_stride * num,
                                 cudaMemcpyHostToDevice, s),
                 "params upload") &&
         cuda_ok(cudaMemcpyAsync(P->inputs.p, P->h_in, sizeof(void *) * num, cudaMemcpyHostToDevice, s),
                 "pointer upload") &&
         cuda_ok(cudaMemsetAsync(P->counters.p, 0, sizeof(int) * sfft::CNT_STRIDE * num, s), "memset") &&
         cuda_ok(cudaMemsetAsync(P->comb_bits.p, 0, sizeof(unsigned) * ((p.W_Comb + 31) / 32) * (size_t)num, s),
                 "memset");
}

// Device side of a staged launch, capturable into a CUDA graph: copies the
// staging, then the batched pipeline writing into the given outputs.
bool plan_launch_staged(sfft_plan *plan, int num, int in_type, int *out_idx, void *out_val, int *out_count,
                        long stride, cudaStream_t s) {
  PlanImpl *P = impl(plan);
  if (!P || num > P->staged_slots) return false;
  std::lock_guard<std::mutex> g(P->mu);
  if (!cuda_ok(cudaMemcpyAsync(P->rparams.p, P->h_rp, sizeof(int) * (size_t)P->rp_stride * num,
                               cudaMemcpyHostToDevice, s),
               "params upload") ||
      !cuda_ok(cudaMemcpyAsync(P->inputs.p, P->h_in, sizeof(void *) * num, cudaMemcpyHostToDevice, s),
               "pointer upload"))
    return false;
  if (P->version < 2) {
    sfft::V12Dev d = v12_view(*P);
    d.in_type = in_type;
    d.out_idx = out_idx;
    d.out_val = out_val;
    d.out_count = out_count;
    d.out_stride = stride;
    return cuda_ok(sfft::v12_run(d, num, s, nullptr), "v1/v2 launch");
  }
  sfft::V3Dev d = v3_view(*P);
  d.in_type = in_type;
  d.out_idx = out_idx;
  d.out_val = out_val;
  d.out_count = out_count;
  d.out_stride = stride;
  d.trace = nullptr;
  return cuda_ok(sfft::v3_run(d, num, s, nullptr), "v3 launch");
}



}  // namespace sfft

// =================================================================== C API

extern "C" {

void *sfft_malloc(size_t s) {
  void *p = nullptr;
  if (cudaMallocHost(&p, s ? s : 16) == cudaSuccess) {
    std::lock_guard<std::mutex> g(g_alloc_mu);
    g_pinned.insert(p);
    return p;
  }
  cudaGetLastError();
  if (posix_memalign(&p, 64, s ? s : 16)) return nullptr;  // memory only, no compute
  return p;
}

void sfft_free(void *p) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> g(g_alloc_mu);
    auto it = g_pinned.find(p);
    if (it != g_pinned.end()) {
      g_pinned.erase(it);
      cudaFreeHost(p);
      return;
    }
  }
  free(p);
}

const char *sfft_last_error(void) { return g_err.c_str(); }

static sfft_plan *make_plan_impl(int n, int k, enum sfft_version version, const sfft_options *opt,
                                 const sfft::V12Knobs *knobs);

sfft_plan *sfft_make_plan_ex(int n, int k, enum sfft_version version, int fftw_optimization,
                             const sfft_options *opt) {
  (void)fftw_optimization;
  return make_plan_impl(n, k, version, opt, nullptr);
}

sfft_plan *sfft_make_plan_params(int n, int k, enum sfft_version version, const sfft_params *params,
                                 const sfft_options *opt) {
  if (!params) return make_plan_impl(n, k, version, opt, nullptr);
  if (version == SFFT_VERSION_3) {
    set_err("explicit parameters apply to v1/v2 plans");
    return nullptr;
  }
  if (params->loc_loops < 1 || params->est_loops < 0 || params->threshold_loops < 1 ||
      params->threshold_loops > params->loc_loops || params->comb_loops < 1 || params->comb_loops > 8 ||
      params->Bcst_loc <= 0 || params->Bcst_est <= 0 || params->Comb_cst <= 0 ||
      !(params->tolerance_loc > 0 && params->tolerance_loc < 1) ||
      !(params->tolerance_est > 0 && params->tolerance_est < 1)) {
    set_err("invalid plan parameters");
    return nullptr;
  }
  sfft::V12Knobs kn;
  kn.set = true;
  kn.Bcst_loc = params->Bcst_loc;
  kn.Bcst_est = params->Bcst_est;
  kn.Comb_cst = params->Comb_cst;
  kn.loc_loops = params->loc_loops;
  kn.est_loops = params->est_loops;
  kn.threshold_loops = params->threshold_loops;
  kn.comb_loops = params->comb_loops;
  kn.tolerance_loc = params->tolerance_loc;
  kn.tolerance_est = params->tolerance_est;
  return make_plan_impl(n, k, version, opt, &kn);
}

static sfft_plan *make_plan_impl(int n, int k, enum sfft_version version, const sfft_options *opt,
                                 const sfft::V12Knobs *knobs) {
  g_err.clear();
  if (version != SFFT_VERSION_1 && version != SFFT_VERSION_2 && version != SFFT_VERSION_3) {
    set_err("unknown sFFT version");
    return nullptr;
  }
  if (n < 16 || (n & (n - 1)) || k < 1 || n > (1 << 30)) {
    set_err("n must be a power of two in [16, 2^30] and k >= 1");
    return nullptr;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_err("no CUDA device: the GB300 sFFT engine has no CPU path");
    return nullptr;
  }
  std::unique_ptr<PlanImpl> P(new (std::nothrow) PlanImpl());
  if (!P) {
    set_err("out of host memory");
    return nullptr;
  }
  P->version = (int)version;
  P->n = n;
  P->k = k;
  if (opt) {
    P->prec = opt->precision == SFFT_PREC_FP32 ? sfft::PREC_FP32 : sfft::PREC_FP64;
    if (opt->max_batch > 0) P->max_batch = opt->max_batch;
  }
  if (P->version == 2) P->prec = sfft::PREC_FP64;  // phase-slope decoding needs FP64
  if (opt && opt->device >= 0) {
    if (!cuda_ok(cudaSetDevice(opt->device), "cudaSetDevice")) return nullptr;
  }
  cudaGetDevice(&P->device);
  std::string err;
  sfft::HostFilter fa, fb;
  sfft::BuildOpts bo;
  bo.fft = device_fft;
  bo.ctx = &P->device;
  if (P->version < 2) {
    if (sfft::build_v12_plan((unsigned)n, (unsigned)k, P->version == 1, P->p12, fa, fb, err, knobs, &bo)) {
      set_err(err);
      return nullptr;
    }
    const auto &p = P->p12;
    int mx = sfft::v12_max_fft(P->prec);
    // SFFT_GB300_MAX_SMEM_FFT lowers the shared-memory FFT limit so the
    // global-memory path can be exercised at small sizes
    if (const char *ov = std::getenv("SFFT_GB300_MAX_SMEM_FFT")) {
      const int v = std::atoi(ov);
      if (v >= 16 && v < mx) mx = v;
    }
    P->large_b = (p.B_loc > mx || p.B_est > mx);
    P->large_c = (P->version == 1 && p.W_Comb > mx);
    if (p.B_loc > (1 << 20) || p.B_est > (1 << 20) || p.W_Comb > (1 << 22)) {
      set_err("bucket or comb FFT longer than 2^20 points");
      return nullptr;
    }
    if (L12(*P) > 32) {
      set_err("more than 32 loops is not supported by this build");
      return nullptr;
    }
    if (!upload_taps(P->taps_a, fa.time, P->prec) || !upload_taps(P->taps_b, fb.time, P->prec) ||
        !upload_v12_window(P->win_a, fa.freq, n, n / p.B_loc, P->prec) ||
        !upload_v12_window(P->win_b, fb.freq, n, n / p.B_est, P->prec) ||
        (P->prec == sfft::PREC_FP64 &&
         (!upload_v12_window(P->win32_a, fa.freq, n, n / p.B_loc, sfft::PREC_FP32) ||
          !upload_v12_window(P->win32_b, fb.freq, n, n / p.B_est, sfft::PREC_FP32))) ||
        !upload_twiddles(P->tw_a, p.B_loc, P->prec) || !upload_twiddles(P->tw_b, p.B_est, P->prec) ||
        !upload_twiddles(P->tw_c, std::max(p.W_Comb, 2), P->prec))
      return nullptr;
  } else {
    if (sfft::build_v3_plan((unsigned)n, (unsigned)k, P->p3, fa, fb, err, &bo)) {
      set_err(err);
      return nullptr;
    }
    const auto &p = P->p3;
    if (p.B_g1 > sfft::v3_max_smem_fft()) {
      set_err("v3 with more than 8192 Gaussian buckets (k >= 8192) is not supported by this build");
      return nullptr;
    }
    P->win_half_a = 3 * (n / p.B_g1) / 2 + 2;
    P->win_half_b = 3 * (n / p.B_g2) / 2 + 2;
    if (2 * P->win_half_a + 1 > n) P->win_half_a = (n - 1) / 2;
    if (2 * P->win_half_b + 1 > n) P->win_half_b = (n - 1) / 2;
    if (!P->taps_a.upload(fa.time) || !P->taps_b.upload(fb.time) ||
        !upload_v3_window(P->win_a, fa.freq, n, P->win_half_a) ||
        !upload_v3_window(P->win_b, fb.freq, n, P->win_half_b) ||
        !upload_twiddles(P->tw_a, p.B_g1, sfft::PREC_FP64) || !upload_twiddles(P->tw_b, p.B_g2, sfft::PREC_FP64) ||
        !upload_twiddles(P->tw_c, p.W_Man, sfft::PREC_FP64))
      return nullptr;
  }
  if (!cuda_ok(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking), "stream")) return nullptr;
  if (!cuda_ok(cudaEventCreateWithFlags(&P->done, cudaEventDisableTiming), "event")) return nullptr;
  if (!cuda_ok(cudaStreamCreateWithFlags(&P->copy_in, cudaStreamNonBlocking), "stream") ||
      !cuda_ok(cudaStreamCreateWithFlags(&P->copy_out, cudaStreamNonBlocking), "stream"))
    return nullptr;
  for (int h = 0; h < 2; h++)
    if (!cuda_ok(cudaEventCreateWithFlags(&P->ev_in[h], cudaEventDisableTiming), "event") ||
        !cuda_ok(cudaEventCreateWithFlags(&P->ev_comp[h], cudaEventDisableTiming), "event") ||
        !cuda_ok(cudaEventCreateWithFlags(&P->ev_out[h], cudaEventDisableTiming), "event"))
      return nullptr;
  if (!ensure_slots(*P, 1)) return nullptr;
  sfft_plan *plan = (sfft_plan *)std::malloc(sizeof(sfft_plan));
  if (!plan) {
    set_err("out of host memory");
    return nullptr;
  }
  plan->version = version;
  plan->n = (unsigned)n;
  plan->k = (unsigned)k;
  plan->data = P.release();
  return plan;
}

sfft_plan *sfft_make_plan(int n, int k, enum sfft_version version, int fftw_optimization) {
  return sfft_make_plan_ex(n, k, version, fftw_optimization, nullptr);
}

void sfft_free_plan(sfft_plan *plan) {
  if (!plan) return;
  PlanImpl *P = impl(plan);
  if (P) {
    if (P->stream) {
      cudaStreamSynchronize(P->stream);
      cudaStreamDestroy(P->stream);
    }
    if (P->done) cudaEventDestroy(P->done);
    for (cudaStream_t st : {P->copy_in, P->copy_out})
      if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
      }
    for (int h = 0; h < 2; h++)
      for (cudaEvent_t e : {P->ev_in[h], P->ev_comp[h], P->ev_out[h]})
        if (e) cudaEventDestroy(e);
    delete P;
  }
  std::free(plan);
}

void *sfft_plan_stream(const sfft_plan *plan) {
  const PlanImpl *P = plan ? (const PlanImpl *)plan->data : nullptr;
  return P ? (void *)P->stream : nullptr;
}

long sfft_plan_footprint(const sfft_plan *plan) {
  const PlanImpl *P = plan ? (const PlanImpl *)plan->data : nullptr;
  if (!P) {
    set_err("null plan");
    return -1;
  }
  const DBuf *bufs[] = {&P->taps_a, &P->taps_b, &P->win_a, &P->win_b, &P->win32_a, &P->win32_b, &P->tw_a,
                        &P->tw_b, &P->tw_c, &P->xs, &P->xs32, &P->xs_tmp, &P->comb_buf, &P->comb_tmp, &P->J,
                        &P->score, &P->hits, &P->comb_bits, &P->comb_list, &P->counters, &P->out_idx,
                        &P->out_val, &P->man, &P->man_tmp, &P->g1, &P->g2, &P->perm, &P->est_f, &P->est_v, &P->map_keys,
                        &P->map_vals, &P->map_list, &P->rparams, &P->inputs, &P->dense_ptrs, &P->in_stage,
                        &P->dense_stage, &P->trace, &P->cnt_stash};
  long total = 0;
  for (const DBuf *b : bufs) total += (long)b->bytes;
  return total;
}

int sfft_plan_v2_voted(sfft_plan *plan, int on) {
  PlanImpl *P = plan ? (PlanImpl *)plan->data : nullptr;
  if (!P || P->version != 1) {
    set_err("the voted mode applies to v2 plans");
    return -1;
  }
  std::lock_guard<std::mutex> g(P->mu);
  if (!cuda_ok(cudaSetDevice(P->device), "cudaSetDevice") || !cuda_ok(cudaStreamSynchronize(P->stream), "sync"))
    return -1;
  P->voted = on ? 1 : 0;
  const int slots = P->slots;
  P->slots = 0;  // re-derive capacities; the output and hit buffers are resized
  P->out_idx.release();
  P->out_val.release();
  P->hits.release();
  return ensure_slots(*P, std::max(1, slots)) ? 0 : -1;
}

long sfft_output_capacity(const sfft_plan *plan) {
  const PlanImpl *P = plan ? (const PlanImpl *)plan->data : nullptr;
  if (!P) {
    set_err("null plan");
    return -1;
  }
  return P->out_cap;
}

void sfft_exec(sfft_plan *plan, complex_t *in, complex_t *out) {
  sfft_exec_many(plan, 1, &in, &out);
}

void sfft_exec_many(sfft_plan *plan, int num, complex_t **in, complex_t **out) {
  PlanImpl *P = impl(plan);
  if (!P || num < 0 || (num && (!in || !out))) {
    set_err("invalid arguments");
    return;
  }
  std::lock_guard<std::mutex> g(P->mu);
  cudaSetDevice(P->device);
  g_err.clear();
  const int chunk = std::max(1, std::min(P->max_batch, num));
  bool all_host = num > 1;
  for (int i = 0; i < num && all_host; i++)
    if (is_device_ptr(in[i]) || is_device_ptr(out[i])) all_host = false;
  if (all_host) {  // about 32 chunks: copies overlap the transforms with little fill and drain
    exec_dense_pipelined(*P, num, in, out, std::max(1, std::min(chunk, (num + 31) / 32)));
    return;
  }
  if (!ensure_slots(*P, chunk)) return;
  for (int i = 0; i < num; i += chunk) {
    const int m = std::min(chunk, num - i);
    if (!exec_dense_chunk(*P, m, in + i, out + i)) return;
  }
}

long sfft_exec_sparse(sfft_plan *plan, const complex_t *in, int *out_idx, complex_t *out_val, long cap) {
  PlanImpl *P = impl(plan);
  if (!P || !in || !out_idx || !out_val) {
    set_err("invalid arguments");
    return -1;
  }
  std::lock_guard<std::mutex> g(P->mu);
  cudaSetDevice(P->device);
  g_err.clear();
  cudaStream_t s = P->stream;
  const size_t nb = sizeof(double) * 2 * (size_t)P->n;
  const void *dev_in = in;
  if (!is_device_ptr(in)) {
    if (!P->in_stage.ensure(nb * std::max(1, P->slots))) return -1;
    if (!cuda_ok(cudaMemcpyAsync(P->in_stage.p, in, nb, cudaMemcpyHostToDevice, s), "input copy")) return -1;
    dev_in = P->in_stage.p;
  }
  if (!launch(*P, 1, &dev_in, sfft::IN_C128, s)) return -1;
  int cnt[sfft::CNT_STRIDE];
  if (!cuda_ok(cudaMemcpyAsync(cnt, P->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, s), "count") ||
      !cuda_ok(cudaStreamSynchronize(s), "exec"))
    return -1;
  if (cnt[sfft::CNT_ERR]) {
    check_device_errors(*P, 1);
    return -1;
  }
  const long c = cnt[sfft::CNT_OUT];
  if (c > cap) {
    set_err("output capacity too small (" + std::to_string(c) + " coefficients)");
    return -1;
  }
  const bool dev_out = is_device_ptr(out_idx);
  const cudaMemcpyKind kind = dev_out ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (!cuda_ok(cudaMemcpyAsync(out_idx, P->out_idx.p, sizeof(int) * c, kind, s), "index copy")) return -1;
  const bool fp32_vals = P->version < 2 && P->prec == sfft::PREC_FP32;
  if (!fp32_vals) {
    if (!cuda_ok(cudaMemcpyAsync(out_val, P->out_val.p, 16 * c, kind, s), "value copy")) return -1;
    if (!cuda_ok(cudaStreamSynchronize(s), "copy")) return -1;
  } else {
    std::vector<float> tmp(2 * (size_t)c);
    if (!cuda_ok(cudaMemcpyAsync(tmp.data(), P->out_val.p, 8 * c, cudaMemcpyDeviceToHost, s), "value copy") ||
        !cuda_ok(cudaStreamSynchronize(s), "copy"))
      return -1;
    std::vector<double> w(2 * (size_t)c);
    for (size_t i = 0; i < w.size(); i++) w[i] = tmp[i];
    if (!cuda_ok(cudaMemcpy(out_val, w.data(), 16 * c, dev_out ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost),
                 "value copy"))
      return -1;
  }
  return c;
}

int sfft_exec_many_sparse(sfft_plan *plan, int num, const complex_t *const *in, int *out_idx, void *out_val,
                          int *out_count, long out_stride) {
  PlanImpl *P = impl(plan);
  if (!P || num < 0 || (num > 0 && (!in || !out_idx || !out_val || !out_count))) {
    set_err("invalid arguments");
    return -1;
  }
  if (num == 0) return 0;
  std::lock_guard<std::mutex> g(P->mu);
  cudaSetDevice(P->device);
  g_err.clear();
  const int chunk = std::max(1, std::min(P->max_batch, (num + 31) / 32));  // about 32 pipelined chunks
  return exec_sparse_pipelined(*P, num, in, out_idx, out_val, out_count, out_stride, chunk) ? 0 : -1;
}

int sfft_exec_batch(sfft_plan *plan, int num, const void *const *in, int in_type, int *out_idx, void *out_val,
                    int *out_count, long out_stride, void *stream) {
  return sfft_exec_batch_ex(plan, num, in, in_type, nullptr, out_idx, out_val, out_count, out_stride, stream);
}

int sfft_exec_batch_ex(sfft_plan *plan, int num, const void *const *in, int in_type, const unsigned *seeds,
                       int *out_idx, void *out_val, int *out_count, long out_stride, void *stream) {
  PlanImpl *P = impl(plan);
  if (!P || num < 1 || !in || !out_idx || !out_val || !out_count || out_stride < 0) {
    set_err("invalid arguments");
    return -1;
  }
  if (out_stride < P->out_cap) {
    set_err("out_stride below sfft_output_capacity");
    return -1;
  }
  std::lock_guard<std::mutex> g(P->mu);
  cudaSetDevice(P->device);
  g_err.clear();
  cudaStream_t s = stream ? (cudaStream_t)stream : P->stream;
  if (!ensure_slots(*P, std::min(num, std::max(1, P->max_batch)))) return -1;
  if (!cuda_ok(cudaStreamWaitEvent(s, P->done, 0), "event wait")) return -1;
  const size_t cs = (P->version < 2 && P->prec == sfft::PREC_FP32) ? 8 : 16;
  for (int i0 = 0; i0 < num; i0 += P->slots) {
    const int m = std::min(P->slots, num - i0);
    // results go straight into the caller's strided buffers
    OutTarget t{out_idx + (size_t)i0 * out_stride, (char *)out_val + cs * (size_t)i0 * out_stride, out_count + i0,
                out_stride};
    if (!launch(*P, m, in + i0, in_type, s, &t, 0, seeds ? seeds + i0 : nullptr)) return -1;
  }
  return cuda_ok(cudaEventRecord(P->done, s), "event") ? 0 : -1;
}

int sfft_sync(sfft_plan *plan) {
  PlanImpl *P = impl(plan);
  if (!P) {
    set_err("null plan");
    return -1;
  }
  std::lock_guard<std::mutex> g(P->mu);
  if (!cuda_ok(cudaEventSynchronize(P->done), "sync") || !cuda_ok(cudaStreamSynchronize(P->stream), "sync"))
    return -1;
  return check_device_errors(*P, std::max(1, P->slots)) ? 0 : -1;
}

long sfft_debug_fetch(sfft_plan *plan, int what, void *dst, long cap) {
  PlanImpl *P = impl(plan);
  if (!P || !dst) {
    set_err("invalid arguments");
    return -1;
  }
  std::lock_guard<std::mutex> g(P->mu);
  if (!cuda_ok(cudaStreamSynchronize(P->stream), "sync")) return -1;
  if (what == 7) {  // the counters of batch slot 0, any version
    if (cap < sfft::CNT_STRIDE) return -1;
    if (!cuda_ok(cudaMemcpy(dst, P->counters.p, sizeof(int) * sfft::CNT_STRIDE, cudaMemcpyDeviceToHost), "debug"))
      return -1;
    return sfft::CNT_STRIDE;
  }
  auto fetch = [&](const void *src, long count, size_t esz) -> long {
    if (count > cap) {
      set_err("debug buffer too small");
      return -1;
    }
    if (!cuda_ok(cudaMemcpy(dst, src, esz * count, cudaMemcpyDeviceToHost), "debug copy")) return -1;
    return count;
  };
  if (P->version < 2) {
    const auto &p = P->p12;
    const int L = L12(*P);
    switch (what) {
      case 0: {
        if (2 * L > cap) return -1;
        std::memcpy(dst, P->last_rp.data(), sizeof(int) * 2 * L);
        return 2 * L;
      }
      case 1:
        return fetch(P->J.p, (long)L * p.B_thresh, sizeof(int));
      case 2: {
        if (P->n > cap) return -1;
        std::vector<unsigned> raw(P->n);
        if (!cuda_ok(cudaMemcpy(raw.data(), P->score.p, sizeof(unsigned) * P->n, cudaMemcpyDeviceToHost), "debug"))
          return -1;
        int *o = (int *)dst;
        // v2 keeps its counters residue-major: frequency rep W + r at r (n / W) + rep
        const bool rmaj = P->version == 1;
        const long W = p.W_Comb, R = rmaj ? P->n / W : 1;
        for (long i = 0; i < P->n; i++) {
          const long f = rmaj ? (i % R) * W + i / R : i;
          o[f] = ((raw[i] >> 8) == P->epoch[0]) ? (int)(raw[i] & 255u) : 0;
        }
        return P->n;
      }
      case 3: {  // bucket values in natural order
        const size_t es = P->prec == sfft::PREC_FP64 ? 16 : 8;
        if (p.x_samp_size > cap) return -1;
        std::vector<unsigned char> raw(es * p.x_samp_size);
        if (!cuda_ok(cudaMemcpy(raw.data(), P->xs.p, raw.size(), cudaMemcpyDeviceToHost), "debug")) return -1;
        const int lg = xs_perm_of(*P);
        unsigned char *o = (unsigned char *)dst;
        long base = 0;
        for (int j = 0; j < L; j++) {
          const long B = j < p.loops_loc ? p.B_loc : p.B_est;
          for (long b = 0; b < B; b++)
            std::memcpy(o + es * (base + b), raw.data() + es * (base + xs_position(b, B, lg)), es);
          base += B;
        }
        return p.x_samp_size;
      }
      case 4: {
        int cnt[sfft::CNT_STRIDE];
        if (!cuda_ok(cudaMemcpy(cnt, P->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost), "debug")) return -1;
        return fetch(P->comb_list.p, cnt[sfft::CNT_COMB], sizeof(int));
      }
      case 8:    // estimation window of the location filter, as uploaded:
      case 9: {  // FP64 (c, d, c^2 + d^2, 0) doubles, FP32 conj(h)/|h|^2 floats
        const long q = P->n / (what == 8 ? p.B_loc : p.B_est);
        const DBuf &w = what == 8 ? P->win_a : P->win_b;
        return P->prec == sfft::PREC_FP64 ? fetch(w.p, 4 * q, 8) : fetch(w.p, 2 * q, 4);
      }
      default:
        break;
    }
  } else if (what == 6) {
    int cnt[sfft::CNT_STRIDE];
    if (!cuda_ok(cudaMemcpy(cnt, P->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost), "debug")) return -1;
    const long nrec = std::min(cnt[sfft::CNT_TRACE], P->map_cap);
    if (5 * nrec > cap) return -1;
    if (!cuda_ok(cudaMemcpy(dst, P->trace.p, sizeof(double) * 5 * nrec, cudaMemcpyDeviceToHost), "debug"))
      return -1;
    return 5 * nrec;
  } else if (what == 5) {
    int cnt[sfft::CNT_STRIDE];
    if (!cuda_ok(cudaMemcpy(cnt, P->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost), "debug")) return -1;
    if (cap < 1) return -1;
    ((int *)dst)[0] = cnt[sfft::CNT_V3];
    return 1;
  } else if (what == 0) {
    if (cap < 5) return -1;
    std::memcpy(dst, P->last_rp.data(), sizeof(int) * 5);
    return 5;
  }
  set_err("unknown diagnostic");
  return -1;
}

int sfft_describe_plan(int n, int k, enum sfft_version version, long *fields, int nfields) {
  g_err.clear();
  if (!fields || n < 16 || (n & (n - 1)) || k < 1) {
    set_err("invalid arguments");
    return -1;
  }
  std::string err;
  sfft::HostFilter fa, fb;
  sfft::BuildOpts bo;
  bo.filters = false;  // parameters and tap counts only
  std::vector<long> v;
  if (version == SFFT_VERSION_1 || version == SFFT_VERSION_2) {
    sfft::V12Params p;
    if (sfft::build_v12_plan((unsigned)n, (unsigned)k, version == SFFT_VERSION_2, p, fa, fb, err, nullptr, &bo)) {
      set_err(err);
      return -1;
    }
    v = {p.B_loc, p.B_thresh, p.B_est, p.W_Comb, p.Comb_loops, p.loops_loc, p.loops_thresh, p.loops_est,
         p.w_loc, p.w_est, p.x_samp_size};
  } else if (version == SFFT_VERSION_3) {
    sfft::V3Params p;
    if (sfft::build_v3_plan((unsigned)n, (unsigned)k, p, fa, fb, err, &bo)) {
      set_err(err);
      return -1;
    }
    v = {p.W_Man, p.B_g1, p.w_g1, p.B_g2, p.w_g2};
  } else {
    set_err("unknown sFFT version");
    return -1;
  }
  const int m = std::min<int>(nfields, (int)v.size());
  for (int i = 0; i < m; i++) fields[i] = v[i];
  return m;
}

int sfft_describe_plan_params(int n, int k, enum sfft_version version, const sfft_params *params, long *fields,
                              int nfields) {
  if (!params) return sfft_describe_plan(n, k, version, fields, nfields);
  g_err.clear();
  if (!fields || n < 16 || (n & (n - 1)) || k < 1 || version == SFFT_VERSION_3) {
    set_err("invalid arguments");
    return -1;
  }
  sfft::V12Knobs kn;
  kn.set = true;
  kn.Bcst_loc = params->Bcst_loc;
  kn.Bcst_est = params->Bcst_est;
  kn.Comb_cst = params->Comb_cst;
  kn.loc_loops = params->loc_loops;
  kn.est_loops = params->est_loops;
  kn.threshold_loops = params->threshold_loops;
  kn.comb_loops = params->comb_loops;
  kn.tolerance_loc = params->tolerance_loc;
  kn.tolerance_est = params->tolerance_est;
  sfft::BuildOpts bo;
  bo.filters = false;
  sfft::V12Params p;
  sfft::HostFilter fa, fb;
  std::string err;
  if (sfft::build_v12_plan((unsigned)n, (unsigned)k, version == SFFT_VERSION_2, p, fa, fb, err, &kn, &bo)) {
    set_err(err);
    return -1;
  }
  const long v[] = {p.B_loc,     p.B_thresh, p.B_est, p.W_Comb, p.Comb_loops,   p.loops_loc,
                    p.loops_thresh, p.loops_est, p.w_loc, p.w_est, p.x_samp_size};
  const int m = std::min<int>(nfields, 11);
  for (int i = 0; i < m; i++) fields[i] = v[i];
  return m;
}

int sfft_describe_filter(int n, int k, enum sfft_version version, int which, double *time, long time_cap,
                         double *freq, long freq_cap) {
  g_err.clear();
  if (n < 16 || (n & (n - 1)) || k < 1 || (which != 0 && which != 1)) {
    set_err("invalid arguments");
    return -1;
  }
  std::string err;
  sfft::HostFilter fa, fb;
  int rc;
  if (version == SFFT_VERSION_1 || version == SFFT_VERSION_2) {
    sfft::V12Params p;
    rc = sfft::build_v12_plan((unsigned)n, (unsigned)k, version == SFFT_VERSION_2, p, fa, fb, err);
  } else if (version == SFFT_VERSION_3) {
    sfft::V3Params p;
    rc = sfft::build_v3_plan((unsigned)n, (unsigned)k, p, fa, fb, err);
  } else {
    set_err("unknown sFFT version");
    return -1;
  }
  if (rc) {
    set_err(err);
    return -1;
  }
  const sfft::HostFilter &f = which ? fb : fa;
  if (time) {
    if (time_cap < 2L * f.w) {
      set_err("time buffer too small");
      return -1;
    }
    std::memcpy(time, f.time.data(), sizeof(double) * 2 * f.w);
  }
  if (freq) {
    if (freq_cap < 2L * n) {
      set_err("freq buffer too small");
      return -1;
    }
    std::memcpy(freq, f.freq.data(), sizeof(double) * 2 * (size_t)n);
  }
  return f.w;
}

int sfft_profile(sfft_plan *plan, int enable) {
  PlanImpl *P = impl(plan);
  if (!P) {
    set_err("null plan");
    return -1;
  }
  std::lock_guard<std::mutex> g(P->mu);
  P->harvest();
  P->profiling = enable != 0;
  for (double &m : P->stage_ms) m = 0;
  P->profiled = 0;
  return 0;
}

long sfft_profile_read(sfft_plan *plan, double *stage_ms, int nstage) {
  PlanImpl *P = impl(plan);
  if (!P || !stage_ms) {
    set_err("invalid arguments");
    return -1;
  }
  std::lock_guard<std::mutex> g(P->mu);
  P->harvest();
  for (int i = 0; i < nstage && i < 8; i++) stage_ms[i] = P->stage_ms[i];
  return P->profiled;
}

long sfft_kernel_launches(void) { return sfft::g_launches.load(); }

}  // extern "C"
