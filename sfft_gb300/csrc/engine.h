// engine.h — device-side view of a plan and the launch entry points of the
// sFFT kernels.  Shared by the C-ABI layer (api.cc) and the kernels
// (v12.cu, v3.cu).  Plain structs of device pointers and sizes.
#pragma once

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

namespace sfft {

// Optional per-stage timing: when non-null, an event is recorded on the
// stream before the first stage and after each stage (stage names in
// api.cc).  Kernel launches are counted in `launches`.
struct StageEvents {
  cudaEvent_t ev[8];
  int recorded = 0;
};
void note_launches(long n);
void mark(StageEvents *se, cudaStream_t s);

enum Precision { PREC_FP64 = 0, PREC_FP32 = 1 };
enum InType { IN_C128 = 0, IN_C64 = 1 };

// Per-slot counters (one block of ints per slot, zeroed before each exec).
enum Counter { CNT_HITS = 0, CNT_COMB = 1, CNT_OUT = 2, CNT_ERR = 3, CNT_VOTED = 4, CNT_V3 = 5,
               CNT_TRACE = 6, CNT_EST = 7, CNT_EXACT = 8, CNT_STRIDE = 16 };

// Error bits reported in counters[CNT_ERR].
enum ErrBits { ERR_HIT_OVERFLOW = 1, ERR_OUT_OVERFLOW = 2, ERR_V3_NOCONVERGE = 4, ERR_V3_CAP = 8,
               ERR_WAIT_TIMEOUT = 16 };

// ---------------------------------------------------------------- v1/v2 --
struct V12Dev {
  int version;  // 0 = v1, 1 = v2
  int prec;
  int n, logn, k, num;
  int B_loc, B_est, L_loc, L_est, L, thresh;
  int W, comb_loops;
  int w_loc, w_est;
  int q_loc, q_est;  // n / B
  long xs_size;      // per slot, complex entries
  // plan constants
  const void *taps_loc, *taps_est;  // w complex (double2 or float2)
  const void *win_loc, *win_est;    // q entries: FP64 double4 (c, d, c^2+d^2, 0); FP32 float2 (g)
  const void *tw_loc, *tw_est, *tw_comb;  // twiddle tables (double2 or float2)
  const void *win32_loc, *win32_est;  // FP64 plans: float2 g = conj-scaled window for bounds
  // per-slot workspace
  void *xs;                 // xs_size complex per slot
  void *xs32;               // FP64 plans: float2 copy of xs (median pre-selection)
  void *xs_tmp;             // large bucket FFTs: ping-pong partner of xs
  void *comb_buf, *comb_tmp;  // large comb FFTs: comb_loops * W per slot
  int large_buckets, large_comb;  // FFT longer than one CTA's shared memory
  // Bucket layout of xs (and xs32).  0: natural, bucket b of a loop at b.
  // lg > 0 (plain v2 FP32 with W a multiple of both n/B): grouped for the
  // estimation by comb residue -- with G = 2^lg and T = B / G, bucket b of
  // a loop sits at (b mod T) * G + b / T, so the buckets one group of G
  // candidates of one residue reads in a loop are G consecutive entries.
  int xs_perm;
  int *J;                   // L * num per slot
  unsigned *score;          // n per slot: (epoch << 8) | votes
  int *hits;                // hit_cap per slot
  unsigned *comb_bits;      // W/32 per slot
  int *comb_list;           // W per slot
  int *counters;            // CNT_STRIDE per slot
  int *out_idx;             // out_stride per slot
  void *out_val;            // out_stride complex per slot (R2)
  int *out_count;           // optional: per-slot coefficient count
  int hit_cap, out_cap;
  int voted;                // v2: estimate only candidates that reached the vote threshold
  long out_stride;
  // per-exec inputs
  const int *rparams;       // per slot: a[L], ai[L], comb_offsets[comb_loops], epoch
  int rp_stride;
  const void *const *inputs;  // device array of per-slot input pointers
  int in_type;
};

// Launches the whole v1/v2 pipeline for `nslots` signals on `stream`.
cudaError_t v12_run(const V12Dev &d, int nslots, cudaStream_t stream, StageEvents *se = nullptr);
// Scatters the sparse result of each slot into dense n-point complex128
// outputs (device array of per-slot pointers, already zeroed).
// Device-to-device copy of `count` ints by a kernel (stream-ordered, no copy
// engine involved).
cudaError_t copy_ints(const int *src, int *dst, int count, cudaStream_t s);
cudaError_t scatter_dense(const int *out_idx, const void *out_val, int prec, const int *counters,
                          int out_cap, void *const *dense, int nslots, cudaStream_t stream);

// Maximum bucket-FFT length held in one CTA's shared memory.
int v12_max_fft(int prec);

// ------------------------------------------- persistent uneven executor --
// One persistent kernel runs the whole v2 pipeline of several FP32 plans
// (plain v2, FFTs in shared memory): a device work queue of (stage, plan,
// signal, tile) items in dependency order, per-signal completion counters
// in global memory, bounded waits.
enum PersistKind { PK_COMB = 0, PK_FOLD = 1, PK_LIST = 2, PK_BUCKET = 3, PK_VOTE = 4, PK_EST = 5 };
struct PersistGroup {
  V12Dev d;          // the plan's view: staged draws and inputs, outputs in the caller's arena
  int gslot0;        // first global signal slot of this plan
  int slots;         // its signals
  int per_comb, per_bucket;   // butterflies per thread of the comb / bucket FFTs (1, 2, 4)
  int fold_chunks;   // 1024-thread chunks of the fold per item
  int vote_cmax, vote_chunks; // comb residues at most; unused (1)
  int est_comb;      // 1: estimation by comb residue (1024 candidates per item), 0: random lookups
  int est_chunks;    // random lookups: 1024-candidate chunks per item
  int nfold, nvote, nest;     // items per signal of those stages
  int pad;
};
struct PersistItem {
  int kind, group, slot, idx;
};
struct PersistProg {
  const PersistGroup *groups;  // device
  const PersistItem *items;    // device, dependency order
  int nitems;
  int *state;                  // device: queue head, abort flag, 4 counters per global slot (zeroed per run)
  int nslots_total;
  size_t smem;                 // dynamic shared memory per CTA
  int in_type;
};
// Dependency-ordered item list for `groups` (host copies; d must be set),
// ordered for `workers` resident CTAs.
void persist_items(const PersistGroup *groups, int ngroups, std::vector<PersistItem> &items, int workers);
// Shared memory the executor needs for these groups, and whether a plan
// view qualifies (plain FP32 v2, FFTs in shared memory, at most 32 loops).
size_t persist_smem(const PersistGroup *groups, int ngroups);
bool persist_eligible(const V12Dev &d);
// Fills a group's launch shape from its view.
void persist_shape(PersistGroup &g);
cudaError_t persist_run(const PersistProg &p, cudaStream_t s);

// -------------------------------------------------------------------- v3 --
struct V3Dev {
  int prec;
  int n, logn, k;
  int W, B1, B2, w1, w2;
  int q1, q2;          // n / B1, n / B2
  int win1_half, win2_half;
  const void *taps1, *taps2;    // double2
  const void *win1, *win2;      // double2, 2*half+1 entries centred on freq index 0
  const void *tw_man, *tw_g1, *tw_g2;
  // per-slot workspace
  void *man;     // 2W complex (interleaved loops)
  void *man_tmp; // large_man: 4W complex (two W-point arrays and their FFT scratch)
  int large_man; // W above the shared-memory FFT: Mansour comb FFTs in global memory
  void *g1;      // 2*B1 complex
  void *g2;      // 2*B2 complex
  void *perm;    // (w2 + 1) complex
  int *est_f;    // cap per slot
  void *est_v;   // cap complex per slot
  int *map_keys; // map_cap per slot
  void *map_vals;
  int *map_table;  // table_cap per slot
  int est_cap, map_cap, table_cap;
  int *counters;
  int *out_idx;
  void *out_val;
  int *out_count;
  int out_cap;
  long out_stride;
  int max_passes;
  double *trace;       // slot 0 only: (round, stage, key, re, im) per estimate
  int trace_cap;
  const int *rparams;  // per slot: a, ai, b, init_offset, init_G_offset
  int rp_stride;
  const void *const *inputs;
  int in_type;
};

cudaError_t v3_run(const V3Dev &d, int nslots, cudaStream_t stream, StageEvents *se = nullptr);
// Largest FP64 FFT the v3 filter kernel runs in shared memory.
int v3_max_smem_fft();
// Whether a v3 plan's Mansour comb FFT of W points runs as eight W/8-point
// FFTs over eight CTAs and a radix-8 combination (W from 4096 up to the
// shared-memory limit) instead of in one CTA of the filter kernel.
inline bool v3_man_split(int W) { return W >= 4096 && W <= v3_max_smem_fft(); }
// Batched complex128 FFTs of length N in global memory (the same stages as
// the shared-memory FFT): narr arrays per slot, arr_stride apart, slots
// slot_stride apart; b is scratch of the same shape; result in a.
cudaError_t global_fft_c128(void *a, void *b, int N, int narr, long arr_stride, long slot_stride, int nslots,
                            const void *tw, cudaStream_t s);

}  // namespace sfft
