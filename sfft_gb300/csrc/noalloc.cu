// noalloc.cu — sfft_exec_noalloc: a v1/v2 transform whose per-call
// scratch is a fixed area compiled into this library instead of memory
// obtained from cudaMalloc.
//
// Some callers of this library cannot allocate GPU memory while they run:
// a host that has handed all device memory to its own pool allocator, a
// process held to a fixed memory budget after start-up, or a latency-bound
// stream on which cudaMalloc/cudaFree would block or synchronise the whole
// device.  For them, the transform's working set (bucket samples, selected
// buckets, vote counters, hits, comb residues, counters and the random
// draws) lives in the static device array below.  The plan's constants
// (filter taps, estimation windows, twiddle tables) were placed on the
// device when the plan was made and are only read here.
//
// Limits: the array holds SFFT_NOALLOC_SCRATCH_BYTES (4 MiB) on every GPU
// that loads the library, for the life of the process.  That covers v1/v2
// plans with n <= 2^18, at most 65536 bucket samples and at most 32 loops;
// larger plans are rejected with an error.
//
// Sharing: every call on a device uses the same array and it keeps the last
// call's contents.  The counters and comb bitmap are cleared on the stream
// at the start of each call; vote counters carry a per-call tag instead of
// being cleared, and they occupy a fixed region at the start of the array
// that nothing else is written to, so plans of different sizes can follow
// one another.  Calls whose GPU work overlaps (different streams, or
// different threads without ordering) race on the array.
//
// Set-up: the first call on each device looks up the array's device
// address (cudaGetSymbolAddress) with that device current; make that first
// call before any stream capture begins.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/sfft.h"
#include "engine.h"

namespace sfft {
bool plan_v12_constants(sfft_plan *plan, V12Dev *d, int *hit_cap, int *out_cap);
void plan_draw(sfft_plan *plan, int *rp, unsigned epoch);
int plan_device(sfft_plan *plan);
void set_last_error(const char *m);
}  // namespace sfft

#define SFFT_NOALLOC_SCRATCH_BYTES (4u << 20)
#define SFFT_NOALLOC_MAX_N (1 << 18)
#define SFFT_NOALLOC_MAX_XS 65536L
#define SFFT_NOALLOC_MAX_LOOPS 32
#define SFFT_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[SFFT_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_mu;
unsigned char *g_dev_scratch[SFFT_NOALLOC_MAX_DEVICES];
unsigned g_epoch[SFFT_NOALLOC_MAX_DEVICES];

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" long sfft_exec_noalloc(sfft_plan *plan, const void *d_in, int in_type, int *d_out_idx, void *d_out_val,
                                  long cap, int *d_status, void *stream) {
  using namespace sfft;
  V12Dev d;
  int hit_cap = 0, out_cap = 0;
  if (!plan || !d_in || !d_out_idx || !d_out_val || !d_status || !plan_v12_constants(plan, &d, &hit_cap, &out_cap)) {
    set_last_error("sfft_exec_noalloc: needs a v1/v2 plan and device buffers for input, outputs and status");
    return -1;
  }
  if (cap < out_cap) {
    set_last_error("sfft_exec_noalloc: output capacity below sfft_output_capacity(plan)");
    return -1;
  }
  const int L = d.L;
  const int rp_stride = 2 * L + d.comb_loops + 1;
  if (rp_stride > 2 * SFFT_NOALLOC_MAX_LOOPS + 16) {
    set_last_error("sfft_exec_noalloc: plan exceeds the static scratch (too many loops)");
    return -1;
  }
  const size_t cs = d.prec == PREC_FP64 ? 16 : 8;
  // Layout of the static area.  The vote counters come first, at a fixed
  // offset and sized for the largest n, so that whatever plan ran before,
  // every word of that region was written only as a vote counter
  // ((tag << 8) | votes) or is still zero: a stale word can never pass for
  // a counter of the current call.  The regions after it move with the
  // plan's sizes and are rewritten before they are read.
  size_t off = 0;
  const size_t o_score = off;
  off += up256(sizeof(unsigned) * (size_t)SFFT_NOALLOC_MAX_N);
  const size_t o_cnt = off;
  off += up256(sizeof(int) * CNT_STRIDE);
  const size_t o_rp = off;
  off += up256(sizeof(int) * rp_stride);
  const size_t o_in = off;
  off += up256(sizeof(void *));
  const size_t o_xs = off;
  off += up256(cs * (size_t)d.xs_size);
  const size_t o_xs32 = off;
  if (d.prec == PREC_FP64) off += up256(8 * (size_t)d.xs_size);
  const size_t o_J = off;
  off += up256(sizeof(int) * (size_t)L * d.num);
  const size_t o_hits = off;
  off += up256(sizeof(int) * (size_t)hit_cap);
  const size_t o_bits = off;
  off += up256(sizeof(unsigned) * (size_t)((d.W + 31) / 32));
  const size_t o_list = off;
  off += up256(sizeof(int) * (size_t)d.W);
  if (d.large_buckets || d.large_comb || d.n > SFFT_NOALLOC_MAX_N || d.xs_size > SFFT_NOALLOC_MAX_XS || L > SFFT_NOALLOC_MAX_LOOPS ||
      off > SFFT_NOALLOC_SCRATCH_BYTES) {
    set_last_error("sfft_exec_noalloc: plan exceeds the 4 MiB static scratch (limits: n <= 2^18, "
                   "at most 65536 bucket samples, at most 32 loops)");
    return -1;
  }
  const int dev = plan_device(plan);
  if (dev < 0 || dev >= SFFT_NOALLOC_MAX_DEVICES) {
    set_last_error("sfft_exec_noalloc: device ordinal out of range");
    return -1;
  }
  std::lock_guard<std::mutex> g(g_mu);
  if (cudaSetDevice(dev) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("sfft_exec_noalloc: cudaSetDevice failed");
    return -1;
  }
  if (!g_dev_scratch[dev]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      cudaGetLastError();
      set_last_error("sfft_exec_noalloc: cudaGetSymbolAddress of the static scratch failed");
      return -1;
    }
    g_dev_scratch[dev] = (unsigned char *)ptr;
  }
  unsigned char *base = g_dev_scratch[dev];
  cudaStream_t s = (cudaStream_t)stream;
  // A fresh vote tag per call on this device (tags start at 1; the array
  // starts zeroed).  When the 24-bit tag would wrap, the whole counter
  // region is cleared so that no counter of an earlier call can carry the
  // new tag.
  if (++g_epoch[dev] >= (1u << 24)) {
    if (cudaMemsetAsync(base + o_score, 0, sizeof(unsigned) * (size_t)SFFT_NOALLOC_MAX_N, s) != cudaSuccess) {
      cudaGetLastError();
      set_last_error("sfft_exec_noalloc: clearing vote counters failed");
      return -1;
    }
    g_epoch[dev] = 1;
  }
  int rp[2 * SFFT_NOALLOC_MAX_LOOPS + 16];
  plan_draw(plan, rp, g_epoch[dev]);
  const void *in_ptr = d_in;
  if (cudaMemcpyAsync(base + o_rp, rp, sizeof(int) * rp_stride, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(base + o_in, &in_ptr, sizeof(void *), cudaMemcpyHostToDevice, s) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("sfft_exec_noalloc: parameter upload failed");
    return -1;
  }
  // Counters left by earlier calls (of any plan) carry earlier tags and
  // count as zero votes; the region holds SFFT_NOALLOC_MAX_N >= n counters.
  d.xs = base + o_xs;
  d.xs32 = d.prec == PREC_FP64 ? base + o_xs32 : nullptr;
  d.J = (int *)(base + o_J);
  d.score = (unsigned *)(base + o_score);
  d.hits = (int *)(base + o_hits);
  d.comb_bits = (unsigned *)(base + o_bits);
  d.comb_list = (int *)(base + o_list);
  d.counters = (int *)(base + o_cnt);
  d.out_idx = d_out_idx;
  d.out_val = d_out_val;
  d.out_count = nullptr;
  d.hit_cap = hit_cap;
  d.out_cap = out_cap;
  d.out_stride = out_cap;
  d.rparams = (const int *)(base + o_rp);
  d.rp_stride = rp_stride;
  d.inputs = (const void *const *)(base + o_in);
  d.in_type = in_type;
  cudaError_t e = v12_run(d, 1, s, nullptr);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_status, base + o_cnt + sizeof(int) * CNT_OUT, sizeof(int), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_status + 1, base + o_cnt + sizeof(int) * CNT_ERR, sizeof(int), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_last_error(cudaGetErrorString(e));
    return -1;
  }
  return 0;
}
