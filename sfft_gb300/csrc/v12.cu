// v12.cu — the sFFT v1/v2 exec pipeline on GB300.
//
//   k_comb      (v2) strided W-point gather + shared-memory FFT + |.|^2 +
//               top-num residues -> comb bitmap     (computefourier-1.0-2.0.cc:48-82)
//   k_comb_list (v2) bitmap -> sorted, de-duplicated residue list   (:491-503)
//   k_fold      permuted-filter fold, one thread per (loop, bucket),
//               taps summed in increasing order                      (:222-261)
//   k_bucket    per loop: B-point FFT in shared memory, |.|^2, top-num
//               bucket selection, then (location loops) integer voting
//               of the n/B frequencies of each selected bucket      (:270-324, :91-184)
//   k_estimate  per candidate: value in each loop, lower median of the
//               real and imaginary parts separately                 (:340-419)
//
// All kernels take a slot index (blockIdx.y) so that one launch serves a
// batch of signals sharing a plan.  FP64 instantiations reproduce the CPU
// definition bit for bit; FP32 ones accumulate in float.
#include <algorithm>
#include <functional>
#include <queue>
#include <cstdlib>
#include <tuple>
#include <mutex>
#include <map>
#include <cfloat>
#include <climits>

#include "common.cuh"
#include "engine.h"

namespace sfft {

template <typename R> __device__ __forceinline__ c2_t<R> cvt_in(double2 v);
template <> __device__ __forceinline__ double2 cvt_in<double>(double2 v) { return v; }
template <> __device__ __forceinline__ float2 cvt_in<float>(double2 v) {
  return make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
}
template <typename R> __device__ __forceinline__ c2_t<R> cvt_in(float2 v);
template <> __device__ __forceinline__ double2 cvt_in<double>(float2 v) {
  return make_double2((double)v.x, (double)v.y);
}
template <> __device__ __forceinline__ float2 cvt_in<float>(float2 v) { return v; }

__device__ __forceinline__ int dlog2(unsigned v) { return 31 - __clz(v); }

// ------------------------------------------------------------------ fold --

template <typename R, typename In>
__global__ void __launch_bounds__(256) k_fold(V12Dev d) {
  const int slot = blockIdx.y;
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= d.xs_size) return;
  const long locsz = (long)d.L_loc * d.B_loc;
  int j, b, B, w;
  const c2_t<R> *taps;
  if (g < locsz) {
    j = (int)(g / d.B_loc);
    b = (int)(g & (d.B_loc - 1));
    B = d.B_loc;
    w = d.w_loc;
    taps = (const c2_t<R> *)d.taps_loc;
  } else {
    const long h = g - locsz;
    j = d.L_loc + (int)(h / d.B_est);
    b = (int)(h & (d.B_est - 1));
    B = d.B_est;
    w = d.w_est;
    taps = (const c2_t<R> *)d.taps_est;
  }
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const unsigned long long ai = (unsigned)rp[d.L + j];
  const unsigned long long mask = (unsigned long long)d.n - 1;
  const In *x = (const In *)d.inputs[slot];
  c2_t<R> acc;
  acc.x = 0;
  acc.y = 0;
  // gathers issued 8 at a time, summed in increasing tap order
  for (int t0 = b; t0 < w; t0 += 8 * B) {
    c2_t<R> xv[8], hv[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int t = t0 + u * B;
      if (t < w) {
        const unsigned long long idx = ((unsigned long long)t * ai) & mask;
        xv[u] = cvt_in<R>(__ldg(x + idx));
        hv[u] = __ldg(taps + t);
      }
    }
#pragma unroll
    for (int u = 0; u < 8; u++)
      if (t0 + u * B < w) acc = cadd<R>(acc, cmul<R>(xv[u], hv[u]));
  }
  ((c2_t<R> *)d.xs)[(long)slot * d.xs_size + g] = acc;
}

// FP32 form of the fold with each bucket's taps split over S adjacent
// lanes (tap m of the bucket goes to lane m mod S), the S partial sums
// combined by shuffles.  A signal then spans S times as many threads as
// buckets, so the GPU's resident threads work on about one signal at a
// time: that signal's input stays in L2 while all its loops gather from it,
// instead of several signals' inputs contending for L2 and being fetched
// from DRAM repeatedly.  The summation order differs from the reference's,
// which the FP32 form does not reproduce anyway.
template <typename In, int S, int U = 4>
__device__ __forceinline__ void fold_split_thread(const V12Dev &d, int slot, long gt) {
  const long g = gt / S;
  const int part = (int)(gt % S);
  const bool live = g < d.xs_size;
  const long locsz = (long)d.L_loc * d.B_loc;
  int j = 0, b = 0, B = 1, w = 0;
  const float2 *taps = nullptr;
  if (live) {
    if (g < locsz) {
      j = (int)(g / d.B_loc);
      b = (int)(g & (d.B_loc - 1));
      B = d.B_loc;
      w = d.w_loc;
      taps = (const float2 *)d.taps_loc;
    } else {
      const long h = g - locsz;
      j = d.L_loc + (int)(h / d.B_est);
      b = (int)(h & (d.B_est - 1));
      B = d.B_est;
      w = d.w_est;
      taps = (const float2 *)d.taps_est;
    }
  }
  float2 acc = make_float2(0.f, 0.f);
  if (live) {
    const int *rp = d.rparams + (long)slot * d.rp_stride;
    const unsigned ai = (unsigned)rp[d.L + j], mask = (unsigned)d.n - 1u;
    const In *x = (const In *)d.inputs[slot];
    const int step = S * B;
    for (int t0 = b + part * B; t0 < w; t0 += U * step) {  // U gathers in flight
      float2 xv[U], hv[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int t = t0 + u * step;
        if (t < w) {
          xv[u] = cvt_in<float>(__ldg(x + (((unsigned)t * ai) & mask)));
          hv[u] = __ldg(taps + t);
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++)
        if (t0 + u * step < w) acc = cadd<float>(acc, cmul<float>(xv[u], hv[u]));
    }
  }
#pragma unroll
  for (int o = S / 2; o > 0; o >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
  }
  if (live && part == 0) ((float2 *)d.xs)[(long)slot * d.xs_size + g] = acc;
}

template <typename In, int S>
__global__ void __launch_bounds__(256) k_fold_split(V12Dev d) {
  fold_split_thread<In, S>(d, blockIdx.y, (long)blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------- smem layout --

template <typename R>
struct BucketSmem {
  static size_t bytes(int B, int num) {
    return (size_t)B * sizeof(c2_t<R>) + (size_t)B * sizeof(key_t<R>) + (264 + 64 + (size_t)num) * 4;
  }
};

template <typename R>
__device__ __forceinline__ void carve(unsigned char *smem, int B, c2_t<R> *&buf, key_t<R> *&keys,
                                      int *&hist, int *&scan, int *&Js) {
  buf = (c2_t<R> *)smem;
  keys = (key_t<R> *)(buf + B);
  hist = (int *)(keys + B);
  scan = hist + 264;
  Js = scan + 64;
}

// ------------------------------------------------------------------ comb --

template <typename R, int PER, typename In>
__device__ __forceinline__ void comb_block(const V12Dev &d, int c, int slot, unsigned char *smem) {
  const int W = d.W;
  c2_t<R> *buf;
  key_t<R> *keys;
  int *hist, *scan, *Js;
  carve<R>(smem, W, buf, keys, hist, scan, Js);
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const long sigma = d.n / W;
  const long offset = rp[2 * d.L + c];
  const In *x = (const In *)d.inputs[slot];
  for (int i = threadIdx.x; i < W; i += blockDim.x) buf[i] = cvt_in<R>(__ldg(x + offset + i * sigma));
  __syncthreads();
  block_fft<R, PER>(buf, W, dlog2(W), (const c2_t<R> *)d.tw_comb);
  for (int i = threadIdx.x; i < W; i += blockDim.x) keys[i] = pkey(cabs2<R>(buf[i]));
  __syncthreads();
  block_top_indices<key_t<R>>(keys, W, d.num, Js, hist, scan);
  unsigned *bits = d.comb_bits + (long)slot * ((W + 31) >> 5);
  for (int i = threadIdx.x; i < d.num; i += blockDim.x) atomicOr(&bits[Js[i] >> 5], 1u << (Js[i] & 31));
}

template <typename R, int PER, typename In>
__global__ void __launch_bounds__(1024) k_comb(V12Dev d) {
  extern __shared__ __align__(16) unsigned char smem[];
  comb_block<R, PER, In>(d, blockIdx.x, blockIdx.y, smem);
}

__device__ __forceinline__ void comb_list_block(const V12Dev &d, int slot) {
  __shared__ int scan[64];
  const int W = d.W;
  const int words = (W + 31) >> 5;
  const unsigned *bits = d.comb_bits + (long)slot * words;
  const int C = (words + blockDim.x - 1) / blockDim.x;
  const int lo = min(words, (int)threadIdx.x * C), hi = min(words, lo + C);
  int cnt = 0;
  for (int i = lo; i < hi; i++) cnt += __popc(bits[i]);
  int pre, dummy;
  int2 tot = block_exscan2(cnt, 0, pre, dummy, scan);
  int *list = d.comb_list + (long)slot * W;
  for (int i = lo; i < hi; i++) {
    unsigned v = bits[i];
    while (v) {
      int bpos = __ffs(v) - 1;
      list[pre++] = i * 32 + bpos;
      v &= v - 1;
    }
  }
  if (threadIdx.x == 0) d.counters[slot * CNT_STRIDE + CNT_COMB] = tot.x;
}

__global__ void __launch_bounds__(1024) k_comb_list(V12Dev d) { comb_list_block(d, blockIdx.x); }

// Voting of the location loops, one thread per (loop, selected bucket,
// position): positions p in [J*q - floor(q/2), +q) (mod n)
// map to frequencies f = p * a (mod n); each gets one vote (v2: only if
// f mod W is a comb residue); reaching the threshold appends f to the
// hits (computefourier-1.0-2.0.cc:91-116, :125-184).  Counters carry the
// exec's epoch in their upper 24 bits, so they never need clearing.
// One vote for frequency f: the counter is (epoch << 8) | votes, so a
// counter from an earlier execution restarts at 1.  The vote that reaches
// the threshold records the frequency (v1, and v2 in the voted mode).
// Tags only grow between clears of the counters, so an atomic max with
// (epoch << 8) resets a counter of an earlier execution to zero votes and
// leaves one of this execution alone; the atomic add that follows (same
// address, same thread: ordered after it) returns this vote's count.  One
// round trip, no compare-and-swap loop.  Plain v2 builds no hit list from
// its votes -- every frequency they reach is a comb candidate, all of
// which are estimated (computefourier-1.0-2.0.cc:505-512) -- so its votes
// only count: both atomics are reductions without a returned value, and
// the voting threads do not wait for them.
// v2's counters are stored residue-major, frequency f = rep W + r at
// r (n / W) + rep: the votes of a round fall on the few comb residues'
// blocks of n / W consecutive counters instead of all over the n of them,
// which keeps the touched counters dense in L2 and DRAM.
__device__ __forceinline__ void vote_one(const V12Dev &d, int slot, unsigned f, unsigned ep, unsigned *score,
                                         int *cnt) {
  unsigned *c = &score[f];
  if (d.version == 1) {
    const int lw = dlog2((unsigned)d.W), lr = dlog2((unsigned)d.n) - lw;
    c = &score[((f & ((unsigned)d.W - 1u)) << lr) | (f >> lw)];
  }
  atomicMax(c, ep << 8);
  if (d.version == 1 && !d.voted) {
    atomicAdd(c, 1u);
    return;
  }
  const unsigned nv = atomicAdd(c, 1u) + 1u;
  if ((int)(nv & 255u) == d.thresh) {
    atomicAdd(&cnt[CNT_VOTED], 1);
    if (d.version == 0 || d.voted) {
      const int pos = atomicAdd(&cnt[CNT_HITS], 1);
      if (pos < d.hit_cap)
        d.hits[(long)slot * d.hit_cap + pos] = (int)f;
      else
        atomicOr(&cnt[CNT_ERR], ERR_HIT_OVERFLOW);
    }
  }
}

__global__ void __launch_bounds__(256) k_vote(V12Dev d) {
  const int slot = blockIdx.y;
  const int q = d.q_loc, lq = dlog2(q);
  const long per_loop = (long)d.num << lq;
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= per_loop * d.L_loc) return;
  const int j = (int)(g / per_loop);
  const long e = g - (long)j * per_loop;
  const int *Js = d.J + ((long)slot * d.L + j) * d.num;
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const unsigned long long a = (unsigned)rp[j];
  const unsigned ep = (unsigned)rp[2 * d.L + d.comb_loops];
  const long n = d.n;
  const unsigned long long mask = (unsigned long long)n - 1;
  unsigned *score = d.score + (long)slot * n;
  const unsigned *bits = d.comb_bits + (long)slot * ((d.W + 31) >> 5);
  int *cnt = d.counters + slot * CNT_STRIDE;
  {
    const int i = (int)(e >> lq), o = (int)(e & (q - 1));
    const long low = ((long)Js[i] * q - (q >> 1) + n) & (long)mask;
    const unsigned long long p = ((unsigned long long)(low + o)) & mask;
    const unsigned f = (unsigned)((p * a) & mask);
    if (d.version == 1) {
      const unsigned r = f & (unsigned)(d.W - 1);
      if (!((bits[r >> 5] >> (r & 31)) & 1u)) return;
    }
    vote_one(d, slot, f, ep, score, cnt);
  }
}

// v2 voting by residue enumeration: for selected bucket J and comb residue
// r, the positions p of J's range whose frequency p a mod n lies in residue
// class r mod W are p = c (mod W) with c = r a^-1 mod W -- one thread per
// (loop, bucket, residue) visits exactly those.  Cheaper than the bitmap
// walk below when the residues are few against the bucket width (many
// light threads instead of a few threads with several votes each).
__global__ void __launch_bounds__(256) k_vote_comb(V12Dev d, int cmax) {
  const int slot = blockIdx.y;
  const long per_loop = (long)d.num * cmax;
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= per_loop * d.L_loc) return;
  const int j = (int)(g / per_loop);
  const long e = g - (long)j * per_loop;
  const int i = (int)(e / cmax), ri = (int)(e - (long)i * cmax);
  int *cnt = d.counters + slot * CNT_STRIDE;
  if (ri >= cnt[CNT_COMB]) return;
  const unsigned r = (unsigned)d.comb_list[(long)slot * d.W + ri];
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const unsigned a = (unsigned)rp[j], ai = (unsigned)rp[d.L + j];
  const unsigned ep = (unsigned)rp[2 * d.L + d.comb_loops];
  const unsigned mask = (unsigned)d.n - 1u, wm = (unsigned)d.W - 1u;
  const int q = d.q_loc;
  const int J = d.J[((long)slot * d.L + j) * d.num + i];
  const unsigned low = ((unsigned)J * (unsigned)q - (unsigned)(q >> 1) + (unsigned)d.n) & mask;
  const unsigned c = (r * ai) & wm;
  unsigned *score = d.score + (long)slot * d.n;
  for (unsigned k = (c - low) & wm; k < (unsigned)q; k += (unsigned)d.W) {
    const unsigned p = (low + k) & mask;
    vote_one(d, slot, (p * a) & mask, ep, score, cnt);
  }
}

// v2 voting by comb-key bitmap.  In location loop j a position p votes iff
// its frequency p a mod n lies in an approved comb residue class, i.e. iff
// p mod W is in K_j = {r ai mod W : r approved} (a ai = 1 mod W, W | n).  A
// block builds K_j as a W-bit bitmap in shared memory; then each thread
// takes 32 consecutive positions of one selected bucket's range at a time:
// the 32 bits starting at (low + o) mod W (two words, funnel shift) name
// exactly the positions that vote.  The reference walks the approved
// residues in the same way through sorted (residue, key) pairs
// (computefourier-1.0-2.0.cc:125-184); the votes are the same, in any order.
constexpr int VB_BUCKETS = 64;   // selected buckets per block

__device__ __forceinline__ void vote_bits_block(const V12Dev &d, int j, int i0, int slot, unsigned *kb) {
  const int W = d.W, nw = W >> 5, L = d.L;
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const unsigned a = (unsigned)rp[j], ai = (unsigned)rp[L + j];
  const unsigned ep = (unsigned)rp[2 * L + d.comb_loops];
  const unsigned mask = (unsigned)d.n - 1u, wm = (unsigned)W - 1u;
  int *cnt = d.counters + slot * CNT_STRIDE;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) kb[w] = 0u;
  __syncthreads();
  const int ncomb = cnt[CNT_COMB];
  const int *list = d.comb_list + (long)slot * W;
  for (int t = threadIdx.x; t < ncomb; t += blockDim.x) {
    const unsigned c = ((unsigned)list[t] * ai) & wm;
    atomicOr(&kb[c >> 5], 1u << (c & 31));
  }
  __syncthreads();
  const int q = d.q_loc, nch = (q + 31) >> 5;
  const int i1 = min(d.num, i0 + VB_BUCKETS);
  const int tasks = (i1 - i0) * nch;
  const int *Js = d.J + ((long)slot * L + j) * d.num;
  unsigned *score = d.score + (long)slot * d.n;
  for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
    const int i = i0 + t / nch, o0 = (t - (t / nch) * nch) << 5;
    const unsigned low = ((unsigned)Js[i] * (unsigned)q - (unsigned)(q >> 1) + (unsigned)d.n) & mask;
    const unsigned b0 = (low + (unsigned)o0) & wm;
    const unsigned w0 = b0 >> 5;
    unsigned word = __funnelshift_r(kb[w0], kb[(w0 + 1) & (unsigned)(nw - 1)], b0 & 31u);
    const int rem = q - o0;
    if (rem < 32) word &= (1u << rem) - 1u;
    while (word) {
      const int k = __ffs(word) - 1;
      word &= word - 1u;
      const unsigned p = (low + (unsigned)(o0 + k)) & mask;
      vote_one(d, slot, (p * a) & mask, ep, score, cnt);
    }
  }
}

__global__ void __launch_bounds__(256) k_vote_bits(V12Dev d) {
  extern __shared__ unsigned vb_keys[];
  const int nbc = (d.num + VB_BUCKETS - 1) / VB_BUCKETS;
  const int j = blockIdx.x / nbc;
  vote_bits_block(d, j, (blockIdx.x - j * nbc) * VB_BUCKETS, blockIdx.y, vb_keys);
}

// ---------------------------------------------------------------- bucket --

template <typename R, int PER>
__device__ __forceinline__ void bucket_block(const V12Dev &d, int j, int slot, unsigned char *smem) {
  const bool loc = j < d.L_loc;
  const int B = loc ? d.B_loc : d.B_est;
  const long off = loc ? (long)j * d.B_loc : (long)d.L_loc * d.B_loc + (long)(j - d.L_loc) * d.B_est;
  c2_t<R> *buf;
  key_t<R> *keys;
  int *hist, *scan, *Js;
  carve<R>(smem, B, buf, keys, hist, scan, Js);
  c2_t<R> *xs = (c2_t<R> *)d.xs + (long)slot * d.xs_size + off;
  for (int i = threadIdx.x; i < B; i += blockDim.x) buf[i] = xs[i];
  __syncthreads();
  block_fft<R, PER>(buf, B, dlog2(B), (const c2_t<R> *)(loc ? d.tw_loc : d.tw_est));
  float2 *xs32 = d.xs32 ? (float2 *)d.xs32 + (long)slot * d.xs_size + off : nullptr;
  // grouped layout (xs_perm): bucket i goes to (i mod T) * G + i / T
  const int lg = d.xs_perm, lt = dlog2(B) - lg;
  const int tmask = (1 << lt) - 1;
  for (int i = threadIdx.x; i < B; i += blockDim.x) {
    const c2_t<R> v = buf[i];
    const int p = lg ? ((i & tmask) << lg) | (i >> lt) : i;
    xs[p] = v;
    if (xs32) xs32[p] = make_float2((float)v.x, (float)v.y);
    keys[i] = pkey(cabs2<R>(v));
  }
  __syncthreads();
  block_top_indices<key_t<R>>(keys, B, d.num, Js, hist, scan);
  int *Jg = d.J + ((long)slot * d.L + j) * d.num;
  for (int i = threadIdx.x; i < d.num; i += blockDim.x) Jg[i] = Js[i];
}

template <typename R, int PER>
__global__ void __launch_bounds__(1024, (sizeof(R) == 4 && PER == 1) ? 2 : 1) k_bucket(V12Dev d) {
  extern __shared__ __align__(16) unsigned char smem[];
  bucket_block<R, PER>(d, blockIdx.x, blockIdx.y, smem);
}

// ------------------------------------------------- FFTs beyond one CTA --

// One Stockham stage over `narr` arrays of N points per slot.
template <typename R>
__global__ void __launch_bounds__(256) k_fft_stage(const c2_t<R> *src, c2_t<R> *dst, int N, int Ns, int radix,
                                                   long arr_stride, int narr, long slot_stride,
                                                   const c2_t<R> *tw) {
  const int slot = blockIdx.y;
  const int per = N / radix;
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long)narr * per) return;
  const int arr = (int)(g / per), j = (int)(g - (long)arr * per);
  const long base = (long)slot * slot_stride + (long)arr * arr_stride;
  stockham_stage<R>(src + base, dst + base, N, Ns, radix, j, tw);
}

// Power, top-2k selection and voting of loop j after a global-memory FFT.
template <typename R>
__global__ void __launch_bounds__(1024) k_select_vote(V12Dev d) {
  __shared__ int hist[264], scan[64];
  extern __shared__ int Js[];
  const int j = blockIdx.x, slot = blockIdx.y;
  const bool loc = j < d.L_loc;
  const int B = loc ? d.B_loc : d.B_est;
  const long off = loc ? (long)j * d.B_loc : (long)d.L_loc * d.B_loc + (long)(j - d.L_loc) * d.B_est;
  const c2_t<R> *xs = (const c2_t<R> *)d.xs + (long)slot * d.xs_size + off;
  if (d.xs32) {
    float2 *xs32 = (float2 *)d.xs32 + (long)slot * d.xs_size + off;
    for (int i = threadIdx.x; i < B; i += blockDim.x) xs32[i] = make_float2((float)xs[i].x, (float)xs[i].y);
  }
  block_top_indices_f<key_t<R>>([xs](int i) { return pkey(cabs2<R>(xs[i])); }, B, d.num, Js, hist, scan);
  int *Jg = d.J + ((long)slot * d.L + j) * d.num;
  for (int i = threadIdx.x; i < d.num; i += blockDim.x) Jg[i] = Js[i];
}

template <typename R, typename In>
__global__ void __launch_bounds__(256) k_comb_gather(V12Dev d) {
  const int slot = blockIdx.z, c = blockIdx.y, W = d.W;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W) return;
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const long sigma = d.n / W, offset = rp[2 * d.L + c];
  const In *x = (const In *)d.inputs[slot];
  ((c2_t<R> *)d.comb_buf)[((long)slot * d.comb_loops + c) * W + i] = cvt_in<R>(__ldg(x + offset + i * sigma));
}

template <typename R>
__global__ void __launch_bounds__(1024) k_comb_select(V12Dev d) {
  __shared__ int hist[264], scan[64];
  extern __shared__ int Js[];
  const int c = blockIdx.x, slot = blockIdx.y, W = d.W;
  const c2_t<R> *v = (const c2_t<R> *)d.comb_buf + ((long)slot * d.comb_loops + c) * W;
  block_top_indices_f<key_t<R>>([v](int i) { return pkey(cabs2<R>(v[i])); }, W, d.num, Js, hist, scan);
  unsigned *bits = d.comb_bits + (long)slot * ((W + 31) >> 5);
  for (int i = threadIdx.x; i < d.num; i += blockDim.x) atomicOr(&bits[Js[i] >> 5], 1u << (Js[i] & 31));
}

// FFT of `narr` arrays per slot held at a (ping) with b as scratch; the
// result ends in a.  Stage sequence of block_fft.
template <typename R>
static cudaError_t global_fft(c2_t<R> *a, c2_t<R> *b, int N, int narr, long arr_stride, long slot_stride,
                              int nslots, const c2_t<R> *tw, cudaStream_t s) {
  int logN = 0;
  while ((1 << logN) < N) logN++;
  c2_t<R> *src = a, *dst = b;
  int Ns = 1, launches = 0;
  auto stage = [&](int radix) -> cudaError_t {
    const long work = (long)narr * (N / radix);
    dim3 grid((unsigned)((work + 255) / 256), nslots);
    k_fft_stage<R><<<grid, 256, 0, s>>>(src, dst, N, Ns, radix, arr_stride, narr, slot_stride, tw);
    launches++;
    c2_t<R> *t = src;
    src = dst;
    dst = t;
    return cudaGetLastError();
  };
  cudaError_t e;
  if (logN & 1) {
    if ((e = stage(2))) return e;
    Ns = 2;
  }
  while (Ns < N) {
    if ((e = stage(4))) return e;
    Ns *= 4;
  }
  note_launches(launches);
  if (src != a) {  // odd number of stages: bring the result home
    for (int sl = 0; sl < nslots; sl++) {
      if ((e = cudaMemcpyAsync(a + sl * slot_stride, src + sl * slot_stride,
                               sizeof(c2_t<R>) * ((narr - 1) * arr_stride + N), cudaMemcpyDeviceToDevice, s)))
        return e;
    }
  }
  return cudaSuccess;
}

// -------------------------------------------------------------- estimate --

// Knuth's merge-exchange sorting network (TAOCP vol. 3, 5.2.2, Algorithm M)
// for N elements, generated at compile time; used through Cswap so that
// every comparator's indices are constants (the values stay in registers).
template <int N>
struct SortNet {
  static constexpr int count() {
    if (N < 2) return 0;
    int t = 0;
    while ((1 << t) < N) t++;
    int c = 0;
    for (int p = 1 << (t - 1); p > 0; p >>= 1) {
      int q = 1 << (t - 1), r = 0, dd = p;
      for (;;) {
        for (int i = 0; i + dd < N; i++)
          if ((i & p) == r) c++;
        if (q == p) break;
        dd = q - p;
        q >>= 1;
        r = p;
      }
    }
    return c;
  }
  static constexpr int C = count();
  int a[C > 0 ? C : 1], b[C > 0 ? C : 1];
  constexpr SortNet() : a(), b() {
    if (N < 2) return;
    int t = 0;
    while ((1 << t) < N) t++;
    int c = 0;
    for (int p = 1 << (t - 1); p > 0; p >>= 1) {
      int q = 1 << (t - 1), r = 0, dd = p;
      for (;;) {
        for (int i = 0; i + dd < N; i++)
          if ((i & p) == r) {
            a[c] = i;
            b[c] = i + dd;
            c++;
          }
        if (q == p) break;
        dd = q - p;
        q >>= 1;
        r = p;
      }
    }
  }
};

template <int N> struct NetOf { static constexpr SortNet<N> net{}; };

template <int N, int c, int C>
struct Cswap {
  static __device__ __forceinline__ void run(float (&v)[N]) {
    constexpr int i = NetOf<N>::net.a[c], j = NetOf<N>::net.b[c];
    const float x = v[i], y = v[j];
    v[i] = fminf(x, y);
    v[j] = fmaxf(x, y);
    Cswap<N, c + 1, C>::run(v);
  }
};
template <int N, int C>
struct Cswap<N, C, C> {
  static __device__ __forceinline__ void run(float (&)[N]) {}
};

template <int N>
__device__ __forceinline__ void sort_net(float (&v)[N]) {
  Cswap<N, 0, SortNet<N>::C>::run(v);
}

// Parberry's pairwise sorting network on P = 2^t wires (I. Parberry, "The
// pairwise sorting network", Parallel Processing Letters 2(2-3), 1992):
// calls f(i, j), i < j, for its comparators in order.  Its first half sorts
// pairs, then quadruples, ... of a bitonic-free layout; its second half
// merges with comparators (b - d a, b).
template <typename F>
constexpr void pairwise_net(int P, F &&f) {
  int a = 1;
  for (; a < P; a *= 2) {
    int b = a, c = 0;
    while (b < P) {
      f(b - a, b);
      b++;
      c = (c + 1) % a;
      if (c == 0) b += a;
    }
  }
  a /= 4;
  for (int e = 1; a > 0; a /= 2, e = 2 * e + 1) {
    for (int d = e; d > 0; d /= 2) {
      int b = (d + 1) * a, c = 0;
      while (b < P) {
        f(b - d * a, b);
        b++;
        c = (c + 1) % a;
        if (c == 0) b += a;
      }
    }
  }
}

constexpr int pow2_ceil(int n) {
  int p = 1;
  while (p < n) p *= 2;
  return p;
}

// A selection network for element M of N values: the pairwise network on
// P = pow2_ceil(N) wires restricted to the N wires [s, s + N) -- with -inf
// below s and +inf from s + N on, a comparator touching an outside wire
// moves nothing, so the inside comparators sort any N values -- then
// pruned to output M by backward liveness: a comparator whose outputs are
// both dead is dropped, one with a single live output keeps only its min
// or its max.  The offset s with the fewest min/max operations is chosen
// at compile time (lower median of 20: 125 operations, against 143 for
// the pruned merge-exchange network).  Comparator kinds: 1 both outputs,
// 2 min only, 3 max only.
template <int N, int M>
struct SelNet {
  static constexpr int P = pow2_ceil(N);
  static constexpr int FULL = [] {
    int c = 0;
    pairwise_net(P, [&](int, int) { c++; });
    return c;
  }();
  int C = 0, ops = 0;
  signed char a[FULL > 0 ? FULL : 1] = {}, b[FULL > 0 ? FULL : 1] = {}, kind[FULL > 0 ? FULL : 1] = {};
  // the network at offset s, pruned: fills a, b, kind, C; returns its operation count
  constexpr int build(int s) {
    int fa[FULL > 0 ? FULL : 1] = {}, fb[FULL > 0 ? FULL : 1] = {};
    int n = 0;
    pairwise_net(P, [&](int i, int j) {
      if (i >= s && j < s + N) {
        fa[n] = i - s;
        fb[n] = j - s;
        n++;
      }
    });
    bool live[N] = {};
    live[M] = true;
    signed char k[FULL > 0 ? FULL : 1] = {};
    int cnt = 0, o = 0;
    for (int c = n - 1; c >= 0; c--) {
      const bool li = live[fa[c]], lj = live[fb[c]];
      k[c] = li && lj ? 1 : li ? 2 : lj ? 3 : 0;
      if (li || lj) {
        live[fa[c]] = live[fb[c]] = true;
        cnt++;
        o += (li && lj) ? 2 : 1;
      }
    }
    C = 0;
    for (int c = 0; c < n; c++)
      if (k[c]) {
        a[C] = (signed char)fa[c];
        b[C] = (signed char)fb[c];
        kind[C] = k[c];
        C++;
      }
    ops = o;
    return o;
  }
  constexpr SelNet() {
    if (N < 2) return;
    int best = -1, bs = 0;
    for (int s = 0; s + N <= P; s++) {
      const int o = build(s);
      if (best < 0 || o < best) {
        best = o;
        bs = s;
      }
    }
    build(bs);
  }
};
template <int N, int M> struct SelOf { static constexpr SelNet<N, M> net{}; };

template <int N, int M, int c, int C>
struct Cmed {
  static __device__ __forceinline__ void run(float (&v)[N]) {
    constexpr int i = SelOf<N, M>::net.a[c], j = SelOf<N, M>::net.b[c];
    constexpr int k = SelOf<N, M>::net.kind[c];
    if constexpr (k == 1) {
      const float x = v[i], y = v[j];
      v[i] = fminf(x, y);
      v[j] = fmaxf(x, y);
    } else if constexpr (k == 2) {
      v[i] = fminf(v[i], v[j]);
    } else {
      v[j] = fmaxf(v[i], v[j]);
    }
    Cmed<N, M, c + 1, C>::run(v);
  }
};
template <int N, int M, int C>
struct Cmed<N, M, C, C> {
  static __device__ __forceinline__ void run(float (&)[N]) {}
};

// Element M of v in sorted order (v is overwritten).
template <int N, int M>
__device__ __forceinline__ float select_net(float (&v)[N]) {
  Cmed<N, M, 0, SelOf<N, M>::net.C>::run(v);
  return v[M];
}

// Lower median of v[0..Lr): the pruned network when Lr == LN is known at
// compile time, else a full sort (v is overwritten).
template <int LN, bool EXACT>
__device__ __forceinline__ float lower_median(float (&v)[LN], int Lr) {
  if constexpr (EXACT) {
    return select_net<LN, (LN - 1) / 2>(v);
  } else {
    sort_net(v);
    const int m = (Lr - 1) >> 1;
    float r = 0;
#pragma unroll
    for (int j = 0; j < LN; j++)
      if (j == m) r = v[j];
    return r;
  }
}

__device__ __forceinline__ long long okey(double v) {
  long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

struct Slot {
  int q, B, lq;
  long off;
};

__device__ __forceinline__ Slot loop_slot(const V12Dev &d, int j) {
  const bool loc = j < d.L_loc;
  Slot s;
  s.q = loc ? d.q_loc : d.q_est;
  s.B = loc ? d.B_loc : d.B_est;
  s.lq = dlog2(s.q);
  s.off = loc ? (long)j * d.B_loc : (long)d.L_loc * d.B_loc + (long)(j - d.L_loc) * d.B_est;
  return s;
}

// bucket and window index of frequency f in loop j
// (computefourier-1.0-2.0.cc:370-378)
__device__ __forceinline__ void bucket_of(const V12Dev &d, const Slot &s, unsigned f, unsigned long long ai,
                                          int &hashed, int &m) {
  // n is a power of two below 2^32: the product's low bits suffice
  const unsigned p = (f * (unsigned)ai) & ((unsigned)d.n - 1u);
  hashed = (int)(p >> s.lq);
  int dist = (int)(p & (s.q - 1));
  if (dist > (s.q >> 1)) {
    hashed = (hashed + 1) & (s.B - 1);
    dist -= s.q;
  }
  m = dist + ((s.q - 1) >> 1);
}

// FP32 value x_samp[bucket] / filter.freq[dist] with the reference's sign
// (conjugate, computefourier-1.0-2.0.cc:383-398), via g = conj(h)/|h|^2.
// scale receives (|a| + |b|)(|g.x| + |g.y|), a bound on the terms summed.
__device__ __forceinline__ void value32(const V12Dev &d, const float2 *xs, const float2 *win_loc,
                                        const float2 *win_est, int j, unsigned f, unsigned long long ai, float &re,
                                        float &im, float &scale) {
  const Slot s = loop_slot(d, j);
  int hashed, m;
  bucket_of(d, s, f, ai, hashed, m);
  const float2 v = xs[s.off + hashed];
  const float2 g = __ldg((j < d.L_loc ? win_loc : win_est) + m);
  re = v.x * g.x + v.y * g.y;
  im = v.x * g.y - v.y * g.x;
  scale = (fabsf(v.x) + fabsf(v.y)) * (fabsf(g.x) + fabsf(g.y));
}

// FP64 value, the reference's exact operation sequence:
// ((a c + b d) / (c^2 + d^2), (a d - b c) / (c^2 + d^2))
__device__ __forceinline__ double2 value64(const V12Dev &d, const double2 *xs, int j, unsigned f,
                                           unsigned long long ai) {
  const Slot s = loop_slot(d, j);
  int hashed, m;
  bucket_of(d, s, f, ai, hashed, m);
  const double2 v = xs[s.off + hashed];
  const double2 *wp = (const double2 *)(j < d.L_loc ? d.win_loc : d.win_est) + 2 * m;
  const double2 h = __ldg(wp);
  const double den = __ldg(wp + 1).x;
  using A = Ar<double>;
  return make_double2(A::div(A::add(A::mul(v.x, h.x), A::mul(v.y, h.y)), den),
                      A::div(A::sub(A::mul(v.x, h.y), A::mul(v.y, h.x)), den));
}

// Exact lower medians of all L FP64 values (used when the FP32 pre-selection
// cannot prove which element is the median, e.g. ties).
__device__ __noinline__ double2 median64_exact(const V12Dev &d, const double2 *xs, const int *rp, unsigned f) {
  double vre[32], vim[32];
  const int L = d.L;
  for (int j = 0; j < L; j++) {
    const double2 v = value64(d, xs, j, f, (unsigned)rp[L + j]);
    vre[j] = v.x;
    vim[j] = v.y;
  }
  const int m = (L - 1) >> 1;
  double mre = 0, mim = 0;
  for (int i = 0; i < L; i++) {
    const long long ki = okey(vre[i]), kj = okey(vim[i]);
    int rr = 0, ri = 0;
    for (int jj = 0; jj < L; jj++) {
      const long long a = okey(vre[jj]), b = okey(vim[jj]);
      rr += (a < ki) || (jj < i && a == ki);
      ri += (b < kj) || (jj < i && b == kj);
    }
    if (rr == m) mre = vre[i];
    if (ri == m) mim = vim[i];
  }
  return make_double2(mre, mim);
}

// Number of candidates of a slot: v1 hits, v2 every comb candidate (or,
// in the opt-in voted mode, v2 hits).
__device__ __forceinline__ long cand_total(const V12Dev &d, int slot) {
  const int *cnt = d.counters + slot * CNT_STRIDE;
  if (d.version == 0 || d.voted) return min(cnt[CNT_HITS], d.hit_cap);
  return (long)cnt[CNT_COMB] * (d.n / d.W);
}

// Frequency of candidate h (< cand_total) of a slot.  v2 candidates are
// numbered residue-major, h = residue index * (n / W) + repetition, so the
// lanes of a warp share a comb residue: for each loop their window index
// (which depends on the residue only when the window length n / B divides
// W) is one broadcast load.  The output is a set; its order is free.
__device__ __forceinline__ unsigned cand_freq(const V12Dev &d, int slot, long h) {
  if (d.version == 0 || d.voted) return (unsigned)d.hits[(long)slot * d.hit_cap + h];
  const unsigned reps = (unsigned)(d.n / d.W);  // a power of two
  const unsigned hu = (unsigned)h, ridx = hu >> (__ffs(reps) - 1), rep = hu & (reps - 1);
  return rep * (unsigned)d.W + (unsigned)d.comb_list[(long)slot * d.W + ridx];
}

// Publishes a slot's output count (and the overflow flag).
__device__ __forceinline__ void publish_count(const V12Dev &d, int slot, long total) {
  int *cnt = d.counters + slot * CNT_STRIDE;
  const int c = (int)min(total, (long)d.out_cap);
  cnt[CNT_OUT] = c;
  if (d.out_count) d.out_count[slot] = c;
  if (total > d.out_cap) atomicOr(&cnt[CNT_ERR], ERR_OUT_OVERFLOW);
}

// Candidate h of a slot; false when h is past the end.  Thread h == 0
// publishes the count.
__device__ __forceinline__ bool candidate(const V12Dev &d, int slot, long h, unsigned &f) {
  const long total = cand_total(d, slot);
  if (h == 0) publish_count(d, slot, total);
  if (h >= total || h >= d.out_cap) return false;
  f = cand_freq(d, slot, h);
  return true;
}

// Picks the lower-median element of v[0..Lr): FP32 approximations whose
// exact values lie within +-e[j] of v[j].  Returns its index if it is
// provably the exact lower median -- exactly m = (Lr-1)/2 intervals lie
// wholly below its interval and Lr-1-m wholly above -- else -1.
// Per-element bounds matter on clean signals: most candidates' values are
// tiny, and a bound taken from the largest value of the loop set (a tone's)
// would swallow their differences.
template <int LN, bool EXACT>
__device__ __forceinline__ int proven_median(const float (&v)[LN], const float (&e)[LN], int Lr) {
  float s[LN];
#pragma unroll
  for (int j = 0; j < LN; j++) s[j] = v[j];
  const int m = (Lr - 1) >> 1;
  const float med = lower_median<LN, EXACT>(s, Lr);
  int idx = -1;
  float em = 0.f;
#pragma unroll
  for (int j = LN - 1; j >= 0; j--)
    if (j < Lr && v[j] == med) {
      idx = j;
      em = e[j];
    }
  int below = 0, above = 0;
#pragma unroll
  for (int j = 0; j < LN; j++) {
    if (j < Lr && j != idx) {
      below += (v[j] + e[j] < med - em);
      above += (v[j] - e[j] > med + em);
    }
  }
  return (below == m && above == Lr - 1 - m) ? idx : -1;
}

// Estimation work is dealt in chunks of one candidate per thread from a
// per-slot queue (counters[CNT_EST]).  A block starts on the slot its SM is
// assigned (%smid modulo the slot count) and moves on only when that slot
// is exhausted, so the blocks resident on one SM read one slot's bucket
// array and its random lookups hit in L1 far more often than when an SM
// serves several slots at once.
__device__ __forceinline__ unsigned sm_id() {
  unsigned r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}

struct EstChunk {
  int slot;
  long base, end;
};

__device__ __forceinline__ bool next_chunk(const V12Dev &d, int nslots, int chunk, int &slot, int &visited,
                                           EstChunk &out) {
  __shared__ EstChunk sc;
  __syncthreads();  // the previous chunk is read by every thread
  if (threadIdx.x == 0) {
    sc.base = -1;
    while (visited < nslots) {
      const long total = min(cand_total(d, slot), (long)d.out_cap);
      const long c = (long)atomicAdd(&d.counters[slot * CNT_STRIDE + CNT_EST], 1) * chunk;
      if (c < total) {
        sc.slot = slot;
        sc.base = c;
        sc.end = min(c + chunk, total);
        break;
      }
      slot = slot + 1 == nslots ? 0 : slot + 1;
      visited++;
    }
  }
  __syncthreads();
  out = sc;
  return out.base >= 0;
}

__device__ __forceinline__ void publish_all(const V12Dev &d, int nslots) {
  if (blockIdx.x == 0)
    for (int sl = threadIdx.x; sl < nslots; sl += blockDim.x) publish_count(d, sl, cand_total(d, sl));
}

// Resident 128-thread blocks per SM the estimation kernels are compiled
// for (registers per thread = 65536 / (128 * blocks), without spills).
constexpr int est32_blocks(int LN) { return LN <= 18 ? 8 : LN <= 24 ? 6 : 5; }
constexpr int est64_blocks(int LN) { return LN <= 14 ? 6 : LN <= 20 ? 5 : 4; }

// One FP32 candidate h (< the slot's total) by random bucket lookups.
template <int LN, bool EXACT>
__device__ __forceinline__ void est32_candidate(const V12Dev &d, int slot, long h) {
  const float2 *wl = (const float2 *)d.win_loc, *we = (const float2 *)d.win_est;
  const int Lr = EXACT ? LN : d.L;
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const float2 *xs = (const float2 *)d.xs + (long)slot * d.xs_size;
  const unsigned f = cand_freq(d, slot, h);
  float re[LN], im[LN];
#pragma unroll
  for (int j = 0; j < LN; j++) {
    if (EXACT || j < Lr) {
      float sc;
      value32(d, xs, wl, we, j, f, (unsigned)rp[d.L + j], re[j], im[j], sc);
    } else {
      re[j] = INFINITY;
      im[j] = INFINITY;
    }
  }
  const float mre = lower_median<LN, EXACT>(re, Lr), mim = lower_median<LN, EXACT>(im, Lr);
  const long o = (long)slot * d.out_stride + h;
  d.out_idx[o] = (int)f;
  ((float2 *)d.out_val)[o] = make_float2(mre, mim);
}

// FP32 form: values and medians in FP32.
template <int LN, bool EXACT>
__global__ void __launch_bounds__(128, est32_blocks(LN)) k_estimate32(V12Dev d, int nslots) {
  publish_all(d, nslots);
  const float2 *wl = (const float2 *)d.win_loc, *we = (const float2 *)d.win_est;
  const int Lr = EXACT ? LN : d.L;
  int slot = (int)(sm_id() % (unsigned)nslots), visited = 0;
  EstChunk ck;
  while (next_chunk(d, nslots, blockDim.x, slot, visited, ck)) {
    const int *rp = d.rparams + (long)ck.slot * d.rp_stride;
    const float2 *xs = (const float2 *)d.xs + (long)ck.slot * d.xs_size;
    const long h = ck.base + threadIdx.x;  // one candidate per thread and chunk
    if (h < ck.end) {
      const unsigned f = cand_freq(d, ck.slot, h);
      float re[LN], im[LN];
#pragma unroll
      for (int j = 0; j < LN; j++) {
        if (EXACT || j < Lr) {
          float sc;
          value32(d, xs, wl, we, j, f, (unsigned)rp[d.L + j], re[j], im[j], sc);
        } else {
          re[j] = INFINITY;
          im[j] = INFINITY;
        }
      }
      const float mre = lower_median<LN, EXACT>(re, Lr), mim = lower_median<LN, EXACT>(im, Lr);
      const long o = (long)ck.slot * d.out_stride + h;
      d.out_idx[o] = (int)f;
      ((float2 *)d.out_val)[o] = make_float2(mre, mim);
    }
  }
}

// FP64 form, bit-exact: the median element is chosen on FP32 copies with a
// rigorous error bound, then only that element is divided in FP64 (the
// reference's exact operation sequence); anything not provable (ties,
// near-ties) takes the all-exact path.
template <int LN, bool EXACT>
__global__ void __launch_bounds__(128, est64_blocks(LN)) k_estimate64(V12Dev d, int nslots) {
  publish_all(d, nslots);
  const float2 *wl = (const float2 *)d.win32_loc, *we = (const float2 *)d.win32_est;
  const int Lr = EXACT ? LN : d.L;
  int slot = (int)(sm_id() % (unsigned)nslots), visited = 0;
  EstChunk ck;
  while (next_chunk(d, nslots, blockDim.x, slot, visited, ck)) {
    const int *rp = d.rparams + (long)ck.slot * d.rp_stride;
    const float2 *xs32 = (const float2 *)d.xs32 + (long)ck.slot * d.xs_size;
    const double2 *xs = (const double2 *)d.xs + (long)ck.slot * d.xs_size;
    const long h = ck.base + threadIdx.x;  // one candidate per thread and chunk
    if (h < ck.end) {
      const unsigned f = cand_freq(d, ck.slot, h);
      float re[LN], im[LN], eb[LN];
#pragma unroll
      for (int j = 0; j < LN; j++) {
        if (EXACT || j < Lr) {
          float sc;
          value32(d, xs32, wl, we, j, f, (unsigned)rp[d.L + j], re[j], im[j], sc);
          // |exact - approx| <= 2^-22 * scale: each FP32 operand carries one
          // rounding (2^-24 relative), plus two products and a sum; the
          // bound below has a 4x margin, which also covers the rounding of
          // the comparisons in proven_median.
          eb[j] = sc * 0x1p-20f + 1e-30f;
        } else {
          re[j] = INFINITY;
          im[j] = INFINITY;
          eb[j] = 0.f;
        }
      }
      const int ir = proven_median<LN, EXACT>(re, eb, Lr);
      const int ii = proven_median<LN, EXACT>(im, eb, Lr);
      double2 res;
      if (ir >= 0 && ii >= 0) {
        res.x = value64(d, xs, ir, f, (unsigned)rp[d.L + ir]).x;
        res.y = value64(d, xs, ii, f, (unsigned)rp[d.L + ii]).y;
      } else {
        res = median64_exact(d, xs, rp, f);
        atomicAdd(&d.counters[ck.slot * CNT_STRIDE + CNT_EXACT], 1);
      }
      const long o = (long)ck.slot * d.out_stride + h;
      d.out_idx[o] = (int)f;
      ((double2 *)d.out_val)[o] = res;
    }
  }
}

// ------------------------------------------- estimate by comb residue --
//
// Plain v2 estimates every comb candidate f = rep * W + r (r a comb residue,
// rep < R = n / W).  When W is a multiple of q = n / B, loop j hashes f to
//   p = f ai mod n = (r ai mod n) + W (rep ai mod R)     (mod n)
// so the window index p mod q -- and the bucket's rounding carry -- depend
// on r only, and the bucket is b = c0 + (W / q) (rep ai mod R) (mod B)
// (computefourier-1.0-2.0.cc:370-378).  ai is odd, so rep -> rep ai mod R
// is a bijection: the R candidates of a residue read R distinct buckets,
// and a group of G = R / S of them with the same rep mod S reads the G
// buckets congruent to one value mod T = B / G.  The bucket kernel stores
// each loop's buckets grouped that way (xs_perm), which makes a group's
// buckets G consecutive entries.
//
// One CTA estimates EC_THREADS candidates (whole groups): one thread per
// (group, loop) computes that pair's table entry and issues one bulk
// asynchronous copy (cp.async.bulk, completion counted in bytes on an
// mbarrier that also counts the table writers' arrivals) of the group's
// bucket run into shared memory; each thread waits on the mbarrier, then
// reads its candidate's value of every loop from shared memory -- lanes i
// of a warp read entries (rot + i ai) mod G, distinct mod 16, so without
// bank conflicts -- and takes the lower medians.  Several CTAs per SM
// overlap one CTA's copies with the others' arithmetic.  Output position
// h = residue index * R + group * G + i; the output is a set, so its order
// is free.

constexpr int EC_THREADS = 256;            // candidates per CTA of k_estimate_comb32
constexpr int EC_MAXL = 32;
constexpr long EC_WAIT_POLLS = 1L << 22;

struct EcVal {   // one (group, loop): entry i of the group reads run[(rot + i ai) mod G]
  int rot;
  unsigned ai;
  float gx, gy;  // FP32 window value conj(h) / |h|^2
};

// Shared state of one item of NTH candidates (groups of G >= 32).
template <int NTH>
struct EcShared {
  EcVal v[(NTH / 32) * EC_MAXL];
  int res[NTH / 32], grp[NTH / 32];
  unsigned long long bar;
};

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(unsigned long long *bar, unsigned parity) {
  unsigned done;
  asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
               : "=r"(done)
               : "r"(smem_u32(bar)), "r"(parity)
               : "memory");
  return done != 0;
}

// at most EC_WAIT_POLLS polls (each may suspend the thread for a bounded time)
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity) {
  for (long i = 0; i < EC_WAIT_POLLS; i++)
    if (mbar_test(bar, parity)) return true;
  return false;
}

// Bulk copy global -> this CTA's shared memory, completion counted in bytes
// on `bar` (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Staging of candidates [h0, h0 + NTH) of a slot (h0 < total, the slot's
// candidate count; total is a multiple of G, so a group is wholly live or
// wholly past the end): one thread per (group, loop) writes the group's
// table entry for that loop and issues one bulk copy of the group's run of
// FP32 bucket values (xsrc) into seg (L * NTH float2); then every thread
// waits.  Every thread of a block of NTH threads calls it.  The mbarrier in
// sh is initialised here; a caller that stages another item with the same
// sh invalidates it first, after a block barrier.  srcmw (optional)
// receives each (group, loop)'s run start and window index.  Returns the
// live groups, or -1 if the wait timed out.
template <int NTH>
__device__ __forceinline__ int ec_stage(const V12Dev &d, int slot, long h0, long total, float2 *seg,
                                        EcShared<NTH> &sh, const float2 *xsrc, const float2 *wl, const float2 *we,
                                        int2 *srcmw) {
  const int L = d.L, lg = d.xs_perm, G = 1 << lg, units = NTH >> lg;
  const unsigned R = (unsigned)(d.n / d.W);
  const int live = (int)min((long)units, (total - h0) >> lg);
  // One thread per (group, loop): its loads and index arithmetic first, so
  // that they overlap the barrier's initialisation.
  const bool tab = threadIdx.x < live * L;
  int j = 0, u = 0, src = 0, mw = 0, rot = 0;
  unsigned ai = 0;
  float2 g = make_float2(0.f, 0.f);
  if (tab) {
    u = threadIdx.x / L;
    j = threadIdx.x - u * L;
    const long h = h0 + ((long)u << lg);
    const int ridx = (int)(h / R);
    const int res = d.comb_list[(long)slot * d.W + ridx];
    const int grp = (int)((h - (long)ridx * R) >> lg);
    if (j == 0) {
      sh.res[u] = res;
      sh.grp[u] = grp;
    }
    const int *rp = d.rparams + (long)slot * d.rp_stride;
    const Slot s = loop_slot(d, j);
    const unsigned mask = (unsigned)d.n - 1u;
    ai = (unsigned)rp[L + j];
    const unsigned p0 = ((unsigned)res * ai) & mask;
    unsigned c0 = p0 >> s.lq;
    int dist = (int)(p0 & (unsigned)(s.q - 1));
    if (dist > (s.q >> 1)) {
      c0++;
      dist -= s.q;
    }
    mw = dist + ((s.q - 1) >> 1);
    const unsigned beta = (c0 + (unsigned)(d.W / s.q) * (unsigned)grp * ai) & ((unsigned)s.B - 1u);
    const int lt = dlog2((unsigned)s.B) - lg;
    src = (int)s.off + (int)((beta & ((1u << lt) - 1u)) << lg);
    rot = (int)(beta >> lt);
    g = __ldg((j < d.L_loc ? wl : we) + mw);
  }
  // the barrier completes once the byte count is announced, every (group,
  // loop) thread has written its table entry and issued its copy (release),
  // and all copied bytes have landed
  if (threadIdx.x == 0) {
    mbar_init(&sh.bar, 1 + live * L);
    mbar_expect(&sh.bar, (unsigned)(live * L * G * sizeof(float2)));
  }
  __syncthreads();
  if (tab) {
    // the copy is issued before the window value is used, so the two loads
    // overlap (the buffer's previous contents were read through the generic
    // proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    bulk_load(seg + j * NTH + (u << lg), xsrc + (long)slot * d.xs_size + src, (unsigned)(G * sizeof(float2)),
              &sh.bar);
    sh.v[u * L + j] = EcVal{rot, ai, g.x, g.y};
    if (srcmw) srcmw[u * L + j] = make_int2(src, mw);
    mbar_arrive(&sh.bar);
  }
  // every thread waits (bounded) on its own
  if (!mbar_wait_bounded(&sh.bar, 0)) {
    atomicOr(&d.counters[slot * CNT_STRIDE + CNT_ERR], ERR_WAIT_TIMEOUT);
    mbar_wait_bounded(&sh.bar, 0);  // copies still in flight land before the block moves on
    return -1;
  }
  return live;
}

// The L FP32 values of candidate i of staged group u (see ec_stage):
// x_samp[bucket] / filter.freq[dist] with the reference's sign.
template <int LN, bool EXACT, int NTH>
__device__ __forceinline__ void ec32_values(const V12Dev &d, const float2 *seg, const EcShared<NTH> &sh, int u,
                                            int i, float (&re)[LN], float (&im)[LN]) {
  const int L = d.L, lg = d.xs_perm, G = 1 << lg;
  const int Lr = EXACT ? LN : L;
  const EcVal *tv = sh.v + u * L;
  const float2 *sg = seg + (u << lg);
#pragma unroll
  for (int j = 0; j < LN; j++) {
    if (EXACT || j < Lr) {
      const EcVal t = tv[j];
      const float2 x = sg[j * NTH + (int)(((unsigned)t.rot + (unsigned)i * t.ai) & (unsigned)(G - 1))];
      re[j] = x.x * t.gx + x.y * t.gy;
      im[j] = x.x * t.gy - x.y * t.gx;
    } else {
      re[j] = INFINITY;
      im[j] = INFINITY;
    }
  }
}

// Lower medians of the values and the output entry of candidate i of
// group (res, grp), position h0 + threadIdx.x of the slot's output.
template <int LN, bool EXACT>
__device__ __forceinline__ void ec32_finish(const V12Dev &d, int slot, long h0, int res, int grp, int i,
                                            float (&re)[LN], float (&im)[LN]) {
  const int Lr = EXACT ? LN : d.L;
  const float mre = lower_median<LN, EXACT>(re, Lr), mim = lower_median<LN, EXACT>(im, Lr);
  const unsigned S = (unsigned)(d.n / d.W) >> d.xs_perm;
  const long o = (long)slot * d.out_stride + h0 + threadIdx.x;
  d.out_idx[o] = (int)(((unsigned)grp + S * (unsigned)i) * (unsigned)d.W + (unsigned)res);
  ((float2 *)d.out_val)[o] = make_float2(mre, mim);
}

// FP32 estimates of a staged item's live groups (see ec_stage).
template <int LN, bool EXACT, int NTH>
__device__ __forceinline__ void ec32_compute(const V12Dev &d, int slot, long h0, int live, const float2 *seg,
                                             const EcShared<NTH> &sh) {
  const int lg = d.xs_perm, G = 1 << lg;
  const int u = threadIdx.x >> lg, i = threadIdx.x & (G - 1);
  if (u >= live) return;  // also after a timeout (live < 0)
  float re[LN], im[LN];
  ec32_values<LN, EXACT, NTH>(d, seg, sh, u, i, re, im);
  ec32_finish<LN, EXACT>(d, slot, h0, sh.res[u], sh.grp[u], i, re, im);
}

// One item staged, waited for and estimated in FP32.
template <int LN, bool EXACT, int NTH>
__device__ __forceinline__ void ec32_block(const V12Dev &d, int slot, long h0, long total, float2 *seg,
                                           EcShared<NTH> &sh) {
  const int live = ec_stage<NTH>(d, slot, h0, total, seg, sh, (const float2 *)d.xs, (const float2 *)d.win_loc,
                                 (const float2 *)d.win_est, nullptr);
  ec32_compute<LN, EXACT, NTH>(d, slot, h0, live, seg, sh);
}

// Exact FP64 value of loop j of a staged candidate: the reference's
// operation sequence on the FP64 bucket value and window.
__device__ __forceinline__ double2 ec_exact64(const V12Dev &d, const EcVal &t, int2 sm, const double2 *xs, int i,
                                             int G, int j) {
  const int idx = (int)(((unsigned)t.rot + (unsigned)i * t.ai) & (unsigned)(G - 1));
  const double2 x = xs[sm.x + idx];
  const double2 *wp = (const double2 *)(j < d.L_loc ? d.win_loc : d.win_est) + 2 * sm.y;
  const double2 hw = __ldg(wp);
  const double den = __ldg(wp + 1).x;
  using A = Ar<double>;
  return make_double2(A::div(A::add(A::mul(x.x, hw.x), A::mul(x.y, hw.y)), den),
                      A::div(A::sub(A::mul(x.x, hw.y), A::mul(x.y, hw.x)), den));
}

__device__ __noinline__ double2 ec_median64_all(const V12Dev &d, const EcVal *tv, const int2 *sm, const double2 *xs,
                                                int i, int G) {
  double vre[EC_MAXL], vim[EC_MAXL];
  const int L = d.L;
  for (int j = 0; j < L; j++) {
    const double2 v = ec_exact64(d, tv[j], sm[j], xs, i, G, j);
    vre[j] = v.x;
    vim[j] = v.y;
  }
  const int m = (L - 1) >> 1;
  double mre = 0, mim = 0;
  for (int a = 0; a < L; a++) {
    const long long ka = okey(vre[a]), kb = okey(vim[a]);
    int rr = 0, ri = 0;
    for (int b = 0; b < L; b++) {
      const long long x = okey(vre[b]), y = okey(vim[b]);
      rr += (x < ka) || (b < a && x == ka);
      ri += (y < kb) || (b < a && y == kb);
    }
    if (rr == m) mre = vre[a];
    if (ri == m) mim = vim[a];
  }
  return make_double2(mre, mim);
}

// FP64 estimates of the staged candidates, bit-exact: the lower-median
// element of each component is chosen on the staged FP32 copy and proven
// with the bound of k_estimate64 (proven_median), then divided exactly in
// FP64; anything not provable takes the all-exact path.
template <int LN, bool EXACT, int NTH>
__device__ __forceinline__ void ec64_block(const V12Dev &d, int slot, long h0, long total, float2 *seg,
                                           EcShared<NTH> &sh, int2 *srcmw) {
  const int live = ec_stage<NTH>(d, slot, h0, total, seg, sh, (const float2 *)d.xs32,
                                 (const float2 *)d.win32_loc, (const float2 *)d.win32_est, srcmw);
  const int L = d.L, lg = d.xs_perm, G = 1 << lg;
  const int u = threadIdx.x >> lg, i = threadIdx.x & (G - 1);
  if (u >= live) return;
  const int Lr = EXACT ? LN : L;
  const EcVal *tv = sh.v + u * L;
  const int2 *sm = srcmw + u * L;
  const float2 *sg = seg + (u << lg);
  const double2 *xs = (const double2 *)d.xs + (long)slot * d.xs_size;
  // One component at a time (fewer live registers, more resident warps):
  // the real part's values and bounds, its proven median, whose exact FP64
  // value is then computed (unconditionally, at a valid index, so that its
  // loads and divisions overlap the imaginary part's selection); then the
  // imaginary part's values with the same bounds.
  float v[LN], eb[LN];
#pragma unroll
  for (int j = 0; j < LN; j++) {
    if (EXACT || j < Lr) {
      const EcVal t = tv[j];
      const float2 x = sg[j * NTH + (int)(((unsigned)t.rot + (unsigned)i * t.ai) & (unsigned)(G - 1))];
      v[j] = x.x * t.gx + x.y * t.gy;
      // the bound of k_estimate64: |exact - approx| <= 2^-22 (|a| + |b|)(|g.x| + |g.y|), with a 4x margin
      eb[j] = (fabsf(x.x) + fabsf(x.y)) * (fabsf(t.gx) + fabsf(t.gy)) * 0x1p-20f + 1e-30f;
    } else {
      v[j] = INFINITY;
      eb[j] = 0.f;
    }
  }
  const int ir = proven_median<LN, EXACT>(v, eb, Lr);
  const int jr = max(ir, 0);
  const double xre = ec_exact64(d, tv[jr], sm[jr], xs, i, G, jr).x;
#pragma unroll
  for (int j = 0; j < LN; j++) {
    if (EXACT || j < Lr) {
      const EcVal t = tv[j];
      const float2 x = sg[j * NTH + (int)(((unsigned)t.rot + (unsigned)i * t.ai) & (unsigned)(G - 1))];
      v[j] = x.x * t.gy - x.y * t.gx;
    }
  }
  const int ii = proven_median<LN, EXACT>(v, eb, Lr);
  double2 res;
  if (ir >= 0 && ii >= 0) {
    res.x = xre;
    res.y = ec_exact64(d, tv[ii], sm[ii], xs, i, G, ii).y;
  } else {
    res = ec_median64_all(d, tv, sm, xs, i, G);
    atomicAdd(&d.counters[slot * CNT_STRIDE + CNT_EXACT], 1);
  }
  const unsigned S = (unsigned)(d.n / d.W) >> lg;
  const long o = (long)slot * d.out_stride + h0 + threadIdx.x;
  d.out_idx[o] = (int)(((unsigned)sh.grp[u] + S * (unsigned)i) * (unsigned)d.W + (unsigned)sh.res[u]);
  ((double2 *)d.out_val)[o] = res;
}

__device__ __forceinline__ long ec_total(const V12Dev &d, int slot) {
  return min((long)d.counters[slot * CNT_STRIDE + CNT_COMB] * (d.n / d.W), (long)d.out_cap);
}

template <int LN, bool EXACT>
__global__ void __launch_bounds__(EC_THREADS, 4) k_estimate_comb32(V12Dev d) {
  extern __shared__ __align__(128) float2 seg[];   // [loop][EC_THREADS]
  __shared__ EcShared<EC_THREADS> sh;
  const int slot = blockIdx.y;
  if (blockIdx.x == 0 && threadIdx.x == 0) publish_count(d, slot, cand_total(d, slot));
  const long total = ec_total(d, slot), h0 = (long)blockIdx.x * EC_THREADS;
  if (h0 >= total) return;
  ec32_block<LN, EXACT, EC_THREADS>(d, slot, h0, total, seg, sh);
}

template <int LN, bool EXACT>
__global__ void __launch_bounds__(EC_THREADS, 3) k_estimate_comb64(V12Dev d) {
  extern __shared__ __align__(128) float2 seg64[];   // [loop][EC_THREADS]
  __shared__ EcShared<EC_THREADS> sh;
  __shared__ int2 srcmw[(EC_THREADS / 32) * EC_MAXL];
  const int slot = blockIdx.y;
  if (blockIdx.x == 0 && threadIdx.x == 0) publish_count(d, slot, cand_total(d, slot));
  const long total = ec_total(d, slot), h0 = (long)blockIdx.x * EC_THREADS;
  if (h0 >= total) return;
  ec64_block<LN, EXACT, EC_THREADS>(d, slot, h0, total, seg64, sh, srcmw);
}

// ---------------------------------------------------------------- scatter --

template <typename R>
__global__ void k_scatter_dense(const int *out_idx, const c2_t<R> *out_val, const int *counters,
                                int out_cap, void *const *dense) {
  const int slot = blockIdx.y;
  const long h = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = counters[slot * CNT_STRIDE + CNT_OUT];
  if (h >= cnt) return;
  const long o = (long)slot * out_cap + h;
  const c2_t<R> v = out_val[o];
  ((double2 *)dense[slot])[out_idx[o]] = make_double2((double)v.x, (double)v.y);
}

// ---------------------------------------------------------------- launch --

int v12_max_fft(int prec) { return prec == PREC_FP64 ? 8192 : 16384; }
int v12_max_fft_any() { return 1 << 20; }

static void fft_shape(int N, int &T, int &per) {
  T = N / 4;
  if (T > 1024) T = 1024;
  if (T < 32) T = 32;
  per = (N / 4 + T - 1) / T;
}

template <typename R, typename In>
static cudaError_t launch_comb(const V12Dev &d, int nslots, cudaStream_t s) {
  int T, per;
  fft_shape(d.W, T, per);
  const size_t sm = BucketSmem<R>::bytes(d.W, d.num);
  dim3 grid(d.comb_loops, nslots);
  cudaError_t e;
#define SFFT_COMB(P)                                             \
  case P:                                                        \
    if ((e = set_smem(k_comb<R, P, In>, sm))) return e;          \
    k_comb<R, P, In><<<grid, T, sm, s>>>(d);                     \
    break;
  switch (per) {
    SFFT_COMB(1)
    SFFT_COMB(2)
    SFFT_COMB(4)
    default:
      return cudaErrorInvalidValue;
  }
#undef SFFT_COMB
  note_launches(1);
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_bucket(const V12Dev &d, int nslots, cudaStream_t s) {
  const int Bmax = d.B_loc > d.B_est ? d.B_loc : d.B_est;
  // FP64: two butterflies per thread and stage -- half-size CTAs, two per SM,
  // so one CTA's stage barriers overlap the other's FP64 arithmetic
  // (measured 0.52 -> 0.455 ms per 32 signals at n = 2^22, k = 100; the FP32
  // form is faster with one butterfly per thread)
  int T = sizeof(R) == 8 ? Bmax / 8 : Bmax / 4, per;
  if (T > 1024) T = 1024;
  if (T < 32) T = 32;
  per = (Bmax / 4 + T - 1) / T;
  const size_t sm = BucketSmem<R>::bytes(Bmax, d.num);
  dim3 grid(d.L, nslots);
  cudaError_t e;
#define SFFT_BUCKET(P)                                        \
  case P:                                                     \
    if ((e = set_smem(k_bucket<R, P>, sm))) return e;         \
    k_bucket<R, P><<<grid, T, sm, s>>>(d);                    \
    break;
  switch (per) {
    SFFT_BUCKET(1)
    SFFT_BUCKET(2)
    SFFT_BUCKET(4)
    default:
      return cudaErrorInvalidValue;
  }
#undef SFFT_BUCKET
  return cudaGetLastError();
}

#define SFFT_EST_KERNEL(NAME, BLOCKS)                                           \
  template <int LN, bool EX>                                                    \
  struct NAME##_k {                                                             \
    static cudaError_t go(int nslots, cudaStream_t s, const V12Dev &d, int nsm) { \
      NAME<LN, EX><<<nsm * BLOCKS(LN), 128, 0, s>>>(d, nslots);                 \
      return cudaSuccess;                                                       \
    }                                                                           \
  };
SFFT_EST_KERNEL(k_estimate32, est32_blocks)
SFFT_EST_KERNEL(k_estimate64, est64_blocks)
#undef SFFT_EST_KERNEL

template <template <int, bool> class KS>
static cudaError_t dispatch_estimate(const V12Dev &d, int nslots, int nsm, cudaStream_t s) {
  cudaError_t e;
  switch (d.L) {
#define SFFT_L(v)                                             \
  case v:                                                     \
    if ((e = KS<v, true>::go(nslots, s, d, nsm))) return e; \
    break;
    SFFT_L(8) SFFT_L(9) SFFT_L(10) SFFT_L(11) SFFT_L(12) SFFT_L(13) SFFT_L(14) SFFT_L(15) SFFT_L(16)
    SFFT_L(17) SFFT_L(18) SFFT_L(19) SFFT_L(20) SFFT_L(21) SFFT_L(22) SFFT_L(23) SFFT_L(24)
#undef SFFT_L
    default:
      if (d.L > 32) return cudaErrorInvalidValue;
      if ((e = KS<32, false>::go(nslots, s, d, nsm))) return e;
  }
  return cudaGetLastError();
}

// Multiprocessor count of the current device (cached per device).
static int sm_count() {
  static int cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cache[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
    cache[dev] = v;
  }
  return cache[dev];
}

// Estimation by comb residue (xs_perm set, FP32): one CTA per EC_THREADS
// candidates, up to min(W, comb_loops * 2k) residues of n / W candidates.
template <int LN, bool EX>
struct EcK32 {
  static cudaError_t go(int nslots, cudaStream_t s, const V12Dev &d, int) {
    const long cmax = std::min<long>(d.W, (long)d.comb_loops * d.num);
    const long cands = std::min<long>(cmax * (d.n / d.W), (long)d.out_cap);
    const size_t sm = sizeof(float2) * EC_THREADS * d.L;
    cudaError_t e;
    if ((e = set_smem(k_estimate_comb32<LN, EX>, sm))) return e;
    dim3 g((unsigned)((cands + EC_THREADS - 1) / EC_THREADS), nslots);
    k_estimate_comb32<LN, EX><<<g, EC_THREADS, sm, s>>>(d);
    return cudaSuccess;
  }
};

template <int LN, bool EX>
struct EcK64 {
  static cudaError_t go(int nslots, cudaStream_t s, const V12Dev &d, int) {
    const long cmax = std::min<long>(d.W, (long)d.comb_loops * d.num);
    const long cands = std::min<long>(cmax * (d.n / d.W), (long)d.out_cap);
    const size_t sm = sizeof(float2) * EC_THREADS * d.L;
    cudaError_t e;
    if ((e = set_smem(k_estimate_comb64<LN, EX>, sm))) return e;
    dim3 g((unsigned)((cands + EC_THREADS - 1) / EC_THREADS), nslots);
    k_estimate_comb64<LN, EX><<<g, EC_THREADS, sm, s>>>(d);
    return cudaSuccess;
  }
};

template <typename R>
static cudaError_t launch_estimate(const V12Dev &d, int nslots, cudaStream_t s) {
  if (sizeof(R) == 4 && d.xs_perm) return dispatch_estimate<EcK32>(d, nslots, 0, s);
  if (sizeof(R) == 8 && d.xs_perm) return dispatch_estimate<EcK64>(d, nslots, 0, s);
  if (sizeof(R) == 8) return dispatch_estimate<k_estimate64_k>(d, nslots, sm_count(), s);
  return dispatch_estimate<k_estimate32_k>(d, nslots, sm_count(), s);
}

template <typename R, typename In>
static cudaError_t run_typed(const V12Dev &d, int nslots, cudaStream_t s, StageEvents *se) {
  cudaError_t e;
  using V = c2_t<R>;
  if ((e = cudaMemsetAsync(d.counters, 0, sizeof(int) * CNT_STRIDE * nslots, s))) return e;
  mark(se, s);
  if (d.version == 1) {
    if ((e = cudaMemsetAsync(d.comb_bits, 0, sizeof(unsigned) * ((d.W + 31) >> 5) * nslots, s))) return e;
    if (!d.large_comb) {
      if ((e = launch_comb<R, In>(d, nslots, s))) return e;
    } else {
      dim3 g((d.W + 255) / 256, d.comb_loops, nslots);
      k_comb_gather<R, In><<<g, 256, 0, s>>>(d);
      if ((e = cudaGetLastError())) return e;
      if ((e = global_fft<R>((V *)d.comb_buf, (V *)d.comb_tmp, d.W, d.comb_loops, d.W, (long)d.comb_loops * d.W,
                             nslots, (const V *)d.tw_comb, s)))
        return e;
      k_comb_select<R><<<dim3(d.comb_loops, nslots), 1024, sizeof(int) * d.num, s>>>(d);
      if ((e = cudaGetLastError())) return e;
      note_launches(2);
    }
    k_comb_list<<<nslots, 1024, 0, s>>>(d);
    if ((e = cudaGetLastError())) return e;
    note_launches(1);
  }
  mark(se, s);
  if (sizeof(R) == 4) {
    constexpr int S = 4;
    dim3 fg((unsigned)((d.xs_size * S + 255) / 256), nslots);
    k_fold_split<In, S><<<fg, 256, 0, s>>>(d);
  } else {
    dim3 fg((unsigned)((d.xs_size + 255) / 256), nslots);
    k_fold<R, In><<<fg, 256, 0, s>>>(d);
  }
  if ((e = cudaGetLastError())) return e;
  mark(se, s);
  if (!d.large_buckets) {
    if ((e = launch_bucket<R>(d, nslots, s))) return e;
  } else {
    V *xs = (V *)d.xs, *tmp = (V *)d.xs_tmp;
    const long locsz = (long)d.L_loc * d.B_loc;
    if ((e = global_fft<R>(xs, tmp, d.B_loc, d.L_loc, d.B_loc, d.xs_size, nslots, (const V *)d.tw_loc, s))) return e;
    if ((e = global_fft<R>(xs + locsz, tmp + locsz, d.B_est, d.L_est, d.B_est, d.xs_size, nslots,
                           (const V *)d.tw_est, s)))
      return e;
    k_select_vote<R><<<dim3(d.L, nslots), 1024, sizeof(int) * d.num, s>>>(d);
    if ((e = cudaGetLastError())) return e;
  }
  {
    const long cmax = std::min<long>(d.W, (long)d.comb_loops * d.num);
    if (d.version == 1 && 4 * cmax < d.q_loc) {
      const long threads = (long)d.num * cmax * d.L_loc;
      k_vote_comb<<<dim3((unsigned)((threads + 255) / 256), nslots), 256, 0, s>>>(d, (int)cmax);
    } else if (d.version == 1 && d.W >= 32) {
      const int nbc = (d.num + VB_BUCKETS - 1) / VB_BUCKETS;
      const size_t sm = sizeof(unsigned) * (size_t)(d.W >> 5);
      if ((e = set_smem(k_vote_bits, sm))) return e;
      k_vote_bits<<<dim3((unsigned)(d.L_loc * nbc), nslots), 256, sm, s>>>(d);
    } else {
      const long votes = ((long)d.num * d.q_loc) * d.L_loc;
      k_vote<<<dim3((unsigned)((votes + 255) / 256), nslots), 256, 0, s>>>(d);
    }
    if ((e = cudaGetLastError())) return e;
    note_launches(1);
  }
  mark(se, s);
  if ((e = launch_estimate<R>(d, nslots, s))) return e;
  mark(se, s);
  note_launches(3);
  return cudaSuccess;
}

// ------------------------------------------------- persistent executor --
//
// sfft_exec_many over plans of different (n, k) as one kernel launch.  Each
// CTA (PT threads, one per SM) takes items from a global queue in list
// order.  An item is one block's worth of one stage of one signal -- a comb
// sampling, a chunk of the fold, the comb residue list, one loop's bucket
// FFT and selection, a chunk of the voting, a chunk of the estimation --
// and runs the same device code as the stage kernels.  Before it starts, its
// CTA waits (bounded) until the signal's counters show the stages it reads
// complete; after it ends, the CTA bumps the counter of its own stage.  The
// list is ordered so that every item's dependencies come earlier: a CTA only
// waits for items that CTAs already took, and those wait only for earlier
// items, so the queue always progresses, whatever the number of resident
// CTAs.  A wait that runs out flags the signal (ERR_WAIT_TIMEOUT) and the
// item is skipped, so the kernel always ends.

constexpr int PT = 1024;                 // threads of the executor's CTA
constexpr long PERSIST_POLLS = 1L << 24;  // polls of a dependency (with back-off)

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Waits until *p >= target.  Bounded; gives up at once when another wait of
// the run has already run out (*abort), so a fault costs one time limit.
__device__ __forceinline__ bool persist_wait(const int *p, int target, int *abort) {
  for (long i = 0; i < PERSIST_POLLS; i++) {
    if (ld_acquire(p) >= target) return true;
    if ((i & 255) == 255 && *(volatile int *)abort) return false;
    __nanosleep(64);
  }
  atomicExch(abort, 1);
  return false;
}

__device__ __forceinline__ void mbar_inval(unsigned long long *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <int LN, bool EX>
__device__ __forceinline__ void persist_est(const V12Dev &d, const PersistGroup &g, int slot, int idx, float2 *seg,
                                            EcShared<PT> &ecsh) {
  if (g.est_comb) {
    const long total = ec_total(d, slot), h0 = (long)idx * PT;
    if (h0 < total) ec32_block<LN, EX, PT>(d, slot, h0, total, seg, ecsh);
    __syncthreads();  // the item's mbarrier is no longer read
    if (threadIdx.x == 0 && h0 < total) mbar_inval(&ecsh.bar);
  } else {
    const long total = min(cand_total(d, slot), (long)d.out_cap);
    for (int c = 0; c < g.est_chunks; c++) {
      const long h = ((long)idx * g.est_chunks + c) * PT + threadIdx.x;
      if (h < total) est32_candidate<LN, EX>(d, slot, h);
    }
  }
}

__device__ __noinline__ void persist_est_any(const V12Dev &d, const PersistGroup &g, int slot, int idx, float2 *seg,
                                             EcShared<PT> &ecsh) {
  switch (d.L) {
#define SFFT_PL(v)                                       \
  case v:                                                \
    persist_est<v, true>(d, g, slot, idx, seg, ecsh);    \
    break;
    SFFT_PL(8) SFFT_PL(9) SFFT_PL(10) SFFT_PL(11) SFFT_PL(12) SFFT_PL(13) SFFT_PL(14) SFFT_PL(15) SFFT_PL(16)
    SFFT_PL(17) SFFT_PL(18) SFFT_PL(19) SFFT_PL(20) SFFT_PL(21) SFFT_PL(22) SFFT_PL(23) SFFT_PL(24)
#undef SFFT_PL
    default:
      persist_est<32, false>(d, g, slot, idx, seg, ecsh);
  }
}

template <typename In>
__global__ void __launch_bounds__(PT, 1) k_persist32(PersistProg p) {
  extern __shared__ __align__(128) unsigned char psmem[];
  __shared__ PersistGroup sg;      // the plan of the current item
  __shared__ EcShared<PT> ecsh;
  __shared__ PersistItem sitem;
  __shared__ int s_ok;
  int *head = p.state, *abort = p.state + 1, *dep = p.state + 2;
  int cached = -1;
  for (;;) {
    if (threadIdx.x == 0) {
      const int it = atomicAdd(head, 1);
      sitem = it < p.nitems ? p.items[it] : PersistItem{-1, -1, 0, 0};
    }
    __syncthreads();
    const PersistItem w = sitem;
    if (w.kind < 0) break;
    if (w.group != cached) {
      const int *src = (const int *)(p.groups + w.group);
      int *dst = (int *)&sg;
      for (int i = threadIdx.x; i < (int)(sizeof(PersistGroup) / sizeof(int)); i += PT) dst[i] = src[i];
      cached = w.group;
      __syncthreads();
    }
    const V12Dev &d = sg.d;
    int *sdep = dep + 4 * (sg.gslot0 + w.slot);
    if (threadIdx.x == 0) {
      bool ok = !*(volatile int *)abort;
      if (ok && w.kind == PK_LIST)
        ok = persist_wait(sdep + 0, d.comb_loops, abort);
      else if (ok && w.kind == PK_BUCKET)
        ok = persist_wait(sdep + 1, sg.nfold, abort);
      else if (ok && (w.kind == PK_VOTE || w.kind == PK_EST))
        ok = persist_wait(sdep + 2, d.L, abort) && persist_wait(sdep + 3, 1, abort);
      if (!ok) atomicOr(&d.counters[w.slot * CNT_STRIDE + CNT_ERR], ERR_WAIT_TIMEOUT);
      s_ok = ok;
    }
    __syncthreads();
    if (s_ok) {
      switch (w.kind) {
        case PK_COMB:
          if (sg.per_comb == 1)
            comb_block<float, 1, In>(d, w.idx, w.slot, psmem);
          else if (sg.per_comb == 2)
            comb_block<float, 2, In>(d, w.idx, w.slot, psmem);
          else
            comb_block<float, 4, In>(d, w.idx, w.slot, psmem);
          break;
        case PK_FOLD:
          for (int c = 0; c < sg.fold_chunks; c++)
            fold_split_thread<In, 4>(d, w.slot, ((long)w.idx * sg.fold_chunks + c) * PT + threadIdx.x);
          break;
        case PK_LIST:
          comb_list_block(d, w.slot);
          break;
        case PK_BUCKET:
          if (sg.per_bucket == 1)
            bucket_block<float, 1>(d, w.idx, w.slot, psmem);
          else if (sg.per_bucket == 2)
            bucket_block<float, 2>(d, w.idx, w.slot, psmem);
          else
            bucket_block<float, 4>(d, w.idx, w.slot, psmem);
          break;
        case PK_VOTE: {  // loop j, buckets [i0, i0 + VB_BUCKETS)
          const int nbc = (d.num + VB_BUCKETS - 1) / VB_BUCKETS, j = w.idx / nbc;
          vote_bits_block(d, j, (w.idx - j * nbc) * VB_BUCKETS, w.slot, (unsigned *)psmem);
          break;
        }
        default:  // PK_EST
          if (w.idx == 0 && threadIdx.x == 0) publish_count(d, w.slot, cand_total(d, w.slot));
          persist_est_any(d, sg, w.slot, w.idx, (float2 *)psmem, ecsh);
      }
    }
    __syncthreads();  // the item's writes precede its completion count
    if (threadIdx.x == 0) {
      const int k = w.kind == PK_COMB ? 0 : w.kind == PK_FOLD ? 1 : w.kind == PK_BUCKET ? 2 : w.kind == PK_LIST ? 3 : -1;
      if (k >= 0) {
        __threadfence();
        atomicAdd(sdep + k, 1);
      }
    }
  }
}

bool persist_eligible(const V12Dev &d) {
  const int mx = v12_max_fft(PREC_FP32);
  return d.version == 1 && !d.voted && d.prec == PREC_FP32 && !d.large_buckets && !d.large_comb && d.L <= 32 &&
         d.W >= 32 && d.W <= mx && d.B_loc <= mx && d.B_est <= mx && d.comb_loops <= 64;
}

static int per_of(int N) {
  const int per = (N / 4 + PT - 1) / PT;
  return per <= 1 ? 1 : per <= 2 ? 2 : 4;
}

void persist_shape(PersistGroup &g) {
  V12Dev &d = g.d;
  if (d.xs_perm && d.L > 24) d.xs_perm = 0;  // the comb-residue items hold L x PT values in shared memory
  g.per_comb = per_of(d.W);
  g.per_bucket = per_of(std::max(d.B_loc, d.B_est));
  g.fold_chunks = 8;
  g.nfold = (int)((d.xs_size * 4 + (long)PT * g.fold_chunks - 1) / ((long)PT * g.fold_chunks));
  g.vote_cmax = (int)std::min<long>(d.W, (long)d.comb_loops * d.num);
  g.vote_chunks = 1;
  g.nvote = d.L_loc * ((d.num + VB_BUCKETS - 1) / VB_BUCKETS);
  const long cands = std::min<long>((long)g.vote_cmax * (d.n / d.W), (long)d.out_cap);
  g.est_comb = d.xs_perm != 0;
  g.est_chunks = g.est_comb ? 1 : 4;
  g.nest = (int)((cands + (long)PT * g.est_chunks - 1) / ((long)PT * g.est_chunks));
}

size_t persist_smem(const PersistGroup *groups, int ngroups) {
  size_t m = 0;
  for (int i = 0; i < ngroups; i++) {
    const V12Dev &d = groups[i].d;
    m = std::max(m, BucketSmem<float>::bytes(std::max(d.W, std::max(d.B_loc, d.B_est)), d.num));
    if (groups[i].est_comb) m = std::max(m, sizeof(float2) * (size_t)PT * d.L);
  }
  return m;
}

// The queue order comes from a simulation of the executor on `workers`
// CTAs: every item gets a rough duration, becomes ready when the stages it
// reads are complete, and a free CTA takes the ready item of the
// highest-ranked signal (signals ranked by decreasing work), later stages
// first.  The items in simulated start order form the queue: an item starts
// only after its dependencies finished, so they precede it in the queue,
// and the order keeps CTAs off dependency waits as far as the durations
// are right.
void persist_items(const PersistGroup *groups, int ngroups, std::vector<PersistItem> &items, int workers) {
  struct Sig {
    int g, s;
    double work;
  };
  std::vector<Sig> sigs;
  for (int g = 0; g < ngroups; g++)
    for (int s = 0; s < groups[g].slots; s++)
      sigs.push_back({g, s, (double)groups[g].d.xs_size * groups[g].d.L + (double)groups[g].nest * PT});
  std::stable_sort(sigs.begin(), sigs.end(), [](const Sig &a, const Sig &b) { return a.work > b.work; });
  // durations (microseconds of one CTA, rough)
  auto dur = [&](const PersistGroup &G, int kind) -> double {
    const V12Dev &d = G.d;
    switch (kind) {
      case PK_COMB: return 2.0 + d.W / 2048.0;
      case PK_FOLD: {
        const double taps = (double)PT * G.fold_chunks / 4.0 * ((double)d.w_loc / d.B_loc + (double)d.w_est / d.B_est) / 2;
        return 1.0 + taps / 700.0;
      }
      case PK_LIST: return 1.0;
      case PK_BUCKET: return 2.0 + std::max(d.B_loc, d.B_est) / 2048.0;
      case PK_VOTE: return 1.0 + (double)VB_BUCKETS * ((d.q_loc + 31) / 32) / 512.0;
      default: return 1.0 + (double)PT * G.est_chunks * d.L / 4000.0;
    }
  };
  const int nsig = (int)sigs.size();
  // per signal: items per stage, remaining counts, completion times
  struct St {
    int comb_left, fold_left, bucket_left, list_left;
    double comb_done, fold_done, bucket_done, list_done;
    bool list_q, bucket_q, tail_q;
  };
  std::vector<St> st(nsig);
  struct Ready {
    double t;
    int rank, kind, idx;
  };
  // ready items: ordered by (rank, later kind first, idx) among those ready by now
  auto cmp = [](const Ready &a, const Ready &b) {
    if (a.rank != b.rank) return a.rank > b.rank;
    if (a.kind != b.kind) return a.kind < b.kind;
    return a.idx > b.idx;
  };
  std::priority_queue<Ready, std::vector<Ready>, decltype(cmp)> ready(cmp);
  auto later = [](const Ready &a, const Ready &b) { return a.t > b.t; };
  std::priority_queue<Ready, std::vector<Ready>, decltype(later)> pending(later);  // not ready yet
  for (int r = 0; r < nsig; r++) {
    const PersistGroup &G = groups[sigs[r].g];
    st[r] = {G.d.comb_loops, G.nfold, G.d.L, 1, 0, 0, 0, 0, false, false, false};
    for (int c = 0; c < G.d.comb_loops; c++) ready.push({0.0, r, PK_COMB, c});
    for (int i = 0; i < G.nfold; i++) ready.push({0.0, r, PK_FOLD, i});
  }
  std::priority_queue<double, std::vector<double>, std::greater<double>> free_at;
  for (int w = 0; w < std::max(1, workers); w++) free_at.push(0.0);
  items.clear();
  auto release = [&](int r, double t) {  // newly ready stages of signal r at time t
    St &x = st[r];
    const PersistGroup &G = groups[sigs[r].g];
    if (!x.list_q && x.comb_left == 0) {
      x.list_q = true;
      pending.push({t, r, PK_LIST, 0});
    }
    if (!x.bucket_q && x.fold_left == 0) {
      x.bucket_q = true;
      for (int j = 0; j < G.d.L; j++) pending.push({t, r, PK_BUCKET, j});
    }
    if (!x.tail_q && x.bucket_left == 0 && x.list_left == 0) {
      x.tail_q = true;
      for (int i = 0; i < G.nvote; i++) pending.push({t, r, PK_VOTE, i});
      for (int i = 0; i < G.nest; i++) pending.push({t, r, PK_EST, i});
    }
  };
  while (!ready.empty() || !pending.empty()) {
    double t = free_at.top();
    free_at.pop();
    while (!pending.empty() && pending.top().t <= t) {
      ready.push(pending.top());
      pending.pop();
    }
    if (ready.empty()) {  // idle until the next item becomes ready
      t = pending.top().t;
      while (!pending.empty() && pending.top().t <= t) {
        ready.push(pending.top());
        pending.pop();
      }
    }
    const Ready it = ready.top();
    ready.pop();
    const int g = sigs[it.rank].g, sl = sigs[it.rank].s;
    const double end = t + dur(groups[g], it.kind);
    items.push_back({it.kind, g, sl, it.idx});
    free_at.push(end);
    St &x = st[it.rank];
    // completion bookkeeping (dependents become ready when the last item of a stage ends)
    if (it.kind == PK_COMB) {
      x.comb_done = std::max(x.comb_done, end);
      if (--x.comb_left == 0) release(it.rank, x.comb_done);
    } else if (it.kind == PK_FOLD) {
      x.fold_done = std::max(x.fold_done, end);
      if (--x.fold_left == 0) release(it.rank, x.fold_done);
    } else if (it.kind == PK_BUCKET) {
      x.bucket_done = std::max(x.bucket_done, end);
      if (--x.bucket_left == 0) release(it.rank, std::max(x.bucket_done, x.list_done));
    } else if (it.kind == PK_LIST) {
      x.list_done = end;
      if (--x.list_left == 0) release(it.rank, std::max(x.bucket_done, x.list_done));
    }
  }
}

cudaError_t persist_run(const PersistProg &p, cudaStream_t s) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(p.state, 0, sizeof(int) * (2 + 4 * (size_t)p.nslots_total), s))) return e;
  const int grid = sm_count();
  // always opted in: with the kernel's static shared memory, 32-48 KB of
  // dynamic shared memory would exceed the default limit
  const size_t sm = std::max<size_t>(p.smem, 40 * 1024);
  if (p.in_type == IN_C128) {
    if ((e = set_smem(k_persist32<double2>, sm))) return e;
    k_persist32<double2><<<grid, PT, sm, s>>>(p);
  } else {
    if ((e = set_smem(k_persist32<float2>, sm))) return e;
    k_persist32<float2><<<grid, PT, sm, s>>>(p);
  }
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t global_fft_c128(void *a, void *b, int N, int narr, long arr_stride, long slot_stride, int nslots,
                            const void *tw, cudaStream_t s) {
  return global_fft<double>((double2 *)a, (double2 *)b, N, narr, arr_stride, slot_stride, nslots, (const double2 *)tw,
                            s);
}

cudaError_t v12_run(const V12Dev &d, int nslots, cudaStream_t s, StageEvents *se) {
  if (d.prec == PREC_FP64)
    return d.in_type == IN_C128 ? run_typed<double, double2>(d, nslots, s, se)
                                : run_typed<double, float2>(d, nslots, s, se);
  return d.in_type == IN_C128 ? run_typed<float, double2>(d, nslots, s, se)
                              : run_typed<float, float2>(d, nslots, s, se);
}

__global__ void k_copy_ints(const int *src, int *dst, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dst[i] = src[i];
}

cudaError_t copy_ints(const int *src, int *dst, int count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_copy_ints<<<(count + 255) / 256, 256, 0, s>>>(src, dst, count);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t scatter_dense(const int *out_idx, const void *out_val, int prec, const int *counters,
                          int out_cap, void *const *dense, int nslots, cudaStream_t s) {
  dim3 grid((out_cap + 255) / 256, nslots);
  if (prec == PREC_FP64)
    k_scatter_dense<double><<<grid, 256, 0, s>>>(out_idx, (const double2 *)out_val, counters, out_cap, dense);
  else
    k_scatter_dense<float><<<grid, 256, 0, s>>>(out_idx, (const float2 *)out_val, counters, out_cap, dense);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace sfft

namespace {

template <int N>
int copy_median_network(int *dst, long cap) {
  constexpr const sfft::SelNet<N, (N - 1) / 2> &net = sfft::SelOf<N, (N - 1) / 2>::net;
  if (!dst || cap < 3L * net.C) return -1;
  for (int c = 0; c < net.C; c++) {
    dst[3 * c] = net.a[c];
    dst[3 * c + 1] = net.b[c];
    dst[3 * c + 2] = net.kind[c];
  }
  return net.C;
}

}  // namespace

extern "C" int sfft_debug_median_network(int n, int *dst, long cap) {
  switch (n) {
#define SFFT_MN(v) \
  case v:          \
    return copy_median_network<v>(dst, cap);
    SFFT_MN(8) SFFT_MN(9) SFFT_MN(10) SFFT_MN(11) SFFT_MN(12) SFFT_MN(13) SFFT_MN(14) SFFT_MN(15) SFFT_MN(16)
    SFFT_MN(17) SFFT_MN(18) SFFT_MN(19) SFFT_MN(20) SFFT_MN(21) SFFT_MN(22) SFFT_MN(23) SFFT_MN(24)
#undef SFFT_MN
    default:
      return -1;
  }
}
