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
#pragma unroll 4
  for (int t = b; t < w; t += B) {
    const unsigned long long idx = ((unsigned long long)t * ai) & mask;
    const c2_t<R> xv = cvt_in<R>(__ldg(x + idx));
    acc = cadd<R>(acc, cmul<R>(xv, __ldg(taps + t)));
  }
  ((c2_t<R> *)d.xs)[(long)slot * d.xs_size + g] = acc;
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
__global__ void __launch_bounds__(1024) k_comb(V12Dev d) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int c = blockIdx.x, slot = blockIdx.y, W = d.W;
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

__global__ void __launch_bounds__(1024) k_comb_list(V12Dev d) {
  __shared__ int scan[64];
  const int slot = blockIdx.x, W = d.W;
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

// ---------------------------------------------------------------- bucket --

template <typename R, int PER>
__global__ void __launch_bounds__(1024) k_bucket(V12Dev d) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int j = blockIdx.x, slot = blockIdx.y;
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
  for (int i = threadIdx.x; i < B; i += blockDim.x) {
    const c2_t<R> v = buf[i];
    xs[i] = v;
    keys[i] = pkey(cabs2<R>(v));
  }
  __syncthreads();
  block_top_indices<key_t<R>>(keys, B, d.num, Js, hist, scan);
  int *Jg = d.J + ((long)slot * d.L + j) * d.num;
  for (int i = threadIdx.x; i < d.num; i += blockDim.x) Jg[i] = Js[i];
  if (!loc) return;

  // voting: positions p in [J*q - floor(q/2), +q) (mod n) map to
  // frequencies f = p * a (mod n)   (computefourier-1.0-2.0.cc:99-113, :147-181)
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const unsigned long long a = (unsigned)rp[j];
  const unsigned ep = (unsigned)rp[2 * d.L + d.comb_loops];
  const int q = d.q_loc, lq = dlog2(q);
  const long n = d.n;
  const unsigned long long mask = (unsigned long long)n - 1;
  unsigned *score = d.score + (long)slot * n;
  const unsigned *bits = d.comb_bits + (long)slot * ((d.W + 31) >> 5);
  int *cnt = d.counters + slot * CNT_STRIDE;
  const int total = d.num << lq;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int i = e >> lq, o = e & (q - 1);
    const long low = ((long)Js[i] * q - (q >> 1) + n) & (long)mask;
    const unsigned long long p = ((unsigned long long)(low + o)) & mask;
    const unsigned f = (unsigned)((p * a) & mask);
    if (d.version == 1) {
      const unsigned r = f & (unsigned)(d.W - 1);
      if (!((bits[r >> 5] >> (r & 31)) & 1u)) continue;
    }
    unsigned cur = score[f], nv;
    for (;;) {
      nv = ((cur >> 8) == ep) ? cur + 1u : ((ep << 8) | 1u);
      const unsigned prev = atomicCAS(&score[f], cur, nv);
      if (prev == cur) break;
      cur = prev;
    }
    if ((int)(nv & 255u) == d.thresh) {
      atomicAdd(&cnt[CNT_VOTED], 1);
      if (d.version == 0) {
        const int pos = atomicAdd(&cnt[CNT_HITS], 1);
        if (pos < d.hit_cap)
          d.hits[(long)slot * d.hit_cap + pos] = (int)f;
        else
          atomicOr(&cnt[CNT_ERR], ERR_HIT_OVERFLOW);
      }
    }
  }
}

// -------------------------------------------------------------- estimate --

__device__ __forceinline__ long long okey(double v) {
  long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

template <typename R> struct Med;
template <> struct Med<double> {
  using K = long long;
  static __device__ __forceinline__ K key(double v) { return okey(v); }
  static __device__ __forceinline__ K pad() { return LLONG_MAX; }
};
template <> struct Med<float> {
  using K = float;
  static __device__ __forceinline__ K key(float v) { return v; }
  static __device__ __forceinline__ K pad() { return FLT_MAX; }
};

// value of one (candidate, loop) pair: x_samp[bucket] / filter.freq[dist],
// with the reference's sign convention (conjugate, src/computefourier-1.0-2.0.cc:383-398)
template <typename R>
__device__ __forceinline__ void loop_value(const V12Dev &d, const c2_t<R> *xs, int j, unsigned f,
                                           unsigned long long ai, R &re, R &im) {
  const bool loc = j < d.L_loc;
  const int q = loc ? d.q_loc : d.q_est;
  const int B = loc ? d.B_loc : d.B_est;
  const long off = loc ? (long)j * d.B_loc : (long)d.L_loc * d.B_loc + (long)(j - d.L_loc) * d.B_est;
  const unsigned long long p = ((unsigned long long)f * ai) & ((unsigned long long)d.n - 1);
  const int lq = dlog2(q);
  int hashed = (int)(p >> lq);
  int dist = (int)(p & (q - 1));
  if (dist > (q >> 1)) {
    hashed = (hashed + 1) & (B - 1);
    dist -= q;
  }
  const int m = dist + ((q - 1) >> 1);
  const c2_t<R> v = xs[off + hashed];
  if constexpr (sizeof(R) == 8) {
    const double2 *wp = (const double2 *)(loc ? d.win_loc : d.win_est) + 2 * m;
    const double2 h = __ldg(wp);           // filter.freq entry (c, d)
    const double den = __ldg(wp + 1).x;    // c*c + d*d
    using A = Ar<double>;
    re = A::div(A::add(A::mul(v.x, h.x), A::mul(v.y, h.y)), den);
    im = A::div(A::sub(A::mul(v.x, h.y), A::mul(v.y, h.x)), den);
  } else {
    const float2 g = __ldg((const float2 *)(loc ? d.win_loc : d.win_est) + m);
    re = v.x * g.x + v.y * g.y;
    im = v.x * g.y - v.y * g.x;
  }
}

template <typename R, int LMAX>
__global__ void __launch_bounds__(128) k_estimate(V12Dev d) {
  using K = typename Med<R>::K;
  const int slot = blockIdx.y;
  const long h = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int *cnt = d.counters + slot * CNT_STRIDE;
  long total;
  unsigned f;
  if (d.version == 0) {
    total = min(cnt[CNT_HITS], d.hit_cap);
    if (h >= total) return;
    f = (unsigned)d.hits[(long)slot * d.hit_cap + h];
  } else {
    const int nc = cnt[CNT_COMB];
    total = (long)nc * (d.n / d.W);
    if (h >= total) return;
    const long rep = h / nc;
    f = (unsigned)(rep * d.W + d.comb_list[(long)slot * d.W + (h - rep * nc)]);
  }
  if (h == 0) {
    cnt[CNT_OUT] = (int)min(total, (long)d.out_cap);
    if (total > d.out_cap) atomicOr(&cnt[CNT_ERR], ERR_OUT_OVERFLOW);
  }
  if (h >= d.out_cap) return;
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const c2_t<R> *xs = (const c2_t<R> *)d.xs + (long)slot * d.xs_size;
  R vre[LMAX], vim[LMAX];
  K kre[LMAX], kim[LMAX];
#pragma unroll
  for (int j = 0; j < LMAX; j++) {
    if (j < d.L) {
      loop_value<R>(d, xs, j, f, (unsigned)rp[d.L + j], vre[j], vim[j]);
      kre[j] = Med<R>::key(vre[j]);
      kim[j] = Med<R>::key(vim[j]);
    } else {
      vre[j] = 0;
      vim[j] = 0;
      kre[j] = Med<R>::pad();
      kim[j] = Med<R>::pad();
    }
  }
  // lower median (nth_element at (L-1)/2), real and imaginary separately
  const int mrank = (d.L - 1) >> 1;
  R mre = 0, mim = 0;
#pragma unroll
  for (int i = 0; i < LMAX; i++) {
    int rr = 0, ri = 0;
#pragma unroll
    for (int jj = 0; jj < LMAX; jj++) {
      rr += (kre[jj] < kre[i]) || (jj < i && kre[jj] == kre[i]);
      ri += (kim[jj] < kim[i]) || (jj < i && kim[jj] == kim[i]);
    }
    if (i < d.L) {
      if (rr == mrank) mre = vre[i];
      if (ri == mrank) mim = vim[i];
    }
  }
  const long o = (long)slot * d.out_cap + h;
  d.out_idx[o] = (int)f;
  c2_t<R> res;
  res.x = mre;
  res.y = mim;
  ((c2_t<R> *)d.out_val)[o] = res;
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

template <typename F>
static cudaError_t set_smem(F *kern, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

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
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_bucket(const V12Dev &d, int nslots, cudaStream_t s) {
  const int Bmax = d.B_loc > d.B_est ? d.B_loc : d.B_est;
  int T, per;
  fft_shape(Bmax, T, per);
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

template <typename R>
static cudaError_t launch_estimate(const V12Dev &d, int nslots, cudaStream_t s) {
  const int cap = d.version == 0 ? d.hit_cap : d.out_cap;
  dim3 grid((cap + 127) / 128, nslots);
  if (d.L <= 12)
    k_estimate<R, 12><<<grid, 128, 0, s>>>(d);
  else if (d.L <= 16)
    k_estimate<R, 16><<<grid, 128, 0, s>>>(d);
  else if (d.L <= 24)
    k_estimate<R, 24><<<grid, 128, 0, s>>>(d);
  else if (d.L <= 32)
    k_estimate<R, 32><<<grid, 128, 0, s>>>(d);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

template <typename R, typename In>
static cudaError_t run_typed(const V12Dev &d, int nslots, cudaStream_t s, StageEvents *se) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(d.counters, 0, sizeof(int) * CNT_STRIDE * nslots, s))) return e;
  mark(se, s);
  if (d.version == 1) {
    if ((e = cudaMemsetAsync(d.comb_bits, 0, sizeof(unsigned) * ((d.W + 31) >> 5) * nslots, s))) return e;
    if ((e = launch_comb<R, In>(d, nslots, s))) return e;
    k_comb_list<<<nslots, 1024, 0, s>>>(d);
    if ((e = cudaGetLastError())) return e;
    note_launches(2);
  }
  mark(se, s);
  dim3 fg((unsigned)((d.xs_size + 255) / 256), nslots);
  k_fold<R, In><<<fg, 256, 0, s>>>(d);
  if ((e = cudaGetLastError())) return e;
  mark(se, s);
  if ((e = launch_bucket<R>(d, nslots, s))) return e;
  mark(se, s);
  if ((e = launch_estimate<R>(d, nslots, s))) return e;
  mark(se, s);
  note_launches(3);
  return cudaSuccess;
}

cudaError_t v12_run(const V12Dev &d, int nslots, cudaStream_t s, StageEvents *se) {
  if (d.prec == PREC_FP64)
    return d.in_type == IN_C128 ? run_typed<double, double2>(d, nslots, s, se)
                                : run_typed<double, float2>(d, nslots, s, se);
  return d.in_type == IN_C128 ? run_typed<float, double2>(d, nslots, s, se)
                              : run_typed<float, float2>(d, nslots, s, se);
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
