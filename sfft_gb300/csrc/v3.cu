// v3.cu — the sFFT v3 ("exactly sparse") exec path on GB300.
//
//   k_v3_filters  six CTAs per signal: the two Mansour comb samplings
//                 (computefourier-3.0.cc:96-127), the two shifts of the
//                 contiguous Gaussian fold (:130-212) and of the permuted
//                 Gaussian fold (:215-297), each followed by its
//                 shared-memory FFT.  The permuted samples of the second
//                 fold take the phases of the reference's running product
//                 (:66-87), formed from tables of its factor's powers, one
//                 sample per thread.
//   k_v3_peel     one thread-block cluster (8 CTAs) per signal runs
//                 alternate_fft's estimate / peel rounds (:784-1088):
//                 bucket estimation spread over the cluster, subtraction of
//                 recovered tones with FP64 atomics, and the bucket-count
//                 fixpoint test, with a bounded number of rounds.
// The result map is a per-signal open-addressing table in global memory.
// FP64 throughout: the phase-slope frequency decode needs phase accuracy
// below pi/n.
#include <cooperative_groups.h>

#include "common.cuh"
#include "engine.h"

namespace cg = cooperative_groups;

namespace sfft {

static constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ double2 ld_x(const void *base, int in_type, long i) {
  if (in_type == IN_C128) return __ldg((const double2 *)base + i);
  const float2 v = __ldg((const float2 *)base + i);
  return make_double2((double)v.x, (double)v.y);
}

// --------------------------------------------------------------- filters --

// Split of the permuted Gaussian fold's phase products into tables:
// LO = the power of two at or above sqrt(count) entries of step^lo and
// ceil(count / LO) of shift_0 step^(LO hi), 16 bytes each, in the filter
// kernel's shared memory.
__host__ __device__ __forceinline__ int v3_phase_lo(int count) {
  int lo = 1;
  while ((long)lo * lo < count) lo *= 2;
  return lo;
}

// a^e, e >= 0, by binary powering in FP64: about 2 log2(e) rounded complex
// products, a relative error of a few 1e-15.
__device__ __forceinline__ double2 cpow64(double2 a, int e) {
  double2 r = make_double2(1.0, 0.0);
  while (e) {
    if (e & 1) r = cmul<double>(r, a);
    e >>= 1;
    if (e) a = cmul<double>(a, a);
  }
  return r;
}


template <int PER>
__global__ void __launch_bounds__(1024) k_v3_filters(V3Dev d, int role0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *buf = (double2 *)smem_raw;
  const int role = blockIdx.x + role0, slot = blockIdx.y, l = role & 1;
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const unsigned long long mask = (unsigned long long)d.n - 1;
  const void *x = d.inputs[slot];
  int N;
  const double2 *tw;
  double2 *dst;
  if (role < 2) {  // Mansour: x[(init_offset + l + i * n/W) mod n]
    N = d.W;
    tw = (const double2 *)d.tw_man;
    dst = (double2 *)d.man + (long)slot * 2 * d.W;
    const long sigma = d.n / d.W;
    const long o = rp[3] + l;
    for (int i = threadIdx.x; i < N; i += blockDim.x)
      buf[i] = ld_x(x, d.in_type, (long)((unsigned long long)(o + i * sigma) & mask));
  } else if (role < 4) {  // Gaussian 1: taps over x[init_G_offset + l + t]
    N = d.B1;
    tw = (const double2 *)d.tw_g1;
    dst = (double2 *)d.g1 + (long)slot * 2 * d.B1;
    const int chunks = d.w1 / d.B1;
    const long base = (long)rp[4] + l;
    const double2 *taps = (const double2 *)d.taps1;
    for (int b = threadIdx.x; b < N; b += blockDim.x) {
      double2 acc = make_double2(0.0, 0.0);
      for (int c = 0; c < chunks; c++) {
        const int t = c * N + b;
        const double2 xv = ld_x(x, d.in_type, (long)((unsigned long long)(base + t) & mask));
        acc = cadd<double>(acc, cmul<double>(xv, __ldg(taps + t)));
      }
      buf[b] = acc;
    }
  } else {  // Gaussian 2 on the permuted, phase-shifted samples
    N = d.B2;
    tw = (const double2 *)d.tw_g2;
    dst = (double2 *)d.g2 + (long)slot * 2 * d.B2;
    const int chunks = d.w2 / d.B2;
    const int ig = rp[4], ai = rp[1], bb = rp[2];
    const double2 *taps = (const double2 *)d.taps2;
    // permute_fourier (computefourier-3.0.cc:66-87): sample i is
    // x[(ig + i*ai) mod n] * shift_i with shift_0 = e^{2 pi i ig b / n} and
    // shift_{i+1} = shift_i * e^{2 pi i ai b / n}, a running product.  Its
    // two factors are formed here as there (the same FP64 angles, cos and
    // sin), but the product is not replayed serially: on GB300's FP64 pipe a
    // one-thread chain of rounded complex multiplications costs about 64
    // cycles per operation (2945 steps at n = 2^24, k = 1000: 0.58 ms).
    // Every thread instead forms shift_i = (shift_0 step^(LO hi)) step^lo
    // from two tables built by binary powering, one sample per thread.  Its
    // relative error, a few 1e-15, is below the serial chain's own
    // accumulated rounding (about i * 2^-53) and far inside the 1e-10 value
    // tolerance against the reference.
    double2 *P = (double2 *)d.perm + (long)slot * (d.w2 + 2) * 2 + (long)l * (d.w2 + 2);
    const int count = chunks * N + 1;
    const int LO = v3_phase_lo(count), HI = (count + LO - 1) / LO;
    double2 *tab = (double2 *)smem_raw;  // [LO] step^lo, then [HI] shift_0 step^(LO hi)
    {
      const double a0 = 2 * kPi * ig * bb / d.n, a1 = 2 * kPi * ai * bb / d.n;
      const double2 sh0 = make_double2(cos(a0), sin(a0)), st = make_double2(cos(a1), sin(a1));
      for (int e = threadIdx.x; e < LO + HI; e += blockDim.x)
        tab[e] = e < LO ? cpow64(st, e) : cmul<double>(sh0, cpow64(cpow64(st, LO), e - LO));
    }
    __syncthreads();
    for (int i = l + threadIdx.x; i < count; i += blockDim.x) {
      const double2 shift = cmul<double>(tab[LO + i / LO], tab[i % LO]);
      const long index = (long)(((unsigned long long)ig + (unsigned long long)i * (unsigned)ai) % (unsigned)d.n);
      P[i - l] = cmul<double>(ld_x(x, d.in_type, index), shift);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < N; b += blockDim.x) {
      double2 acc = make_double2(0.0, 0.0);
      for (int c = 0; c < chunks; c++) {
        const int t = c * N + b;
        acc = cadd<double>(acc, cmul<double>(P[t], __ldg(taps + t)));
      }
      buf[b] = acc;
    }
  }
  __syncthreads();
  block_fft<double, PER>(buf, N, 31 - __clz(N), tw);
  for (int i = threadIdx.x; i < N; i += blockDim.x) dst[2 * i + l] = buf[i];
}

// Mansour comb of width W above the shared-memory FFT: the two samplings go
// to contiguous arrays (man_tmp[slot][l][i]), are transformed by the
// global-memory FFT, and are interleaved into man[slot][2 i + l].
__global__ void k_v3_man_gather(V3Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, l = blockIdx.y, slot = blockIdx.z;
  if (i >= d.W) return;
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const unsigned long long mask = (unsigned long long)d.n - 1;
  const long sigma = d.n / d.W, o = rp[3] + l;
  double2 *a = (double2 *)d.man_tmp + (long)slot * 4 * d.W + (long)l * d.W;
  a[i] = ld_x(d.inputs[slot], d.in_type, (long)((unsigned long long)(o + i * sigma) & mask));
}

__global__ void k_v3_man_interleave(V3Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, l = blockIdx.y, slot = blockIdx.z;
  if (i >= d.W) return;
  const double2 *a = (const double2 *)d.man_tmp + (long)slot * 4 * d.W + (long)l * d.W;
  ((double2 *)d.man + (long)slot * 2 * d.W)[2 * i + l] = a[i];
}

int v3_max_smem_fft() { return 8192; }

// Mansour comb FFT of W points (4096 <= W <= 8192) as eight W/8-point FFTs:
// the one-CTA FP64 FFT of 8192 points in the filter kernel takes about 280 k
// cycles on GB300's narrow FP64 pipe, one SM's worth.  CTA r of a (signal,
// shift) transforms the samples a[8m + r] (m < M = W/8) in shared memory,
// multiplies entry m by w_W^(r m) and stores Y_r; k_v3_man_combine then
// forms X[k + M q] = sum_r Y_r[k] w_8^(r q) (a radix-2 FFT of 8 points per
// k).  The arithmetic differs from the one-CTA Stockham order only in
// rounding (the v3 results are held to 1e-10 of the reference's).
constexpr int V3_MAN_SPLIT = 8;

__global__ void __launch_bounds__(256) k_v3_man_split(V3Dev d) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = d.W / V3_MAN_SPLIT;
  double2 *buf = (double2 *)smem_raw;  // [M]
  double2 *tws = buf + M;              // [M]: w_M^e = w_W^(8 e)
  const int r = blockIdx.x, l = blockIdx.y, slot = blockIdx.z;
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  const unsigned long long mask = (unsigned long long)d.n - 1;
  const long sigma = d.n / d.W, o = rp[3] + l;
  const double2 *tw = (const double2 *)d.tw_man;
  const void *x = d.inputs[slot];
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    tws[m] = __ldg(tw + V3_MAN_SPLIT * m);
    buf[m] = ld_x(x, d.in_type, (long)((unsigned long long)(o + (long)(V3_MAN_SPLIT * m + r) * sigma) & mask));
  }
  __syncthreads();
  block_fft<double, 1>(buf, M, 31 - __clz(M), tws);
  double2 *Y = (double2 *)d.man_tmp + (long)slot * 4 * d.W + (long)l * d.W + (long)r * M;
  for (int m = threadIdx.x; m < M; m += blockDim.x) Y[m] = cmul<double>(buf[m], __ldg(tw + r * m));
}

__global__ void __launch_bounds__(128) k_v3_man_combine(V3Dev d) {
  const int M = d.W / V3_MAN_SPLIT;
  const int k = blockIdx.x * blockDim.x + threadIdx.x, l = blockIdx.y, slot = blockIdx.z;
  if (k >= M) return;
  const double2 *Y = (const double2 *)d.man_tmp + (long)slot * 4 * d.W + (long)l * d.W;
  const double2 *tw = (const double2 *)d.tw_man;
  double2 v[V3_MAN_SPLIT];
  constexpr int br[V3_MAN_SPLIT] = {0, 4, 2, 6, 1, 5, 3, 7};  // bit-reversed r
#pragma unroll
  for (int i = 0; i < V3_MAN_SPLIT; i++) v[i] = Y[(long)br[i] * M + k];
#pragma unroll
  for (int h = 1; h < V3_MAN_SPLIT; h *= 2) {
#pragma unroll
    for (int s0 = 0; s0 < V3_MAN_SPLIT; s0 += 2 * h) {
#pragma unroll
      for (int j = 0; j < h; j++) {
        // w_8^(j 8 / (2 h)) = w_W^(M j 8 / (2 h))
        const double2 t = j ? cmul<double>(v[s0 + j + h], __ldg(tw + (long)M * j * (V3_MAN_SPLIT / (2 * h))))
                            : v[s0 + j + h];
        const double2 u = v[s0 + j];
        v[s0 + j] = cadd<double>(u, t);
        v[s0 + j + h] = csub<double>(u, t);
      }
    }
  }
  double2 *man = (double2 *)d.man + (long)slot * 2 * d.W;
#pragma unroll
  for (int q = 0; q < V3_MAN_SPLIT; q++) man[2 * (k + M * q) + l] = v[q];
}

// ------------------------------------------------------------------ peel --

struct PeelCtx {
  const V3Dev *d;
  int n, n1;
  double2 *man, *g1, *g2;
  int *tkey;
  double2 *tval;
  int *list;
  int tmask;
  int *est_f;
  double2 *est_v;
  int a, ai, b, io, ig, aG, shift;
};

__device__ __forceinline__ double2 win_at(const double2 *win, int half, int n, int dist, int *err) {
  int ds = dist >= (n >> 1) ? dist - n : dist;
  if (ds < -half || ds > half) {
    atomicOr(err, ERR_V3_CAP);
    ds = ds < -half ? -half : half;
  }
  return __ldg(win + ds + half);
}

__device__ __forceinline__ int wrapmul(int x, int y) { return (int)((unsigned)x * (unsigned)y); }

// Subtract a recovered tone from the three nearest buckets of both shifts
// of a Gaussian filter (computefourier-3.0.cc:354-463).
__device__ void update_gauss(const PeelCtx &c, double2 *SAMP, const double2 *win, int half, int B,
                             int key, double2 v, int offset, int step, int l, int *err) {
  const int n = c.n, n1 = c.n1;
  const unsigned q = n / B;
  // key / q with q a power of two: the product with 1 / q is the same double
  const int h = (int)(key * (1. / q) + 0.5) % B;
  const int dist1 = (int)(((unsigned)h * q - (unsigned)key + (unsigned)n) & (unsigned)n1);
  const int dist2 = (int)(((unsigned)dist1 + (unsigned)n + q) & (unsigned)n1);
  const int dist3 = (int)(((unsigned)dist1 + 2u * (unsigned)n - q) & (unsigned)n1);
  // shift l of the two: time offset `offset` (l = 0) or `offset + step` (l = 1)
  const int ko = wrapmul(key, (int)((unsigned)offset + (l ? (unsigned)step : 0u))) % n;
  const double PI2_DIV_N = 2 * kPi / n;
  double sn, cs;
  sincos(PI2_DIV_N * ko, &sn, &cs);
  const double2 vl = cmul<double>(v, make_double2(cs, sn));
  const int dists[3] = {dist1, dist2, dist3};
  const int bks[3] = {h, (h + 1) % B, (h + B - 1) % B};
#pragma unroll
  for (int qd = 0; qd < 3; qd++) {
    const double2 f = win_at(win, half, n, dists[qd], err);
    const double2 r = cmul<double>(vl, f);
    double *p = (double *)&SAMP[2 * bks[qd] + l];
    atomicAdd(p, -r.x);
    atomicAdd(p + 1, -r.y);
  }
}

// (computefourier-3.0.cc:300-351), shift l of the two
__device__ void update_mansour(const PeelCtx &c, int key, double2 v, int l) {
  const int W = c.d->W;
  const int h = key & (W - 1);
  const double PI2_OVER_N = 2 * kPi / c.n;
  double s, co;
  sincos(PI2_OVER_N * key * (double)(c.io + l), &s, &co);
  const double rr = (double)W * (v.x * co - v.y * s);
  const double ri = (double)W * (v.x * s + v.y * co);
  double *p = (double *)&c.man[2 * h + l];
  atomicAdd(p, -rr);
  atomicAdd(p + 1, -ri);
}

// Subtraction of a recovered tone from one filter's buckets of one shift:
// part = 2 * filter + shift, filter 0 the permuted Gaussian, 1 the
// contiguous Gaussian, 2 the Mansour comb.  The six parts of a tone are
// independent (atomic subtractions), so they are separate work items:
// their FP64 chains (one sincos each) run on different sub-partitions.
__device__ void update_part(const PeelCtx &c, int key, double2 v, int part, int *err) {
  const V3Dev &d = *c.d;
  const int l = part & 1;
  if (part < 2) {
    const int k2 = (int)((((long long)key * c.ai) % c.n + c.shift) % c.n);
    update_gauss(c, c.g2, (const double2 *)d.win2, d.win2_half, d.B2, k2, v, c.aG, 1, l, err);
  } else if (part < 4) {
    update_gauss(c, c.g1, (const double2 *)d.win1, d.win1_half, d.B1, key, v, c.ig, 1, l, err);
  } else {
    update_mansour(c, key, v, l);
  }
}

// Result map: key -> accumulated value; returns nothing, keys of one round
// are distinct so the value update has a single writer.
__device__ void map_add(const PeelCtx &c, int key, double2 v, bool assign, int *count, int cap,
                        int *err) {
  unsigned h = ((unsigned)key * 2654435761u) & (unsigned)c.tmask;
  for (int probe = 0; probe <= c.tmask; probe++) {
    const int cur = atomicCAS(&c.tkey[h], -1, key);
    if (cur == -1) {
      const int idx = atomicAdd(count, 1);
      if (idx < cap)
        c.list[idx] = (int)h;
      else
        atomicOr(err, ERR_V3_CAP);
      c.tval[h] = v;
      return;
    }
    if (cur == key) {
      if (assign) {
        c.tval[h] = v;
      } else {
        double2 o = c.tval[h];
        c.tval[h] = make_double2(o.x + v.x, o.y + v.y);
      }
      return;
    }
    h = (h + 1) & (unsigned)c.tmask;
  }
  atomicOr(err, ERR_V3_CAP);
}

// The estimation loops below visit every bucket, but only buckets that pass
// the reference's zero-bucket check do FP64 work (atan2, sincos, sqrt) --
// and on GB300 a warp's FP64 instruction occupies its SM sub-partition's
// narrow FP64 pipe for tens of cycles whether one lane or 32 are active.
// So each CTA first lists its passing buckets in shared memory (the cheap
// check), then deals the list out one per lane over warps of all four
// sub-partitions: the FP64 work of a phase costs about one warp's chain
// per sub-partition instead of one per warp that holds a passing bucket.
constexpr int V3_LIST = 1024;  // list entries per CTA and pass (= threads per CTA)

// Position in the list of thread `tid` of a 1024-thread CTA: consecutive
// entries go to consecutive sub-partitions (warp mod 4), then lanes.
__device__ __forceinline__ int v3_spread(int tid) {
  return ((tid >> 7) << 7) | ((tid & 31) << 2) | ((tid >> 5) & 3);
}

// Per-CTA shared scratch of the estimation loops: the list of passing
// buckets and, per (entry, shift), the phase and one more quantity.  Each
// passing bucket is two work items in a first step -- the atan2 of one
// shift each, plus sqrt(c0) or 1 / c0 -- and one in a second step, so its
// FP64 chain is split over two sub-partitions.
struct EstScratch {
  int list[V3_LIST];
  int cnt;
  double ang[2 * V3_LIST], aux[2 * V3_LIST];
};

// Lists this CTA's buckets among [base + t0] (one per thread) that pass
// `pass`; every thread of the CTA calls it.  Returns the count.
__device__ __forceinline__ int est_list(EstScratch &x, int bk, bool pass) {
  if (threadIdx.x == 0) x.cnt = 0;
  __syncthreads();
  if (pass) x.list[atomicAdd(&x.cnt, 1)] = bk;
  __syncthreads();
  return x.cnt;
}

// estimate_freq_mansour_loops2 (computefourier-3.0.cc:642-776)
__device__ void est_mansour(const PeelCtx &c, int *nfound, int cap, int *err, int t0, int tstride, EstScratch &x) {
  const int W = c.d->W, n = c.n;
  const double PI2 = 2 * kPi, N_OVER_PI2 = n / PI2, PI2_OVER_N = PI2 / n;
  const unsigned FREQ_MASK = ((unsigned)(n - 1) & ~((unsigned)W - 1));
  const double NORM = 1. / W, NORM2 = NORM * NORM;
  for (int base = 0; base < W; base += tstride) {
    const int bk0 = base + t0;
    bool pass = false;
    if (bk0 < W) {
      const double2 s0 = c.man[2 * bk0], s1 = c.man[2 * bk0 + 1];
      const double c0 = (s0.x * s0.x + s0.y * s0.y) * NORM2;
      const double c1 = (s1.x * s1.x + s1.y * s1.y) * NORM2;
      pass = c0 + c1 > 1e-8;
    }
    const int cnt = est_list(x, bk0, pass);
    for (int w = v3_spread(threadIdx.x); w < 2 * cnt; w += V3_LIST) {
      const int bk = x.list[w >> 1], l = w & 1;
      const double2 sl = c.man[2 * bk + l];
      x.ang[w] = atan2(sl.y * NORM, sl.x * NORM);
      const double2 s0 = c.man[2 * bk];
      const double c0 = (s0.x * s0.x + s0.y * s0.y) * NORM2;
      x.aux[w] = l ? 1. / c0 : sqrt(c0);
    }
    __syncthreads();
    for (int e = v3_spread(threadIdx.x); e < cnt; e += V3_LIST) {
      const int bk = x.list[e];
      const double2 s1 = c.man[2 * bk + 1];
      const double c1 = (s1.x * s1.x + s1.y * s1.y) * NORM2;
      const double s0x = c.man[2 * bk].x, s0y = c.man[2 * bk].y;
      const double c0 = (s0x * s0x + s0y * s0y) * NORM2;
      const double d0 = x.ang[2 * e], d1 = x.ang[2 * e + 1];
      const double bb = (c1 * x.aux[2 * e + 1]) - 1;
      if ((bb * bb < n * 1e-10) && (c0 > 0.01)) {
        const int freq1 = (int)__double2ll_rn((d1 - d0) * N_OVER_PI2);
        const int freq3 = (int)((unsigned)freq1 & FREQ_MASK) | bk;
        const double ph = d0 - PI2_OVER_N * wrapmul(freq3, c.io);
        const double ab = x.aux[2 * e];
        double sn, co;
        sincos(ph, &sn, &co);
        const int i = atomicAdd(nfound, 1);
        if (i < cap) {
          c.est_f[i] = freq3;
          c.est_v[i] = make_double2(ab * co, ab * sn);
        } else {
          atomicOr(err, ERR_V3_CAP);
        }
      }
    }
    __syncthreads();  // the scratch is reused by the next pass
  }
}

// estimate_freq_gauss_loops2 (computefourier-3.0.cc:484-640)
__device__ void est_gauss(const PeelCtx &c, const double2 *SAMP, int B, const double2 *win,
                          int half, int a, int b, int *nfound, int cap, int *err, int t0, int tstride,
                          EstScratch &x) {
  const int n = c.n;
  const unsigned n1 = n - 1, B1 = B - 1;
  const double PI2 = 2 * kPi, N_OVER_PI2 = n / PI2;
  const double PI2_A_OFFSET_OVER_N = PI2 * a * c.ig / n;
  const double BUCKETS_OVER_N = (double)B / n;
  const double INV_N = 1. / n;  // n is a power of two: the product equals the quotient
  const unsigned q = n / B;
  for (int base = 0; base < B; base += tstride) {
    const int bk0 = base + t0;
    bool pass = false;
    if (bk0 < B) {
      const double2 s0 = SAMP[2 * bk0], s1 = SAMP[2 * bk0 + 1];
      const double c0 = s0.x * s0.x + s0.y * s0.y;
      const double c1 = s1.x * s1.x + s1.y * s1.y;
      pass = c0 + c1 > 1e-8;
    }
    const int cnt = est_list(x, bk0, pass);
    for (int w = v3_spread(threadIdx.x); w < 2 * cnt; w += V3_LIST) {
      const int bk = x.list[w >> 1], l = w & 1;
      const double2 sl = SAMP[2 * bk + l];
      x.ang[w] = atan2(sl.y, sl.x);
      const double2 s0 = SAMP[2 * bk];
      const double c0 = s0.x * s0.x + s0.y * s0.y;
      if (l) {
        const double c1 = sl.x * sl.x + sl.y * sl.y;
        x.aux[w] = c1 / c0 - 1;
      } else {
        x.aux[w] = sqrt(c0);
      }
    }
    __syncthreads();
    for (int e = v3_spread(threadIdx.x); e < cnt; e += V3_LIST) {
      const int bk = x.list[e];
      const double2 s0 = SAMP[2 * bk];
      const double c0 = s0.x * s0.x + s0.y * s0.y;
      const double d0 = x.ang[2 * e], d1 = x.ang[2 * e + 1];
      const double eb = x.aux[2 * e + 1];
      const double err2 = (eb * eb) * INV_N;
      if ((err2 < 1e-12) && (c0 > 0.01)) {
        const int freq = (int)((unsigned)((int)__double2ll_rn(N_OVER_PI2 * (d1 - d0)) + n) & n1);
        const unsigned hashed = (unsigned)__double2ll_rn(freq * BUCKETS_OVER_N) & B1;
        if (hashed == (unsigned)bk) {
          const double ph = d0 - PI2_A_OFFSET_OVER_N * freq;
          const double r = x.aux[2 * e];
          double sn, co;
          sincos(ph, &sn, &co);
          const double mr = r * co, mi = r * sn;
          const int dist = (int)((hashed * q - (unsigned)freq + (unsigned)n) & n1);
          const double2 f = win_at(win, half, n, dist, err);
          const double den = f.x * f.x + f.y * f.y;
          const double2 v = make_double2((mr * f.x + mi * f.y) / den, (mi * f.x - mr * f.y) / den);
          const int fo = (int)((unsigned)((int)(((long long)freq * a) % n) - b + n) & n1);
          const int i = atomicAdd(nfound, 1);
          if (i < cap) {
            c.est_f[i] = fo;
            c.est_v[i] = v;
          } else {
            atomicOr(err, ERR_V3_CAP);
          }
        }
      }
    }
    __syncthreads();  // the scratch is reused by the next pass
  }
}

__device__ __forceinline__ void trace_rec(const V3Dev &d, int slot, int *cnt, int round, int stage, int key,
                                          double2 v) {
  if (slot != 0 || !d.trace) return;
  const int i = atomicAdd(&cnt[CNT_TRACE], 1);
  if (i < d.trace_cap) {
    double *t = d.trace + 5 * (long)i;
    t[0] = round;
    t[1] = stage;
    t[2] = key;
    t[3] = v.x;
    t[4] = v.y;
  }
}

// One thread-block cluster of V3_CLUSTER CTAs per signal runs the
// estimate / peel rounds: every loop over buckets, estimates and map
// entries is spread over the cluster's threads, and each block-wide
// barrier of the round structure is a cluster barrier (release / acquire
// at cluster scope, so the global-memory bucket arrays and the map written
// before it are visible after it).  The round's counters live in the
// shared memory of the cluster's first CTA and are updated through
// distributed shared memory.  Control flow is uniform across the cluster:
// every branch is taken on values read after a barrier.
constexpr int V3_CLUSTER = 8;

struct PeelShared {
  int found, count, err, cnt[3], prev[3], stop;
};

__global__ void __cluster_dims__(V3_CLUSTER, 1, 1) __launch_bounds__(1024) k_v3_peel(V3Dev d) {
  __shared__ PeelShared sh_local;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  PeelShared *S = cl.map_shared_rank(&sh_local, 0);
  const int slot = blockIdx.x / V3_CLUSTER;
  const int *rp = d.rparams + (long)slot * d.rp_stride;
  PeelCtx c;
  c.d = &d;
  c.n = d.n;
  c.n1 = d.n - 1;
  c.man = (double2 *)d.man + (long)slot * 2 * d.W;
  c.g1 = (double2 *)d.g1 + (long)slot * 2 * d.B1;
  c.g2 = (double2 *)d.g2 + (long)slot * 2 * d.B2;
  c.tkey = d.map_keys + (long)slot * d.table_cap;
  c.tval = (double2 *)d.map_vals + (long)slot * d.table_cap;
  c.list = d.map_table + (long)slot * d.map_cap;
  c.tmask = d.table_cap - 1;
  c.est_f = d.est_f + (long)slot * d.est_cap;
  c.est_v = (double2 *)d.est_v + (long)slot * d.est_cap;
  c.a = rp[0];
  c.ai = rp[1];
  c.b = rp[2];
  c.io = rp[3];
  c.ig = rp[4];
  c.aG = wrapmul(c.a, c.ig);
  c.shift = ((wrapmul(c.ai, c.b) % d.n) + d.n) % d.n;
  int *cnt = d.counters + slot * CNT_STRIDE;
  // The cluster's threads; work item i of a loop over the cluster goes to
  // CTA i mod 8 and, within it, to consecutive sub-partitions and lanes
  // (v3_spread), so a short loop spreads its FP64 work over all 32
  // sub-partitions of the cluster's SMs.
  const int T = blockDim.x * V3_CLUSTER;
  const int gt = v3_spread(threadIdx.x) * V3_CLUSTER + rank;
  __shared__ EstScratch est_x;
  const bool lead = rank == 0 && threadIdx.x == 0;
  if (lead) {
    S->found = 0;
    S->count = 0;
    S->err = 0;
    S->stop = 0;
    for (int i = 0; i < 3; i++) S->prev[i] = 0;
  }
  cl.sync();

  // ---- Mansour estimate; first tones are assigned, their buckets cleared
  est_mansour(c, &S->found, d.est_cap, &S->err, gt, T, est_x);
  cl.sync();
  int F = min(S->found, d.est_cap);
  for (int i = gt; i < F; i += T) {
    trace_rec(d, slot, cnt, -2, 0, c.est_f[i], c.est_v[i]);
    map_add(c, c.est_f[i], c.est_v[i], true, &S->count, d.map_cap, &S->err);
    const int bk = c.est_f[i] % d.W;
    c.man[2 * bk] = make_double2(0.0, 0.0);
    c.man[2 * bk + 1] = make_double2(0.0, 0.0);
  }
  cl.sync();
  if (F == d.k) {  // the reference returns before writing its output (:859-860)
    if (lead) {
      cnt[CNT_OUT] = 0;
      if (d.out_count) d.out_count[slot] = 0;
      cnt[CNT_V3] = -1;
    }
    cl.sync();     // the first CTA's shared memory outlives every reader
    return;
  }

  // ---- first Gaussian filter: peel the known tones, estimate, peel
  int M = min(S->count, d.map_cap);
  for (int w = gt; w < 2 * M; w += T) {  // items (tone, shift)
    const int h = c.list[w >> 1];
    update_part(c, c.tkey[h], c.tval[h], 2 + (w & 1), &S->err);
  }
  if (lead) S->found = 0;
  cl.sync();
  est_gauss(c, c.g1, d.B1, (const double2 *)d.win1, d.win1_half, 1, 0, &S->found, d.est_cap, &S->err, gt, T,
            est_x);
  cl.sync();
  F = min(S->found, d.est_cap);
  for (int w = gt; w < 4 * F; w += T) {  // items (tone, part 2..5)
    const int i = w >> 2;
    if (!(w & 3)) {
      trace_rec(d, slot, cnt, -1, 1, c.est_f[i], c.est_v[i]);
      map_add(c, c.est_f[i], c.est_v[i], false, &S->count, d.map_cap, &S->err);
    }
    update_part(c, c.est_f[i], c.est_v[i], 2 + (w & 3), &S->err);
  }
  cl.sync();

  // ---- second (permuted) Gaussian filter: peel every known tone
  M = min(S->count, d.map_cap);
  for (int w = gt; w < 2 * M; w += T) {  // items (tone, shift)
    const int h = c.list[w >> 1];
    update_part(c, c.tkey[h], c.tval[h], w & 1, &S->err);
  }
  cl.sync();

  // ---- round robin: G2, then Mansour, G1, G2, ... until the counts of
  //      non-empty buckets repeat after a G2 round (:959-1076)
  int stage = 2, rounds = 0;
  for (;;) {
    if (lead) S->found = 0;
    cl.sync();
    if (stage == 0)
      est_mansour(c, &S->found, d.est_cap, &S->err, gt, T, est_x);
    else if (stage == 1)
      est_gauss(c, c.g1, d.B1, (const double2 *)d.win1, d.win1_half, 1, 0, &S->found, d.est_cap, &S->err, gt, T,
                est_x);
    else
      est_gauss(c, c.g2, d.B2, (const double2 *)d.win2, d.win2_half, c.a, c.b, &S->found, d.est_cap, &S->err,
                gt, T, est_x);
    cl.sync();
    F = min(S->found, d.est_cap);
    for (int w = gt; w < 6 * F; w += T) {  // items (tone, part)
      const int i = w / 6, part = w - 6 * i;
      if (part == 0) {
        trace_rec(d, slot, cnt, rounds, stage, c.est_f[i], c.est_v[i]);
        map_add(c, c.est_f[i], c.est_v[i], false, &S->count, d.map_cap, &S->err);
      }
      update_part(c, c.est_f[i], c.est_v[i], part, &S->err);
    }
    if (stage == 2 && rounds >= 1 && lead) S->cnt[0] = S->cnt[1] = S->cnt[2] = 0;
    cl.sync();
    if (stage == 2 && rounds >= 1) {
      int cm = 0, c1 = 0, c2 = 0;
      for (int j = gt; j < d.B1; j += T) {
        const double2 v = c.g1[j];
        c1 += (v.x * v.x + v.y * v.y > 1e-6);
      }
      for (int j = gt; j < d.B2; j += T) {
        const double2 v = c.g2[j];
        c2 += (v.x * v.x + v.y * v.y > 1e-6);
      }
      const double inv_w = 1. / d.W;  // W is a power of two: the products equal the quotients
      for (int j = gt; j < d.W; j += T) {
        const double2 v = c.man[2 * j];
        const double re = v.x * inv_w, im = v.y * inv_w;
        cm += (re * re + im * im > 1e-6);
      }
      if (cm) atomicAdd(&S->cnt[0], cm);
      if (c1) atomicAdd(&S->cnt[1], c1);
      if (c2) atomicAdd(&S->cnt[2], c2);
      cl.sync();
      if (lead) {
        S->stop = (S->cnt[0] == S->prev[0] && S->cnt[1] == S->prev[1] && S->cnt[2] == S->prev[2]);
        for (int i = 0; i < 3; i++) S->prev[i] = S->cnt[i];
      }
      cl.sync();
      if (S->stop) break;
    }
    rounds++;
    if (rounds > d.max_passes) {
      if (lead) atomicOr(&S->err, ERR_V3_NOCONVERGE);
      break;
    }
    stage = (stage + 1) % 3;
  }
  cl.sync();

  // ---- output: every key of the map with its accumulated value
  M = min(S->count, d.map_cap);
  const int outn = min(M, d.out_cap);
  for (int i = gt; i < outn; i += T) {
    const int h = c.list[i];
    d.out_idx[(long)slot * d.out_stride + i] = c.tkey[h];
    ((double2 *)d.out_val)[(long)slot * d.out_stride + i] = c.tval[h];
  }
  if (lead) {
    cnt[CNT_OUT] = outn;
    if (d.out_count) d.out_count[slot] = outn;
    cnt[CNT_V3] = rounds;
    cnt[CNT_ERR] |= S->err | (M > d.out_cap ? ERR_OUT_OVERFLOW : 0);
  }
  cl.sync();       // the first CTA's shared memory outlives every reader
}

// ---------------------------------------------------------------- launch --

cudaError_t v3_run(const V3Dev &d, int nslots, cudaStream_t s, StageEvents *se) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(d.counters, 0, sizeof(int) * CNT_STRIDE * nslots, s))) return e;
  if ((e = cudaMemsetAsync(d.map_keys, 0xFF, sizeof(int) * (size_t)d.table_cap * nslots, s))) return e;
  int Nmax = d.B1 > d.B2 ? d.B1 : d.B2;
  if (!d.large_man && d.W > Nmax) Nmax = d.W;
  int T = Nmax / 4;
  if (T > 1024) T = 1024;
  if (T < 32) T = 32;
  const int per = (Nmax / 4 + T - 1) / T;
  const int count2 = (d.w2 / d.B2) * d.B2 + 1, lo2 = v3_phase_lo(count2);
  const size_t sm = std::max((size_t)Nmax * sizeof(double2), sizeof(double2) * (size_t)(lo2 + (count2 + lo2 - 1) / lo2));
  mark(se, s);
  int role0 = 0;
  if (!d.large_man && v3_man_split(d.W)) {
    const int M = d.W / V3_MAN_SPLIT;
    const size_t msm = 2 * sizeof(double2) * (size_t)M;
    if ((e = set_smem(k_v3_man_split, msm))) return e;
    k_v3_man_split<<<dim3(V3_MAN_SPLIT, 2, nslots), 256, msm, s>>>(d);
    if ((e = cudaGetLastError())) return e;
    k_v3_man_combine<<<dim3((M + 127) / 128, 2, nslots), 128, 0, s>>>(d);
    if ((e = cudaGetLastError())) return e;
    note_launches(2);
    role0 = 2;
  } else if (d.large_man) {
    const dim3 g((d.W + 255) / 256, 2, nslots);
    k_v3_man_gather<<<g, 256, 0, s>>>(d);
    if ((e = cudaGetLastError())) return e;
    double2 *a = (double2 *)d.man_tmp;
    if ((e = global_fft_c128(a, a + 2L * d.W, d.W, 2, d.W, 4L * d.W, nslots, d.tw_man, s))) return e;
    k_v3_man_interleave<<<g, 256, 0, s>>>(d);
    if ((e = cudaGetLastError())) return e;
    note_launches(2);
    role0 = 2;
  }
  dim3 grid(6 - role0, nslots);
  switch (per) {
    case 1:
      if ((e = set_smem(k_v3_filters<1>, sm))) return e;
      k_v3_filters<1><<<grid, T, sm, s>>>(d, role0);
      break;
    case 2:
      if ((e = set_smem(k_v3_filters<2>, sm))) return e;
      k_v3_filters<2><<<grid, T, sm, s>>>(d, role0);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  if ((e = cudaGetLastError())) return e;
  mark(se, s);
  k_v3_peel<<<nslots * V3_CLUSTER, 1024, 0, s>>>(d);
  mark(se, s);
  note_launches(2);
  return cudaGetLastError();
}

}  // namespace sfft
