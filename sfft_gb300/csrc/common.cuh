// common.cuh — device building blocks shared by the sFFT kernels.
//
// Arithmetic contract.  The FP64 ("parity") instantiations perform the
// same IEEE-754 double operations, in the same order, as the CPU
// definition of the sFFT pipeline: every product that feeds a sum is a
// separately rounded __dmul_rn, so nothing is contracted into an FMA.  The
// FP32 instantiations use ordinary float arithmetic (FMA allowed).
//
// FFT.  block_fft() is the radix-4/2 Stockham FFT defined for this project
// (twiddle table tw[t] = (cos, -sin)(2 pi t / N) by quarter-wave symmetry,
// radix-2 stage first when log2 N is odd, twiddle applied only when its
// exponent is non-zero, out[(j - j%Ns)*R + j%Ns + r*Ns]).  It runs in place
// in shared memory: each stage loads all of its butterfly inputs to
// registers, synchronises, then stores.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <utility>

namespace sfft {

// ---------------------------------------------------------------- types --

template <typename R> struct C2;
template <> struct C2<double> { using T = double2; };
template <> struct C2<float> { using T = float2; };
template <typename R> using c2_t = typename C2<R>::T;

template <typename R> struct Ar;

template <> struct Ar<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};

template <> struct Ar<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
  static __device__ __forceinline__ float div(float a, float b) { return a / b; }
};

// (a + ib)(c + id) = (ac - bd) + i(ad + bc), products rounded separately.
template <typename R>
__device__ __forceinline__ c2_t<R> cmul(c2_t<R> x, c2_t<R> w) {
  using A = Ar<R>;
  c2_t<R> r;
  r.x = A::sub(A::mul(x.x, w.x), A::mul(x.y, w.y));
  r.y = A::add(A::mul(x.x, w.y), A::mul(x.y, w.x));
  return r;
}

template <typename R>
__device__ __forceinline__ c2_t<R> cadd(c2_t<R> a, c2_t<R> b) {
  c2_t<R> r;
  r.x = Ar<R>::add(a.x, b.x);
  r.y = Ar<R>::add(a.y, b.y);
  return r;
}

template <typename R>
__device__ __forceinline__ c2_t<R> csub(c2_t<R> a, c2_t<R> b) {
  c2_t<R> r;
  r.x = Ar<R>::sub(a.x, b.x);
  r.y = Ar<R>::sub(a.y, b.y);
  return r;
}

// |x|^2 = re*re + im*im, each square rounded before the sum.
template <typename R>
__device__ __forceinline__ R cabs2(c2_t<R> x) {
  return Ar<R>::add(Ar<R>::mul(x.x, x.x), Ar<R>::mul(x.y, x.y));
}

// Order-preserving unsigned key of a non-negative value (powers are >= 0).
__device__ __forceinline__ unsigned long long pkey(double v) {
  return (unsigned long long)__double_as_longlong(v);
}
__device__ __forceinline__ unsigned pkey(float v) { return __float_as_uint(v); }

template <typename R> struct Key;
template <> struct Key<double> { using T = unsigned long long; };
template <> struct Key<float> { using T = unsigned; };
template <typename R> using key_t = typename Key<R>::T;

// ------------------------------------------------------------ block scan --

// Exclusive prefix sums of two ints per thread over the block (blockDim.x
// a multiple of 32, <= 1024).  `sm` holds 2 * 32 ints.  Returns totals.
__device__ __forceinline__ int2 block_exscan2(int a, int b, int &pa, int &pb, int *sm) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int sa = a, sb = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int ta = __shfl_up_sync(0xffffffffu, sa, o);
    int tb = __shfl_up_sync(0xffffffffu, sb, o);
    if (lane >= o) { sa += ta; sb += tb; }
  }
  if (lane == 31) { sm[wid] = sa; sm[32 + wid] = sb; }
  __syncthreads();
  if (wid == 0) {
    int va = lane < nw ? sm[lane] : 0, vb = lane < nw ? sm[32 + lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int ta = __shfl_up_sync(0xffffffffu, va, o);
      int tb = __shfl_up_sync(0xffffffffu, vb, o);
      if (lane >= o) { va += ta; vb += tb; }
    }
    if (lane < nw) { sm[lane] = va; sm[32 + lane] = vb; }
  }
  __syncthreads();
  int ba = wid ? sm[wid - 1] : 0, bb = wid ? sm[32 + wid - 1] : 0;
  pa = ba + sa - a;
  pb = bb + sb - b;
  int2 tot = make_int2(sm[nw - 1], sm[32 + nw - 1]);
  __syncthreads();
  return tot;
}

// --------------------------------------------------------- shared-mem FFT --

// Forward FFT of buf[0..N) in shared memory, N = 2^logN <= PER*4*blockDim.
// tw: the N-entry twiddle table of that length (global memory).
template <typename R, int PER>
__device__ void block_fft(c2_t<R> *buf, int N, int logN, const c2_t<R> *__restrict__ tw) {
  using V = c2_t<R>;
  const int T = blockDim.x;
  int Ns = 1;
  if (logN & 1) {
    const int h = N >> 1;
    V a[2 * PER], b[2 * PER];
#pragma unroll
    for (int s = 0; s < 2 * PER; s++) {
      int j = threadIdx.x + s * T;
      if (j < h) { a[s] = buf[j]; b[s] = buf[j + h]; }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 2 * PER; s++) {
      int j = threadIdx.x + s * T;
      if (j < h) { buf[2 * j] = cadd<R>(a[s], b[s]); buf[2 * j + 1] = csub<R>(a[s], b[s]); }
    }
    __syncthreads();
    Ns = 2;
  }
  const int q4 = N >> 2;
  while (Ns < N) {
    const int stride = N / (Ns * 4);
    V v[PER][4];
#pragma unroll
    for (int s = 0; s < PER; s++) {
      int j = threadIdx.x + s * T;
      if (j < q4) {
        int k = j & (Ns - 1);
#pragma unroll
        for (int r = 0; r < 4; r++) v[s][r] = buf[j + r * q4];
#pragma unroll
        for (int r = 1; r < 4; r++) {
          int e = r * k * stride;
          if (e) v[s][r] = cmul<R>(v[s][r], tw[e]);
        }
        V t0 = cadd<R>(v[s][0], v[s][2]), t1 = csub<R>(v[s][0], v[s][2]);
        V t2 = cadd<R>(v[s][1], v[s][3]), t3 = csub<R>(v[s][1], v[s][3]);
        V u3;  // t3 * (-i)
        u3.x = t3.y;
        u3.y = -t3.x;
        v[s][0] = cadd<R>(t0, t2);
        v[s][1] = cadd<R>(t1, u3);
        v[s][2] = csub<R>(t0, t2);
        v[s][3] = csub<R>(t1, u3);
      }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < PER; s++) {
      int j = threadIdx.x + s * T;
      if (j < q4) {
        int k = j & (Ns - 1);
        int base = (j - k) * 4 + k;
#pragma unroll
        for (int r = 0; r < 4; r++) buf[base + r * Ns] = v[s][r];
      }
    }
    __syncthreads();
    Ns *= 4;
  }
}

// ---------------------------------------------------- top-num selection --

// Indices of the `num` largest of p[0..N) with the tie rule of the
// reference's find_largest_indices (src/utils.cc:130-158): the cutoff is the
// (N-num-1)-th smallest value, every index above it is taken, then indices
// equal to it in increasing order until num; the output is ascending.
// keys: order-preserving keys of p in shared memory.  hist: 256 + 2 ints of
// shared memory; scan: 64 ints.  Writes out[0..num).  Block-wide.
template <typename K, typename KeyAt>
__device__ void block_top_indices_f(KeyAt keyat, int N, int num, int *__restrict__ out, int *hist,
                                    int *scan) {
  constexpr int BITS = sizeof(K) * 8;
  const int rank = N - num - 1;  // ascending rank of the cutoff
  K prefix = 0, mask = 0;
  int remaining = rank;
  for (int shift = BITS - 8; shift >= 0; shift -= 8) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    // warp-aggregated: lanes with the same digit add once (keys of similar
    // magnitude share their top digits, which would serialise the atomics)
    for (int i0 = 0; i0 < N; i0 += blockDim.x) {
      const int i = i0 + threadIdx.x;
      int bin = -1;
      if (i < N) {
        const K k = keyat(i);
        if ((k & mask) == prefix) bin = (int)((k >> shift) & 0xFF);
      }
      const unsigned peers = __match_any_sync(0xffffffffu, bin);
      if (bin >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&hist[bin], __popc(peers));
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      // find digit d: cum(d) <= remaining < cum(d) + hist[d]
      const int lane = threadIdx.x;
      int c[8], tot = 0;
#pragma unroll
      for (int q = 0; q < 8; q++) { c[q] = hist[lane * 8 + q]; tot += c[q]; }
      int inc = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
      }
      int before = inc - tot;
      if (remaining >= before && remaining < inc) {
        int acc = before;
#pragma unroll
        for (int q = 0; q < 8; q++) {
          if (remaining >= acc && remaining < acc + c[q]) {
            hist[256] = lane * 8 + q;
            hist[257] = remaining - acc;
            hist[258] = c[q];
          }
          acc += c[q];
        }
      }
    }
    __syncthreads();
    const int d = hist[256];
    remaining = hist[257];
    const int in_bin = hist[258];
    prefix |= ((K)d) << shift;
    mask |= ((K)0xFF) << shift;
    __syncthreads();
    if (in_bin == 1 && shift > 0) {
      // the cutoff's bin holds a single key: that key is the cutoff, so its
      // remaining digits need no further histogram passes
      for (int i0 = 0; i0 < N; i0 += blockDim.x) {
        const int i = i0 + threadIdx.x;
        if (i < N) {
          const K k = keyat(i);
          if ((k & mask) == prefix) {
            hist[260] = (int)(unsigned)(k & 0xffffffffu);
            if constexpr (sizeof(K) == 8) hist[261] = (int)(unsigned)(k >> 32);
          }
        }
      }
      __syncthreads();
      K kk = (K)(unsigned)hist[260];
      if constexpr (sizeof(K) == 8) kk |= ((K)(unsigned)hist[261]) << 32;
      prefix = kk;
      __syncthreads();
      break;
    }
  }
  const K cutoff = prefix;
  // contiguous chunk per thread, in index order
  const int C = (N + blockDim.x - 1) / blockDim.x;
  const int lo = min(N, (int)threadIdx.x * C), hi = min(N, lo + C);
  int ngt = 0, neq = 0;
  for (int i = lo; i < hi; i++) {
    K k = keyat(i);
    ngt += (k > cutoff);
    neq += (k == cutoff);
  }
  int pgt, peq;
  int2 tot = block_exscan2(ngt, neq, pgt, peq, scan);
  const int need = num - tot.x;  // equal-to-cutoff entries to take
  int pos = pgt + min(peq, max(need, 0));
  int eqr = peq;
  for (int i = lo; i < hi; i++) {
    K k = keyat(i);
    if (k > cutoff) {
      if (pos < num) out[pos] = i;
      pos++;
    } else if (k == cutoff) {
      if (eqr < need) {
        if (pos < num) out[pos] = i;
        pos++;
      }
      eqr++;
    }
  }
  __syncthreads();
}

template <typename K>
__device__ void block_top_indices(const K *keys, int N, int num, int *__restrict__ out, int *hist,
                                  int *scan) {
  block_top_indices_f<K>([keys](int i) { return keys[i]; }, N, num, out, hist, scan);
}

// One radix-R stage (R = 2 with Ns = 1, or R = 4) of block_fft's Stockham
// FFT on arrays in global memory: butterfly j of array `arr`.  Same
// operations, same order, same rounding as the shared-memory stages.
template <typename R>
__device__ __forceinline__ void stockham_stage(const c2_t<R> *__restrict__ src, c2_t<R> *__restrict__ dst,
                                               int N, int Ns, int radix, int j,
                                               const c2_t<R> *__restrict__ tw) {
  using V = c2_t<R>;
  if (radix == 2) {
    const int h = N >> 1;
    const V a = src[j], b = src[j + h];
    dst[2 * j] = cadd<R>(a, b);
    dst[2 * j + 1] = csub<R>(a, b);
    return;
  }
  const int q4 = N >> 2, stride = N / (Ns * 4), k = j & (Ns - 1);
  V v[4];
#pragma unroll
  for (int r = 0; r < 4; r++) v[r] = src[j + r * q4];
#pragma unroll
  for (int r = 1; r < 4; r++) {
    const int e = r * k * stride;
    if (e) v[r] = cmul<R>(v[r], tw[e]);
  }
  const V t0 = cadd<R>(v[0], v[2]), t1 = csub<R>(v[0], v[2]);
  const V t2 = cadd<R>(v[1], v[3]), t3 = csub<R>(v[1], v[3]);
  V u3;
  u3.x = t3.y;
  u3.y = -t3.x;
  const int base = (j - k) * 4 + k;
  dst[base] = cadd<R>(t0, t2);
  dst[base + Ns] = cadd<R>(t1, u3);
  dst[base + 2 * Ns] = csub<R>(t0, t2);
  dst[base + 3 * Ns] = csub<R>(t1, u3);
}

// Raises a kernel's dynamic shared-memory limit on the current device once
// (per size it needs), so that later launches, including ones captured
// into CUDA graphs, make no attribute call.
template <typename F>
inline cudaError_t set_smem(F *kern, size_t bytes) {
  // below 48 KB no opt-in is needed, as long as the kernel's static shared
  // memory leaves room: opt in from 32 KB on
  if (bytes <= 32 * 1024) return cudaSuccess;
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e) return e;
  std::lock_guard<std::mutex> g(mu);
  const auto key = std::make_pair(dev, (const void *)kern);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done[key] = bytes;
  return e;
}

// Sets a kernel attribute on the current device once, so that later
// launches (including captured ones) make no attribute call.
template <typename F>
inline cudaError_t set_attr_once(F *kern, cudaFuncAttribute attr, int value) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, int> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e) return e;
  std::lock_guard<std::mutex> g(mu);
  const auto key = std::make_pair(dev * 64 + (int)attr, (const void *)kern);
  auto it = done.find(key);
  if (it != done.end() && it->second == value) return cudaSuccess;
  e = cudaFuncSetAttribute(kern, attr, value);
  if (e == cudaSuccess) done[key] = value;
  return e;
}

}  // namespace sfft
