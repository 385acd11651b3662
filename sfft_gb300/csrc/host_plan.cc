// host_plan.cc — plan construction for the GPU engine.
//
// Parameters and filters are computed exactly as sFFT 0.1 computes them
// (src/sfft.cc:298-420, :506-579; src/filters.cc:62-160; the tables of
// src/parameters.cc), so plans agree with the reference's to the bit.  The
// FFT used here is this project's radix-4/2 Stockham FFT (Bluestein for
// other lengths); the GPU kernels evaluate the same operation sequence.
// Compiled with -ffp-contract=off: no product below may fuse into an FMA.
#include "host_plan.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>

extern "C" {
_Complex double cacosh(_Complex double);
_Complex double ccosh(_Complex double);
_Complex double cexp(_Complex double);
}

namespace sfft {

static inline _Complex double mkc(double re, double im) {
  _Complex double z;
  __real__ z = re;
  __imag__ z = im;
  return z;
}

int floor_to_pow2(double x) {  // src/utils.cc:243-248
  unsigned int ans;
  for (ans = 1; ans <= x; ans <<= 1) {
  }
  return ans / 2;
}

// ------------------------------------------------------------------ FFT --

static int exact_log2(long n) {
  int m = 0;
  while ((1L << m) < n) m++;
  return ((1L << m) == n) ? m : -1;
}

static std::vector<double> make_twiddles(long N) {
  std::vector<double> tw(2 * (size_t)std::max(N, 2L));
  if (N < 4) {
    tw[0] = 1.0;
    tw[1] = -0.0;
    tw[2] = -1.0;
    tw[3] = -0.0;
    return tw;
  }
  const long Q = N / 4;
#pragma omp parallel for schedule(static) if (Q >= (1 << 14))
  for (long u = 0; u < Q; u++) {
    const double a = (2.0 * M_PI * (double)u) / (double)N;
    const double c = std::cos(a), s = std::sin(a);
    const double C[4] = {c, -s, -c, s};
    const double S[4] = {s, c, -s, -c};
    for (int q = 0; q < 4; q++) {
      const long t = q * Q + u;
      tw[2 * t] = C[q];
      tw[2 * t + 1] = -S[q];
    }
  }
  return tw;
}

const std::vector<double> &fft_twiddles(long N) {
  static std::mutex mu;
  static std::map<long, std::unique_ptr<std::vector<double>>> cache;
  std::lock_guard<std::mutex> g(mu);
  auto &slot = cache[N];
  if (!slot) slot.reset(new std::vector<double>(make_twiddles(N)));
  return *slot;
}

static inline void cmul_inplace(double &re, double &im, const double *w) {
  const double a = re, b = im, c = w[0], d = w[1];
  const double ac = a * c, bd = b * d, ad = a * d, bc = b * c;
  re = ac - bd;
  im = ad + bc;
}

static void fft_pow2_forward(long N, double *a) {
  if (N <= 1) return;
  const double *tw = fft_twiddles(N).data();
  std::vector<double> tmpv(2 * (size_t)N);
  double *src = a, *dst = tmpv.data();
  long Ns = 1;
  if (exact_log2(N) & 1) {
    const long h = N / 2;
    for (long j = 0; j < h; j++) {
      const double v0r = src[2 * j], v0i = src[2 * j + 1];
      const double v1r = src[2 * (j + h)], v1i = src[2 * (j + h) + 1];
      dst[4 * j] = v0r + v1r;
      dst[4 * j + 1] = v0i + v1i;
      dst[4 * j + 2] = v0r - v1r;
      dst[4 * j + 3] = v0i - v1i;
    }
    std::swap(src, dst);
    Ns = 2;
  }
  const long q4 = N / 4;
  while (Ns < N) {
    const long stride = N / (Ns * 4);
    for (long j = 0; j < q4; j++) {
      const long k = j & (Ns - 1);
      double vr[4], vi[4];
      for (int r = 0; r < 4; r++) {
        vr[r] = src[2 * (j + r * q4)];
        vi[r] = src[2 * (j + r * q4) + 1];
      }
      for (int r = 1; r < 4; r++) {
        const long e = (long)r * k * stride;
        if (e) cmul_inplace(vr[r], vi[r], tw + 2 * e);
      }
      const double t0r = vr[0] + vr[2], t0i = vi[0] + vi[2];
      const double t1r = vr[0] - vr[2], t1i = vi[0] - vi[2];
      const double t2r = vr[1] + vr[3], t2i = vi[1] + vi[3];
      const double t3r = vr[1] - vr[3], t3i = vi[1] - vi[3];
      const double u3r = t3i, u3i = -t3r;  // (v1 - v3) * (-i)
      const long base = (j - k) * 4 + k;
      dst[2 * base] = t0r + t2r;
      dst[2 * base + 1] = t0i + t2i;
      dst[2 * (base + Ns)] = t1r + u3r;
      dst[2 * (base + Ns) + 1] = t1i + u3i;
      dst[2 * (base + 2 * Ns)] = t0r - t2r;
      dst[2 * (base + 2 * Ns) + 1] = t0i - t2i;
      dst[2 * (base + 3 * Ns)] = t1r - u3r;
      dst[2 * (base + 3 * Ns) + 1] = t1i - u3i;
    }
    std::swap(src, dst);
    Ns *= 4;
  }
  if (src != a) std::memcpy(a, src, sizeof(double) * 2 * (size_t)N);
}

static void conj_all(long n, double *a) {
  for (long i = 0; i < n; i++) a[2 * i + 1] = -a[2 * i + 1];
}

static void fft_pow2(long N, double *a, int sign) {
  if (sign > 0) conj_all(N, a);
  fft_pow2_forward(N, a);
  if (sign > 0) conj_all(N, a);
}

static void fft_bluestein(long w, double *x, int sign) {
  long M = 1;
  while (M < 2 * w - 1) M <<= 1;
  std::vector<double> ch(2 * (size_t)w), A(2 * (size_t)M, 0.0), Bv(2 * (size_t)M, 0.0);
  for (long m = 0; m < w; m++) {
    const long e = (long)(((uint64_t)m * (uint64_t)m) % (uint64_t)(2 * w));
    const double p = (M_PI * (double)e) / (double)w;
    ch[2 * m] = std::cos(p);
    ch[2 * m + 1] = -std::sin(p);
  }
  if (sign > 0) conj_all(w, x);
  for (long m = 0; m < w; m++) {
    double re = x[2 * m], im = x[2 * m + 1];
    cmul_inplace(re, im, &ch[2 * m]);
    A[2 * m] = re;
    A[2 * m + 1] = im;
    Bv[2 * m] = ch[2 * m];
    Bv[2 * m + 1] = -ch[2 * m + 1];
    if (m) {
      Bv[2 * (M - m)] = ch[2 * m];
      Bv[2 * (M - m) + 1] = -ch[2 * m + 1];
    }
  }
  fft_pow2(M, A.data(), -1);
  fft_pow2(M, Bv.data(), -1);
  for (long i = 0; i < M; i++) cmul_inplace(A[2 * i], A[2 * i + 1], &Bv[2 * i]);
  fft_pow2(M, A.data(), +1);
  for (long kk = 0; kk < w; kk++) {
    double re = A[2 * kk], im = A[2 * kk + 1];
    cmul_inplace(re, im, &ch[2 * kk]);
    x[2 * kk] = re / (double)M;
    x[2 * kk + 1] = im / (double)M;
  }
  if (sign > 0) conj_all(w, x);
}

void host_fft(long n, double *data, int sign) {
  if (n <= 1) return;
  if (exact_log2(n) >= 0)
    fft_pow2(n, data, sign);
  else
    fft_bluestein(n, data, sign);
}

// -------------------------------------------------------------- filters --

static double cheb(double m, double x) {  // src/filters.cc:62-68
  if (std::fabs(x) <= 1) return std::cos(m * std::acos(x));
  _Complex double z = cacosh(mkc(x, 0.0));
  _Complex double mz = mkc(m * __real__ z, m * __imag__ z);
  _Complex double c = ccosh(mz);
  return __real__ c;
}

// src/filters.cc:70-86: Dolph-Chebyshev window, time domain, w odd.
static void make_dolph_chebyshev(double lobefrac, double tolerance, HostFilter &f) {
  int w = (int)((1 / M_PI) * (1 / lobefrac) * std::acosh(1. / tolerance));
  if (!(w % 2)) w--;
  std::vector<double> x(2 * (size_t)w);
  const double t0 = std::cosh(std::acosh(1 / tolerance) / (w - 1));
  for (int i = 0; i < w; i++) {
    x[2 * i] = cheb(w - 1, t0 * std::cos(M_PI * i / w)) * tolerance;
    x[2 * i + 1] = 0.0;
  }
  host_fft(w, x.data(), -1);
  const int r = w / 2;  // circular shift by w/2, keep the real part
  f.w = w;
  f.time.assign(2 * (size_t)w, 0.0);
  for (int i = 0; i < w; i++) f.time[2 * i] = x[2 * ((i - r + w) % w)];
}

static void plan_fft(long n, double *data, int sign, const BuildOpts *opts) {
  if (opts && opts->fft && opts->fft(n, data, sign, opts->ctx)) return;
  host_fft(n, data, sign);
}

// src/filters.cc:109-160: flat-top "multiple" filter of width b over n.
// The running sums and the phase oscillator are sequential (their rounding
// is part of the result); the magnitude maximum and the scaling are
// elementwise and run in parallel.
static void make_multiple(HostFilter &f, int n, int b, const BuildOpts *opts) {
  const int w = f.w;
  std::vector<double> g(2 * (size_t)n, 0.0);
  std::memcpy(g.data(), f.time.data() + 2 * (w / 2), sizeof(double) * 2 * (size_t)(w - w / 2));
  std::memcpy(g.data() + 2 * (size_t)(n - w / 2), f.time.data(), sizeof(double) * 2 * (size_t)(w / 2));
  plan_fft(n, g.data(), -1, opts);
  double sr = 0, si = 0;
  for (int i = 0; i < b; i++) {
    sr += g[2 * i];
    si += g[2 * i + 1];
  }
  std::vector<double> &h = f.freq;
  h.assign(2 * (size_t)n, 0.0);
  const int offset = b / 2;
  for (long i = 0; i < n; i++) {
    const long d = (i + n + offset) % n;
    h[2 * d] = sr;
    h[2 * d + 1] = si;
    const long ib = (i + b) % n;
    const double dr = g[2 * ib] - g[2 * i], di = g[2 * ib + 1] - g[2 * i + 1];
    sr = sr + dr;
    si = si + di;
  }
  double mx = 0;
#pragma omp parallel for reduction(max : mx) schedule(static) if (n >= (1 << 16))
  for (long i = 0; i < n; i++) {
    const double m = std::hypot(h[2 * i], h[2 * i + 1]);
    mx = (mx < m) ? m : mx;
  }
#pragma omp parallel for schedule(static) if (n >= (1 << 16))
  for (long i = 0; i < n; i++) {
    h[2 * i] /= mx;
    h[2 * i + 1] /= mx;
  }
  const double theta = ((-2 * M_PI) * (double)(w / 2)) / (double)n;
  const _Complex double step = cexp(mkc(-0.0, theta));
  const double str = __real__ step, sti = __imag__ step;
  double ocr = 1.0, oci = 0.0;
  for (long i = 0; i < n; i++) {
    const double a = h[2 * i], bb = h[2 * i + 1];
    h[2 * i] = a * ocr - bb * oci;
    h[2 * i + 1] = a * oci + bb * ocr;
    const double nr = ocr * str - oci * sti, ni = ocr * sti + oci * str;
    ocr = nr;
    oci = ni;
  }
  std::memcpy(g.data(), h.data(), sizeof(double) * 2 * (size_t)n);
  plan_fft(n, g.data(), +1, opts);
  for (int i = 0; i < w; i++) {
    f.time[2 * i] = g[2 * i] / n;
    f.time[2 * i + 1] = g[2 * i + 1] / n;
  }
}

// ------------------------------------------------------ parameter tables --

namespace {
// src/parameters.cc:24-513 (as data): key, Bcst_loc, Bcst_est, Comb_cst,
// comb_loops, est_loops, loc_loops, threshold_loops, tol_loc, tol_est.
struct Row {
  int key;
  double bl, be, cc;
  int cl, el, ll, tl;
  double tol_l, tol_e;
};
const Row kNComb[] = {
    {8192, 2, 2, 32, 8, 16, 7, 6, 1e-8, 1e-8},      {16384, 4, 4, 32, 8, 10, 6, 5, 1e-8, 1e-8},
    {32768, 4, 2, 64, 4, 8, 5, 4, 1e-8, 1e-8},      {65536, 4, 2, 128, 6, 10, 4, 2, 1e-8, 1e-8},
    {131072, 1, 1, 8, 2, 12, 4, 3, 1e-6, 1e-8},     {262144, 1, 1, 8, 2, 14, 5, 4, 1e-6, 1e-8},
    {524288, 0.5, 0.5, 8, 1, 10, 4, 3, 1e-6, 1e-8}, {1048576, 0.5, 0.5, 8, 2, 12, 4, 2, 1e-6, 1e-8},
    {2097152, 0.5, 0.2, 8, 1, 10, 3, 2, 1e-6, 1e-8}, {4194304, 0.5, 0.2, 8, 1, 8, 3, 2, 1e-6, 1e-8},
    {8388608, 0.5, 0.2, 8, 1, 8, 3, 2, 1e-6, 1e-8}, {16777216, 0.5, 0.2, 16, 1, 8, 3, 2, 1e-6, 1e-8},
};
const Row kNPlain[] = {
    {8192, 2, 2, 1, 1, 16, 7, 6, 1e-8, 1e-8},       {16384, 4, 4, 1, 1, 10, 6, 5, 1e-8, 1e-8},
    {32768, 4, 2, 1, 1, 8, 5, 4, 1e-8, 1e-8},       {65536, 4, 2, 1, 1, 8, 5, 4, 1e-8, 1e-8},
    {131072, 2, 1, 1, 1, 10, 5, 4, 1e-6, 1e-8},     {262144, 2, 0.5, 1, 1, 14, 4, 3, 1e-6, 1e-8},
    {524288, 1, 0.5, 1, 1, 12, 5, 4, 1e-6, 1e-8},   {1048576, 2, 0.5, 1, 1, 12, 4, 3, 1e-6, 1e-8},
    {2097152, 2, 0.2, 1, 1, 15, 3, 2, 1e-6, 1e-8},  {4194304, 4, 0.2, 1, 1, 10, 3, 2, 1e-6, 1e-8},
    {8388608, 2, 0.2, 1, 1, 8, 3, 2, 1e-6, 1e-8},   {16777216, 4, 0.2, 1, 1, 8, 3, 2, 1e-6, 1e-8},
};
const Row kKComb[] = {
    {50, 0.5, 0.2, 16, 1, 10, 3, 2, 1e-6, 1.0e-8},   {100, 0.5, 0.2, 16, 1, 12, 4, 2, 1e-6, 1.0e-8},
    {200, 0.5, 0.5, 32, 1, 8, 4, 3, 1e-6, 0.5e-8},   {500, 0.5, 0.5, 64, 1, 10, 4, 3, 1e-6, 0.5e-8},
    {1000, 1, 1, 128, 3, 12, 4, 3, 1e-6, 0.5e-8},    {2000, 1, 1, 512, 3, 16, 4, 3, 1e-7, 0.2e-8},
    {2500, 1, 1, 512, 3, 16, 4, 3, 1e-7, 0.2e-8},    {4000, 1, 2, 512, 3, 14, 8, 7, 1e-8, 0.5e-8},
};
const Row kKPlain[] = {
    {50, 4, 0.2, 1, 1, 10, 3, 2, 1e-6, 1.0e-8},      {100, 2, 0.2, 1, 1, 12, 3, 2, 1e-6, 1.0e-8},
    {200, 4, 0.5, 1, 1, 10, 3, 2, 1e-6, 0.5e-8},     {500, 2, 1, 1, 1, 12, 4, 3, 1e-6, 0.5e-8},
    {1000, 2, 1, 1, 1, 12, 5, 4, 1e-6, 1.0e-8},      {2000, 2, 1, 1, 1, 16, 5, 4, 1e-7, 0.5e-8},
    {2500, 2, 1, 1, 1, 16, 5, 4, 1e-7, 0.5e-8},      {4000, 2, 2, 1, 1, 14, 6, 5, 1e-8, 1.0e-8},
};

template <size_t L>
const Row *find_row(const Row (&t)[L], int key) {
  for (size_t i = 0; i < L; i++)
    if (t[i].key == key) return &t[i];
  return nullptr;
}
}  // namespace

int build_v12_plan(unsigned n, unsigned k, bool comb, V12Params &p, HostFilter &loc,
                   HostFilter &est, std::string &err, const V12Knobs *knobs, const BuildOpts *opts) {
  double Bcst_loc = 1, Bcst_est = 1, Comb_cst = 2;
  int loc_loops = 4, est_loops = 16, threshold_loops = 3, comb_loops = 1;
  double tolerance_loc = 1.e-8, tolerance_est = 1.e-8;
  // src/sfft.cc:316-327: k > 50 consults the per-k table with n as the key
  const Row *r = (k > 50) ? (comb ? find_row(kKComb, (int)n) : find_row(kKPlain, (int)n))
                          : (comb ? find_row(kNComb, (int)n) : find_row(kNPlain, (int)n));
  if (knobs && knobs->set) {
    Bcst_loc = knobs->Bcst_loc;
    Bcst_est = knobs->Bcst_est;
    Comb_cst = knobs->Comb_cst;
    comb_loops = knobs->comb_loops;
    est_loops = knobs->est_loops;
    loc_loops = knobs->loc_loops;
    threshold_loops = knobs->threshold_loops;
    tolerance_loc = knobs->tolerance_loc;
    tolerance_est = knobs->tolerance_est;
  } else if (r) {
    Bcst_loc = r->bl;
    Bcst_est = r->be;
    Comb_cst = r->cc;
    comb_loops = r->cl;
    est_loops = r->el;
    loc_loops = r->ll;
    threshold_loops = r->tl;
    tolerance_loc = r->tol_l;
    tolerance_est = r->tol_e;
  }
  n = floor_to_pow2(n);
  p.n = (int)n;
  p.k = (int)k;
  p.comb = comb;
  const double BB_loc = (unsigned)(Bcst_loc * std::sqrt((double)(int)n * k / (std::log2(n))));
  const double BB_est = (unsigned)(Bcst_est * std::sqrt((double)(int)n * k / (std::log2(n))));
  const double lobefrac_loc = 0.5 / (BB_loc);
  const double lobefrac_est = 0.5 / (BB_est);
  const int b_loc = (int)(1.2 * 1.1 * ((double)n / BB_loc));
  const int b_est = (int)(1.4 * 1.1 * ((double)n / BB_est));
  p.B_loc = floor_to_pow2(BB_loc);
  p.B_thresh = 2 * k;
  p.B_est = floor_to_pow2(BB_est);
  p.W_Comb = floor_to_pow2(Comb_cst * n / p.B_loc);
  p.Comb_loops = comb_loops;
  p.loops_loc = loc_loops;
  p.loops_thresh = threshold_loops;
  p.loops_est = est_loops;
  if (p.B_loc < p.B_thresh + 1 || p.B_est < p.B_thresh + 1 || (comb && p.W_Comb < p.B_thresh + 1)) {
    err = "bucket count below 2k+1: (n, k) outside the algorithm's domain (find_largest_indices needs n >= num+1)";
    return -1;
  }
  if (p.W_Comb < 1 || (int)n % p.W_Comb) {
    err = "comb width does not divide n";
    return -1;
  }
  make_dolph_chebyshev(lobefrac_loc, tolerance_loc, loc);
  make_dolph_chebyshev(lobefrac_est, tolerance_est, est);
  if (loc.w > (int)n || est.w > (int)n || b_loc > (int)n || b_est > (int)n) {
    err = "filter wider than the signal";
    return -1;
  }
  if (!opts || opts->filters) {
    make_multiple(loc, (int)n, b_loc, opts);
    make_multiple(est, (int)n, b_est, opts);
  }
  p.w_loc = loc.w;
  p.w_est = est.w;
  p.x_samp_size = (long)p.loops_loc * p.B_loc + (long)p.loops_est * p.B_est;
  return 0;
}

int build_v3_plan(unsigned n, unsigned k, V3Params &p, HostFilter &g1, HostFilter &g2,
                  std::string &err, const BuildOpts *opts) {
  const double Bcst = 1, Bcst2 = 0.25, Mancst = 10;
  const double tolerance_g1 = 1.e-8, tolerance_g2 = 1.e-8;
  n = floor_to_pow2(n);
  p.n = (int)n;
  p.k = (int)k;
  p.W_Man = floor_to_pow2(Mancst * ((double)k));
  p.W_Man = (int)std::min(n / 2, (unsigned)p.W_Man);
  const double BB = (unsigned)(Bcst * ((double)k));
  p.B_g1 = floor_to_pow2(BB);
  const double lobefrac_g1 = 0.5 / (BB);
  const int b_g1 = (int)(1.00 * ((double)n / p.B_g1));
  const double BB2 = (unsigned)(Bcst2 * ((double)k));
  p.B_g2 = floor_to_pow2(BB2);
  if (p.B_g2 < 2 || p.W_Man < 2) {
    err = "v3 needs k >= 8 (second Gaussian filter would have fewer than 2 buckets)";
    return -1;
  }
  const double lobefrac_g2 = 0.5 / (BB2);
  const int b_g2 = (int)(1.00 * ((double)n / p.B_g2));
  make_dolph_chebyshev(lobefrac_g1, tolerance_g1, g1);
  make_dolph_chebyshev(lobefrac_g2, tolerance_g2, g2);
  if (g1.w > (int)n || g2.w + 2 > (int)n) {
    err = "filter wider than the signal";
    return -1;
  }
  if (!opts || opts->filters) {
    make_multiple(g1, (int)n, b_g1, opts);
    make_multiple(g2, (int)n, b_g2, opts);
  }
  p.w_g1 = g1.w;
  p.w_g2 = g2.w;
  return 0;
}

}  // namespace sfft
