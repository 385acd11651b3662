// host_plan.h — plan-time math of the sFFT engine (runs on the host once
// per plan): parameter selection, filter construction and the FFT that
// both use.  Mirrors src/sfft.cc:298-420 and :506-579, src/filters.cc,
// src/parameters.cc of sFFT 0.1.
#pragma once

#include <string>
#include <vector>

namespace sfft {

// One filter: w time-domain taps and its n-point spectrum, both as
// interleaved (re, im) doubles.  (src/filters.h:27-32)
struct HostFilter {
  int w = 0;
  std::vector<double> time;  // 2*w
  std::vector<double> freq;  // 2*n
};

struct V12Params {
  int n = 0, k = 0;
  bool comb = false;
  int B_loc = 0, B_thresh = 0, B_est = 0, W_Comb = 0, Comb_loops = 0;
  int loops_loc = 0, loops_thresh = 0, loops_est = 0;
  int w_loc = 0, w_est = 0;
  long x_samp_size = 0;
};

struct V3Params {
  int n = 0, k = 0;
  int W_Man = 0, B_g1 = 0, w_g1 = 0, B_g2 = 0, w_g2 = 0;
};

// Tunable constants of a v1/v2 plan (the quantities the reference takes
// from src/parameters.cc).  When `set`, they replace the table lookup.
struct V12Knobs {
  bool set = false;
  double Bcst_loc = 1, Bcst_est = 1, Comb_cst = 2;
  int loc_loops = 4, est_loops = 16, threshold_loops = 3, comb_loops = 1;
  double tolerance_loc = 1e-8, tolerance_est = 1e-8;
};

// How plan-time work is done.  `filters` false: only the parameters and
// the filters' tap counts (the n-point filter spectra are skipped).  `fft`:
// runs an n-point FFT of the same definition as host_fft (for instance on
// the GPU the plan is for) and returns true, or returns false to leave it to
// host_fft.
struct BuildOpts {
  bool filters = true;
  bool (*fft)(long n, double *data, int sign, void *ctx) = nullptr;
  void *ctx = nullptr;
};

// Returns 0, or -1 with `err` set when (n, k) is outside the domain on
// which the reference's algorithm is defined.
int build_v12_plan(unsigned n, unsigned k, bool comb, V12Params &p, HostFilter &loc,
                   HostFilter &est, std::string &err, const V12Knobs *knobs = nullptr,
                   const BuildOpts *opts = nullptr);
int build_v3_plan(unsigned n, unsigned k, V3Params &p, HostFilter &g1, HostFilter &g2,
                  std::string &err, const BuildOpts *opts = nullptr);

// The project's FFT (radix-4/2 Stockham + Bluestein); sign -1 forward,
// +1 backward unnormalised.  data: n interleaved (re, im) doubles.
void host_fft(long n, double *data, int sign);

// Twiddle table of the power-of-two FFT of length N: 2*N doubles.
const std::vector<double> &fft_twiddles(long N);

int floor_to_pow2(double x);

}  // namespace sfft
