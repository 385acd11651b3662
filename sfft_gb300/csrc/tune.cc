// tune.cc — constants of v1/v2 plans chosen by this project rather than
// taken from the reference's tables (src/parameters.cc of sFFT 0.1): a
// table written by the autotuner (sfft_gb300/autotune.py), keyed by n and
// the k bucket (the next power of two >= max(k, 16)), and a rule for
// shapes the table does not hold.
#include <cmath>

#include "../../include/sfft.h"

namespace sfft {

namespace {
struct TunedRow {
  int n, kb, version;
  double Bcst_loc, Bcst_est, Comb_cst;
  int loc_loops, est_loops, threshold_loops, comb_loops;
  double tolerance_loc, tolerance_est;
};

const TunedRow kTuned[] = {
#include "tuned_table.inc"
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}};  // sentinel
}  // namespace

int k_bucket(int k) {
  int b = 16;
  while (b < k) b *= 2;
  return b;
}

// Rule for shapes without a table row: bucket counts of about 8k (at least
// 2k+1 for the threshold), comb width giving about 8k bucketed candidates
// per residue class.
bool rule_params(int n, int k, sfft_params &p) {
  const double s = std::sqrt((double)n * k / std::log2((double)n));
  if (8.0 * k > n / 2) return false;
  p.Bcst_loc = p.Bcst_est = 8.0 * k / s;
  int B = 1;
  while (B * 2 <= p.Bcst_loc * s) B *= 2;
  p.Comb_cst = std::max(2.0, 8.0 * k * B / (double)n);
  p.loc_loops = 4;
  p.est_loops = 16;
  p.threshold_loops = 3;
  p.comb_loops = 1;
  p.tolerance_loc = 1e-8;
  p.tolerance_est = 1e-8;
  return true;
}

// 1: table row for (n, bucket of k, version); 0: rule; -1: neither applies.
int tuned_lookup(int n, int k, int version, sfft_params &p) {
  const int kb = k_bucket(k);
  for (const TunedRow *r = kTuned; r->n; r++) {
    if (r->n == n && r->kb == kb && r->version == version) {
      p.Bcst_loc = r->Bcst_loc;
      p.Bcst_est = r->Bcst_est;
      p.Comb_cst = r->Comb_cst;
      p.loc_loops = r->loc_loops;
      p.est_loops = r->est_loops;
      p.threshold_loops = r->threshold_loops;
      p.comb_loops = r->comb_loops;
      p.tolerance_loc = r->tolerance_loc;
      p.tolerance_est = r->tolerance_est;
      return 1;
    }
  }
  return rule_params(n, k, p) ? 0 : -1;
}

// A plan under a tuning mode: 0 the reference's constants only; 1 those,
// else tuned ones where the reference's leave (n, k) outside the domain;
// 2 tuned constants (table or rule), else the reference's.  v3 plans always
// use the reference's constants.
sfft_plan *make_plan_tuned(int n, int k, int version, const sfft_options &o, int mode, bool &tuned) {
  tuned = false;
  sfft_params prm;
  const bool v12 = version == SFFT_VERSION_1 || version == SFFT_VERSION_2;
  if (mode == 2 && v12 && tuned_lookup(n, k, version, prm) >= 0) {
    sfft_plan *p = sfft_make_plan_params(n, k, (enum sfft_version)version, &prm, &o);
    if (p) {
      tuned = true;
      return p;
    }
  }
  sfft_plan *p = sfft_make_plan_ex(n, k, (enum sfft_version)version, FFTW_ESTIMATE, &o);
  if (!p && mode == 1 && v12 && tuned_lookup(n, k, version, prm) >= 0) {
    p = sfft_make_plan_params(n, k, (enum sfft_version)version, &prm, &o);
    tuned = p != nullptr;
  }
  return p;
}

}  // namespace sfft

extern "C" {

int sfft_tuned_params(int n, int k, int version, sfft_params *params) {
  if (!params || n < 2 || k < 1 || version < 0 || version > 1) return -1;
  return sfft::tuned_lookup(n, k, version, *params);
}

int sfft_tuned_k(int k) { return sfft::k_bucket(k); }

}  // extern "C"
