// jfem_tune.h — an entry of the batched solver's autotuner cache and the rule
// that decides whether a cached entry may be launched (host C++).
#pragma once

#include <cmath>

namespace jfem {

// One configuration in relative form, re-derived for each batch: block size
// and CTAs per SM of the single-CTA teams; for the clustered part the cluster
// size, its block size, the share of instances on clusters (the largest n/frac;
// frac 0: none) and cluster CTAs per SM; the batch time it was measured at.
struct TuneEntry {
  int bs, per_sm, cluster, bs_c, frac, per_sm_c;
  double ms;
};

// True exactly for the configurations the autotuner can choose.  Anything else
// read back from a cache file (another version's fields, a hand edit, a torn
// line) is ignored and the batch is tuned again, rather than launched with a
// block or cluster shape the kernels were not written for.
inline bool tune_entry_valid(const TuneEntry& e) {
  const bool bs_ok = e.bs == 128 || e.bs == 256 || e.bs == 512 || e.bs == 1024;
  const bool per_sm_ok = (e.per_sm == 1 || e.per_sm == 2 || e.per_sm == 4) && e.bs * e.per_sm <= 2048;
  const bool single = e.cluster == 1 && e.bs_c == 0 && e.frac == 0 && e.per_sm_c == 1;
  const bool clustered = (e.cluster == 2 || e.cluster == 4 || e.cluster == 8) && (e.bs_c == 256 || e.bs_c == 512) &&
                         (e.frac == 2 || e.frac == 4 || e.frac == 8) && (e.per_sm_c == 1 || e.per_sm_c == 2);
  return bs_ok && per_sm_ok && (single || clustered) && std::isfinite(e.ms) && e.ms >= 0.0;
}

}  // namespace jfem
