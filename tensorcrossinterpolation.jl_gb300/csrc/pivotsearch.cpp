// Greedy point searches over a solve's f, run for many start points in lockstep
// so that each step is one device evaluation (EVAL tasks, f and the train):
//   optfirstpivot (util.jl:78-108): coordinate ascent of |f|;
//   estimatetrueerror / _floatingzone (globalsearch.jl:1-96): coordinate ascent
//   of |f - tt| with the solve's site tensors.
#include <algorithm>
#include <cmath>

#include "engine.h"

namespace tci {

namespace {

// Every point that differs from the active starts' pivots at `site` only, for
// each start in `who` (local index fastest).
std::vector<uint8_t> site_variants(const std::vector<std::vector<uint8_t>>& piv, const std::vector<int>& who,
                                   int site, int D) {
  std::vector<uint8_t> pts;
  const size_t L = piv.empty() ? 0 : piv[0].size();
  pts.reserve(who.size() * (size_t)D * L);
  for (int q : who)
    for (int v = 0; v < D; ++v) {
      pts.insert(pts.end(), piv[(size_t)q].begin(), piv[(size_t)q].end());
      pts[pts.size() - L + (size_t)site] = (uint8_t)v;
    }
  return pts;
}

}  // namespace

// For one site the reference's greedy scan (pivot[i] = d kept when |f| beats the
// running best, strictly) ends at the first maximum above the current value, so
// all candidates of a site can be evaluated at once.
CoTask co_optfirstpivots(Engine& e, Solve& s, std::vector<std::vector<uint8_t>>* piv, std::vector<double>* valf,
                         int maxsweep) {
  const int n = (int)piv->size();
  valf->assign((size_t)n, 0.0);
  if (n == 0) co_return 0;
  {
    std::vector<uint8_t> pts;
    for (auto& p : *piv) pts.insert(pts.end(), p.begin(), p.end());
    std::vector<double> v((size_t)n);
    CO_TRY(co_evaluate(e, s, pts.data(), n, v.data(), nullptr));
    for (int q = 0; q < n; ++q) (*valf)[(size_t)q] = std::fabs(v[(size_t)q]);
  }
  std::vector<char> active((size_t)n, 1);
  for (int sweep = 0; sweep < maxsweep; ++sweep) {
    const std::vector<double> prev = *valf;
    std::vector<int> who;
    for (int q = 0; q < n; ++q)
      if (active[(size_t)q]) who.push_back(q);
    if (who.empty()) break;
    for (int site = 0; site < s.L; ++site) {
      const int D = s.d[(size_t)site];
      const std::vector<uint8_t> pts = site_variants(*piv, who, site, D);
      std::vector<double> vals(who.size() * (size_t)D);
      CO_TRY(co_evaluate(e, s, pts.data(), (i64)vals.size(), vals.data(), nullptr));
      for (size_t w = 0; w < who.size(); ++w) {
        const size_t q = (size_t)who[w];
        for (int v = 0; v < D; ++v) {
          const double nv = std::fabs(vals[w * (size_t)D + (size_t)v]);
          if (nv > (*valf)[q]) {
            (*valf)[q] = nv;
            (*piv)[q][(size_t)site] = (uint8_t)v;
          }
        }
      }
    }
    for (int q : who)
      if (prev[(size_t)q] == (*valf)[(size_t)q]) active[(size_t)q] = 0;
  }
  co_return 0;
}

// estimatetrueerror (globalsearch.jl:19-45) with _floatingzone (:48-96): per
// start, for each site in turn the error |f - tt| over the site's values, the
// pivot moved to its first maximum and maxerror = max(maximum(err), maxerror),
// sweeps until maxerror stops changing; then (pivot, error) sorted by error,
// descending (stable), repeats removed.
CoTask co_estimatetrueerror(Engine& e, Solve& s, std::vector<std::vector<uint8_t>> piv,
                            std::vector<std::pair<std::vector<uint8_t>, double>>* out) {
  out->clear();
  const int n = (int)piv.size();
  if (n == 0) co_return 0;
  std::vector<double> maxerr((size_t)n);
  {
    std::vector<uint8_t> pts;
    for (auto& p : piv) pts.insert(pts.end(), p.begin(), p.end());
    std::vector<double> fv((size_t)n), tv((size_t)n);
    CO_TRY(co_evaluate(e, s, pts.data(), n, fv.data(), tv.data()));
    for (int q = 0; q < n; ++q) maxerr[(size_t)q] = std::fabs(fv[(size_t)q] - tv[(size_t)q]);
  }
  std::vector<char> active((size_t)n, 1);
  for (;;) {
    const std::vector<double> prev = maxerr;
    std::vector<int> who;
    for (int q = 0; q < n; ++q)
      if (active[(size_t)q]) who.push_back(q);
    if (who.empty()) break;
    for (int site = 0; site < s.L; ++site) {
      const int D = s.d[(size_t)site];
      const std::vector<uint8_t> pts = site_variants(piv, who, site, D);
      std::vector<double> fv(who.size() * (size_t)D), tv(fv.size());
      CO_TRY(co_evaluate(e, s, pts.data(), (i64)fv.size(), fv.data(), tv.data()));
      for (size_t w = 0; w < who.size(); ++w) {
        const size_t q = (size_t)who[w];
        int arg = 0;
        double best = -1.0;
        for (int v = 0; v < D; ++v) {
          const double err = std::fabs(fv[w * (size_t)D + (size_t)v] - tv[w * (size_t)D + (size_t)v]);
          if (err > best) {  // argmax: the first maximum
            best = err;
            arg = v;
          }
        }
        piv[q][(size_t)site] = (uint8_t)arg;
        maxerr[q] = std::max(best, maxerr[q]);
      }
    }
    for (int q : who)
      if (maxerr[(size_t)q] == prev[(size_t)q]) active[(size_t)q] = 0;
  }
  std::vector<int> order((size_t)n);
  for (int q = 0; q < n; ++q) order[(size_t)q] = q;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return maxerr[(size_t)a] > maxerr[(size_t)b]; });
  for (int q : order) {
    std::pair<std::vector<uint8_t>, double> x{piv[(size_t)q], maxerr[(size_t)q]};
    if (std::find(out->begin(), out->end(), x) == out->end()) out->push_back(std::move(x));
  }
  co_return 0;
}

}  // namespace tci
