// planner.cpp -- orders each rule's similarity predicates by measured
// selectivity and cost.
//
// The reference evaluates predicates in YAML order, equalities first
// (execution_plan_generator.h:111-137) and never uses its declared
// Prioritizer() (execution_plan_generator.h:223).  Here equalities always run
// first, as the equality join that produces candidate blocks, and the
// similarity predicates of a rule are ordered by
//     rank = cost / (1 - pass_rate)
// ascending (the classic optimal order for a conjunction of independent
// filters), with pass_rate and cost measured on a seeded sample of row pairs.
// AND is commutative, so the order changes work, never the result.
#include <algorithm>
#include <cstring>
#include <numeric>

#include "hbx_core.h"

namespace hbx {

namespace {

inline size_t c_len(const Column& c, int64_t i) {
  const char* p = c.ptr(i);
  const void* z = std::memchr(p, 0, (size_t)c.len(i));
  return z ? (size_t)((const char*)z - p) : (size_t)c.len(i);
}

// Jaro match count by the greedy scan (maximum matching inside the window
// h = (min_len + 1) / 2); sampling only, so no 256-byte cap handling.
double approx_jw(const char* a, size_t la, const char* b, size_t lb) {
  if (la == 0 || lb == 0) return (la == 0 && lb == 0) ? 1.0 : 0.0;
  const size_t ls = std::min(la, lb), ll = std::max(la, lb);
  const size_t h = (ls + 1) / 2;
  std::vector<char> used(la, 0);
  size_t m = 0;
  for (size_t i = 0; i < lb; i++) {
    size_t lo = i > h ? i - h : 0, hi = std::min(la - 1, i + h);
    if (lo > hi || lo >= la) continue;
    for (size_t j = lo; j <= hi; j++)
      if (!used[j] && a[j] == b[i]) {
        used[j] = 1;
        m++;
        break;
      }
  }
  if (!m) return 0.0;
  double j = ((double)m / ls + (double)m / ll + 1.0) / 3.0;
  size_t p = 0;
  while (p < ls && a[p] == b[p]) p++;
  j += (1.0 - j) * (double)p * 0.1;
  return j > 1.0 ? 1.0 : j;
}

}  // namespace

void order_predicates(Plan* plan, const Table& left, const Table& right) {
  if (left.n_rows == 0 || right.n_rows == 0) return;
  const int kSamples = 2048;
  uint64_t state = 0x48594250ull;
  auto next = [&]() {
    state = state * 6364136223846793005ull + 1442695040888963407ull;
    return state >> 17;
  };
  std::vector<std::pair<int64_t, int64_t>> pairs;
  for (int i = 0; i < kSamples; i++)
    pairs.emplace_back((int64_t)(next() % (uint64_t)left.n_rows),
                       (int64_t)(next() % (uint64_t)right.n_rows));
  for (auto& cr : plan->compiled) {
    if (cr.sims.size() < 2) continue;
    std::vector<double> rank(cr.sims.size());
    for (size_t s = 0; s < cr.sims.size(); s++) {
      const Pred& p = cr.sims[s];
      if (p.col_l >= left.n_cols() || p.col_r >= right.n_cols()) {
        rank[s] = 1e30;
        continue;
      }
      const Column& cl = left.cols[(size_t)p.col_l];
      const Column& cr2 = right.cols[(size_t)p.col_r];
      double pass = 0, cost = 0;
      for (auto& pr : pairs) {
        size_t la = c_len(cl, pr.first), lb = c_len(cr2, pr.second);
        cost += (double)lb * (double)((std::min<size_t>(la, 256) + 31) / 32 + 2);
        if (approx_jw(cl.ptr(pr.first), la, cr2.ptr(pr.second), lb) >= (double)p.thr) pass += 1;
      }
      pass /= (double)pairs.size();
      cost /= (double)pairs.size();
      rank[s] = cost / std::max(1e-3, 1.0 - pass);
    }
    std::vector<size_t> ord(cr.sims.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return rank[a] < rank[b]; });
    std::vector<Pred> sorted;
    for (size_t k : ord) sorted.push_back(cr.sims[k]);
    cr.sims = std::move(sorted);
  }
}

}  // namespace hbx
