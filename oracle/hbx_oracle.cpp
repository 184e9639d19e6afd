// hbx_oracle.cpp -- CPU oracle for the rule-based blocking hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs may load
// it.  The product (libhbx.so) never links, loads or calls it.
//
// It restates, in plain C++17, the reference's algorithm for the pair
// evaluation path of HyperBlocker:
//   * partitioning            core/components/data_mngr.h:150-207
//   * plan interpretation     core/gpu/global_func.cuh:115-183 (blocking_kernel)
//   * string equality         core/gpu/device_func.cuh:39-52  (equalities_kernel)
//   * Jaro ratio              core/gpu/device_func.cuh:54-132 (lev_jaro_ratio)
//   * Jaro-Winkler            core/gpu/device_func.cuh:210-231 (lev_jaro_winkler_ratio)
//   * rule ordering           core/components/execution_plan_generator.h:75-79
//
// The evaluation is the reference's brute-force nested loop over every
// left x right pair of every partition, so it is also the honest CPU
// baseline of that algorithm.  Work is split over std::threads by left row.
//
// Two places where the reference has undefined behaviour get a stated
// definition here (the GPU engine implements the same definition):
//   * lev_jaro_ratio indexes a uint16_t idx[256] with j up to 256 when the
//     shorter string is longer than 256 bytes (device_func.cuh:83,103-107).
//     The oracle gives idx 257 entries, i.e. position 256 behaves like any
//     other position.
//   * lev_jaro_winkler_ratio's update j += (1-j)*p*0.1 may be contracted to an
//     FMA by nvcc.  hbo_jw() takes fma_mode: 1 = fma((1-j)*p, 0.1, j) (what
//     nvcc's default --fmad=true produces), 0 = separate multiply and add.
//     hbo_block() evaluates both and counts threshold decisions that differ.

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <vector>

extern "C" {

// One table: n_rows x n_cols cells, row-major, each cell (ptr, len).
// Cells need not be NUL-terminated; len is the std::string length the
// reference hashes (data_mngr.h:157); equality and JW use the bytes up to the
// first NUL, as the reference's NUL-terminated device strings do.
typedef struct {
  int64_t n_rows;
  int32_t n_cols;
  const char* const* cell_ptr;  // [n_rows * n_cols]
  const int64_t* cell_len;      // [n_rows * n_cols]
} hbo_table;

typedef struct {
  int64_t pairs_covered;        // sum over partitions of |L_p| * |R_p|
  int64_t pair_comparisons;     // (rule, l, r) triples whose equalities all hold
  int64_t n_matches;            // emitted pairs
  int64_t fma_ambiguous;        // JW threshold decisions that differ fma vs no-fma
  int64_t long_string_pairs;    // JW calls whose shorter string exceeds 256 bytes
  // FP64 report: every JW evaluation is also computed with no float rounding
  // at all (jw_fp64 below); the reference's decisions stay the ones above
  int64_t jw_evals;             // JW evaluations (pair, similarity predicate)
  int64_t fp64_flips;           // evaluations whose threshold decision differs in FP64
  double fp64_max_abs_diff;     // max |JW (reference float/double path) - JW (FP64)|
} hbo_stats;

}  // extern "C"

namespace {

const int kCheckPoint = INT_MAX;  // core/common/types.h:13

inline size_t c_strnlen(const char* p, int64_t len) {
  const void* z = std::memchr(p, 0, (size_t)len);
  return z ? (size_t)((const char*)z - p) : (size_t)len;
}

// device_func.cuh:39-52: bytes equal up to and including the terminator.
inline bool ref_equal(const char* a, size_t la, const char* b, size_t lb) {
  return la == lb && std::memcmp(a, b, la) == 0;
}

// device_func.cuh:54-132, restated loop for loop.  Strings are given with
// their strlen; s[len] reads as the terminator (never equal to a character of
// the other string inside its own length).
//
// Split in two: ref_jaro_matches runs the two greedy loops (65-111) and
// returns the match count m; ref_jaro_value applies the formula (127-128).
// Both take the strings already swapped so that the first is the shorter
// (71-79), and non-empty.
size_t ref_jaro_matches(const char* term_l, size_t len_l, const char* term_r, size_t len_r) {
  const size_t halflen = (len_l + 1) / 2;
  uint16_t idx[257];
  std::memset(idx, 0, sizeof(idx));
  size_t match = 0;
  auto at_l = [&](size_t j) -> char { return j < len_l ? term_l[j] : '\0'; };
  // first loop: i in [0, halflen), j in [0, i + halflen], stop at j >= 256
  for (size_t i = 0; i < halflen; i++) {
    for (size_t j = 0; j <= i + halflen; j++) {
      if (j >= 256) break;
      if (at_l(j) == term_r[i] && !idx[j]) {
        match++;
        idx[j] = (uint16_t)match;
        break;
      }
    }
  }
  const size_t to = len_l + halflen < len_r ? len_l + halflen : len_r;
  // second loop: i in [halflen, to), j in [i - halflen, len_l), stop at j > 256
  for (size_t i = halflen; i < to; i++) {
    for (size_t j = i - halflen; j < len_l; j++) {
      if (j > 256) break;
      if (term_l[j] == term_r[i] && !idx[j]) {
        match++;
        idx[j] = (uint16_t)match;
        break;
      }
    }
  }
  // transpositions are counted by the reference (116-126) and never used.
  return match;
}

float ref_jaro_value(size_t match, size_t len_l, size_t len_r) {
  if (!match) return 0.0f;
  const float md = (float)match;
  // (md / len_l + md / len_r + 1.0) / 3.0 : float quotients, float sum,
  // then double add and divide, rounded to float on return (127-128).
  const float q = md / (float)len_l + md / (float)len_r;
  volatile double t = (double)q + 1.0;  // volatile: keep the double rounding steps
  const double r = t / 3.0;
  return (float)r;
}

// Match count m and the Jaro value of two strings given with their strlen
// (65-69: both empty -> 1, one empty -> 0, m = 0 for those).
float ref_jaro_m(const char* term_l, size_t len_l, const char* term_r, size_t len_r, size_t* m_out) {
  *m_out = 0;
  if (len_r == 0 || len_l == 0) {
    if (len_l == 0 && len_r == 0) return 1.0f;
    return 0.0f;
  }
  if (len_l > len_r) {
    std::swap(term_l, term_r);
    std::swap(len_l, len_r);
  }
  *m_out = ref_jaro_matches(term_l, len_l, term_r, len_r);
  return ref_jaro_value(*m_out, len_l, len_r);
}

float ref_jaro(const char* term_l, size_t len_l, const char* term_r, size_t len_r) {
  size_t m;
  return ref_jaro_m(term_l, len_l, term_r, len_r, &m);
}

// Common prefix of the unswapped strings up to min(len1, len2), uncapped
// (device_func.cuh:218-226).
size_t ref_prefix(const char* s1, size_t l1, const char* s2, size_t l2) {
  const size_t m = l1 < l2 ? l1 : l2;
  size_t p = 0;
  for (p = 0; p < m; p++)
    if (s1[p] != s2[p]) break;
  return p;
}

// device_func.cuh:227-230 from the Jaro value j and the prefix p:
// j += (1 - j) * p * 0.1 in double (fma_mode as described in the header),
// clamped to 1.
double ref_jw_from(double j, size_t p, int fma_mode) {
  volatile double a = (1.0 - j) * (double)p;
  double out;
  if (fma_mode) {
    out = std::fma((double)a, 0.1, j);
  } else {
    volatile double b = (double)a * 0.1;
    out = j + (double)b;
  }
  return out > 1.0 ? 1.0 : out;
}

// device_func.cuh:210-231.  pfweight = 0.1; the prefix is taken on the
// unswapped strings up to min(len1, len2), without the textbook cap of 4.
double ref_jw(const char* s1, size_t l1, const char* s2, size_t l2, int fma_mode,
              size_t* prefix_out) {
  const double j = ref_jaro(s1, l1, s2, l2);
  const size_t p = ref_prefix(s1, l1, s2, l2);
  if (prefix_out) *prefix_out = p;
  return ref_jw_from(j, p, fma_mode);
}

// The same Jaro-Winkler value with no float rounding anywhere: the match
// count m, lengths and prefix of the reference's loops, then
// j = (m / ls + m / ll + 1) / 3 and j + (1 - j) * p * 0.1 in double
// (clamped to 1).  Not the reference's arithmetic: it is the report of how
// far the reference's float/double path lies from a double evaluation.
double jw_fp64(size_t m, size_t l1, size_t l2, size_t p) {
  double j;
  if (l1 == 0 || l2 == 0) {
    j = (l1 == 0 && l2 == 0) ? 1.0 : 0.0;
  } else if (m == 0) {
    j = 0.0;
  } else {
    const double ls = (double)(l1 < l2 ? l1 : l2), ll = (double)(l1 < l2 ? l2 : l1);
    j = ((double)m / ls + (double)m / ll + 1.0) / 3.0;
  }
  const double out = j + (1.0 - j) * (double)p * 0.1;
  return out > 1.0 ? 1.0 : out;
}

struct Cell {
  const char* p;
  size_t n;       // strnlen (what the device functions see)
  int64_t full;   // std::string length (what std::hash sees)
};

inline Cell cell(const hbo_table* t, int64_t row, int col) {
  const int64_t k = row * t->n_cols + col;
  Cell c;
  c.p = t->cell_ptr[k];
  c.full = t->cell_len[k];
  c.n = c_strnlen(c.p, c.full);
  return c;
}

inline size_t std_hash(const char* p, int64_t n) {
  return std::hash<std::string>{}(std::string(p, (size_t)n));
}

// data_mngr.h:150-172 (left) and 180-202 (right): the same code for both
// tables; the right table is hashed on the LEFT column index of plan slot 0.
void partition_rows(const hbo_table* t, const int* pred_index, const char* pred_type,
                    int plan_len, uint64_t n_part, int prefix_idx,
                    std::vector<std::vector<int64_t>>* buckets) {
  buckets->assign(n_part, {});
  for (int64_t i = 0; i < t->n_rows; i++) {
    int bucket_id = 0;
    for (int j = 0; j < plan_len && j < 1 /* MAX_HASH_TIMES */; j++) {
      if (pred_type[j] == 'e') {
        Cell c = cell(t, i, pred_index[j]);
        size_t local = std_hash(c.p, c.full) % n_part;
        bucket_id = (int)(((size_t)bucket_id + local) % n_part);
      }
    }
    if (prefix_idx != INT_MAX) {
      Cell c = cell(t, i, prefix_idx);
      if (c.full > 2) {
        size_t two_d = (std_hash(c.p, 1) + (size_t)bucket_id) % n_part;
        bucket_id = (int)(((size_t)bucket_id + two_d) % n_part);
      }
    }
    (*buckets)[bucket_id].push_back(i);
  }
}

struct Eval {
  const hbo_table* L;
  const hbo_table* R;
  const int* pred_index;
  const char* pred_type;
  const float* pred_threshold;
  int plan_len;
  int fma_mode;
};

struct ThreadOut {
  std::vector<uint32_t> l, r;
  int64_t comparisons = 0;
  int64_t ambiguous = 0;
  int64_t long_pairs = 0;
  int64_t jw_evals = 0;
  int64_t fp64_flips = 0;
  double fp64_max = 0.0;
};

// global_func.cuh:117-183 for one (l, r) pair.  Also counts the rule
// candidates (triples whose equalities hold) for the pair-comparison metric;
// that count walks every rule and is independent of the short-circuit.
bool eval_pair(const Eval& E, int64_t row_l, int64_t row_r, ThreadOut* to) {
  const int len = E.plan_len;
  // metric: per rule, do all equalities hold?
  {
    bool all_eq = true;
    for (int i = 0; i < len;) {
      if (E.pred_index[i] == kCheckPoint) {
        if (all_eq) to->comparisons++;
        all_eq = true;
        i += 1;
        continue;
      }
      if (E.pred_type[i] == 'e' && all_eq) {
        Cell a = cell(E.L, row_l, E.pred_index[i]);
        Cell b = cell(E.R, row_r, E.pred_index[i + 1]);
        if (!ref_equal(a.p, a.n, b.p, b.n)) all_eq = false;
      }
      i += 2;
    }
  }
  bool is_match = false;
  for (int i = 0; i < len; i += 2) {
    bool to_skip = false;
    const int pl = E.pred_index[i];
    const int pr = E.pred_index[i + 1];
    switch (E.pred_type[i]) {
      case 'e': {
        Cell a = cell(E.L, row_l, pl);
        Cell b = cell(E.R, row_r, pr);
        if (!ref_equal(a.p, a.n, b.p, b.n)) to_skip = true;
        break;
      }
      case 's': {
        Cell a = cell(E.L, row_l, pl);
        Cell b = cell(E.R, row_r, pr);
        if (std::min(a.n, b.n) > 256) to->long_pairs++;
        // one run of the loops (m) and of the prefix serves the FMA form,
        // the separate form and the FP64 report
        size_t m = 0;
        const double j = ref_jaro_m(a.p, a.n, b.p, b.n, &m);
        const size_t p = ref_prefix(a.p, a.n, b.p, b.n);
        const double sim = ref_jw_from(j, p, E.fma_mode);
        const double other = ref_jw_from(j, p, !E.fma_mode);
        const double thr = (double)E.pred_threshold[i];
        if ((sim < thr) != (other < thr)) to->ambiguous++;
        const double wide = jw_fp64(m, a.n, b.n, p);
        to->jw_evals++;
        if ((wide < thr) != (sim < thr)) to->fp64_flips++;
        to->fp64_max = std::max(to->fp64_max, std::fabs(sim - wide));
        if (sim < thr) to_skip = true;
        break;
      }
      default:
        break;
    }
    if (to_skip) {
      while (i + 2 < len) {
        if (E.pred_index[i + 2] == kCheckPoint) {
          i++;
          break;
        }
        i += 2;
      }
    } else {
      if (i < len && i + 2 < len && E.pred_index[i + 2] == kCheckPoint) {
        is_match = true;
        break;
      }
    }
  }
  return is_match;
}

}  // namespace

extern "C" {

// Reference Jaro ratio (float) of two byte strings.
float hbo_jaro(const char* a, int64_t la, const char* b, int64_t lb) {
  return ref_jaro(a, c_strnlen(a, la), b, c_strnlen(b, lb));
}

// Reference Jaro-Winkler (double); fma_mode as described in the header.
double hbo_jw(const char* a, int64_t la, const char* b, int64_t lb, int fma_mode) {
  return ref_jw(a, c_strnlen(a, la), b, c_strnlen(b, lb), fma_mode, nullptr);
}

// The FP64 restatement of Jaro-Winkler (jw_fp64) of two byte strings.
double hbo_jw_fp64(const char* a, int64_t la, const char* b, int64_t lb) {
  const size_t na = c_strnlen(a, la), nb = c_strnlen(b, lb);
  size_t m = 0;
  ref_jaro_m(a, na, b, nb, &m);
  return jw_fp64(m, na, nb, ref_prefix(a, na, b, nb));
}

// libstdc++ std::hash<std::string> of a byte string (data_mngr.h:157).
uint64_t hbo_std_hash(const char* p, int64_t n) { return (uint64_t)std_hash(p, n); }

// Permutation that std::sort with the reference's comparator
// (execution_plan_generator.h:75-79: equality-vector size, descending)
// applies to rules read in directory order.
void hbo_sort_rules(const int32_t* eq_sizes, int32_t n, int32_t* perm) {
  struct R {
    int32_t eq;
    int32_t idx;
  };
  std::vector<R> v((size_t)n);
  for (int32_t i = 0; i < n; i++) v[i] = {eq_sizes[i], i};
  std::sort(v.begin(), v.end(), [](const R& a, const R& b) { return a.eq > b.eq; });
  for (int32_t i = 0; i < n; i++) perm[i] = v[i].idx;
}

// Bucket of every row of one table (data_mngr.h:150-202).
void hbo_partition(const hbo_table* t, const int* pred_index, const char* pred_type,
                   int plan_len, uint64_t n_part, int prefix_idx, int32_t* bucket_out) {
  std::vector<std::vector<int64_t>> b;
  partition_rows(t, pred_index, pred_type, plan_len, n_part, prefix_idx, &b);
  for (uint64_t p = 0; p < n_part; p++)
    for (int64_t r : b[p]) bucket_out[r] = (int32_t)p;
}

// The whole path: partition both tables, then evaluate every pair of every
// partition (data_mngr.h:209-215 drops partitions with an empty side, which
// contribute no pairs).  Writes matching (left row, right row) pairs sorted by
// (l, r).  Returns the number of matches, or -(needed) if capacity is short
// (nothing written in that case).  left_row_filter (nullable, n_rows_l bytes)
// restricts evaluation to a sample of left rows.
int64_t hbo_block(const hbo_table* L, const hbo_table* R, const int* pred_index,
                  const char* pred_type, const float* pred_threshold, int plan_len,
                  uint64_t n_partitions, int prefix_idx, int fma_mode, int n_threads,
                  const uint8_t* left_row_filter, uint32_t* out_l, uint32_t* out_r,
                  int64_t capacity, hbo_stats* stats) {
  if (n_partitions == 0 || plan_len <= 0) return 0;
  std::vector<std::vector<int64_t>> bl, br;
  partition_rows(L, pred_index, pred_type, plan_len, n_partitions, prefix_idx, &bl);
  partition_rows(R, pred_index, pred_type, plan_len, n_partitions, prefix_idx, &br);
  Eval E{L, R, pred_index, pred_type, pred_threshold, plan_len, fma_mode};

  // Flatten (partition, left row) work so threads share it evenly.
  struct Item {
    uint64_t part;
    int64_t row_l;
  };
  std::vector<Item> items;
  int64_t covered = 0;
  for (uint64_t p = 0; p < n_partitions; p++) {
    if (bl[p].empty() || br[p].empty()) continue;
    for (int64_t rl : bl[p]) {
      if (left_row_filter && !left_row_filter[rl]) continue;
      items.push_back({p, rl});
      covered += (int64_t)br[p].size();
    }
  }
  if (n_threads < 1) n_threads = 1;
  std::vector<ThreadOut> outs((size_t)n_threads);
  std::atomic<size_t> next{0};
  auto worker = [&](int tid) {
    ThreadOut& o = outs[(size_t)tid];
    for (;;) {
      const size_t k = next.fetch_add(16);
      if (k >= items.size()) break;
      const size_t end = std::min(items.size(), k + 16);
      for (size_t x = k; x < end; x++) {
        const Item& it = items[x];
        for (int64_t rr : br[it.part]) {
          if (eval_pair(E, it.row_l, rr, &o)) {
            o.l.push_back((uint32_t)it.row_l);
            o.r.push_back((uint32_t)rr);
          }
        }
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < n_threads; t++) th.emplace_back(worker, t);
  worker(0);
  for (auto& t : th) t.join();

  std::vector<std::pair<uint32_t, uint32_t>> all;
  hbo_stats s{};
  s.pairs_covered = covered;
  for (auto& o : outs) {
    for (size_t i = 0; i < o.l.size(); i++) all.emplace_back(o.l[i], o.r[i]);
    s.pair_comparisons += o.comparisons;
    s.fma_ambiguous += o.ambiguous;
    s.long_string_pairs += o.long_pairs;
    s.jw_evals += o.jw_evals;
    s.fp64_flips += o.fp64_flips;
    s.fp64_max_abs_diff = std::max(s.fp64_max_abs_diff, o.fp64_max);
  }
  std::sort(all.begin(), all.end());
  s.n_matches = (int64_t)all.size();
  if (stats) *stats = s;
  if ((int64_t)all.size() > capacity) return -(int64_t)all.size();
  for (size_t i = 0; i < all.size(); i++) {
    out_l[i] = all[i].first;
    out_r[i] = all[i].second;
  }
  return (int64_t)all.size();
}

}  // extern "C"
