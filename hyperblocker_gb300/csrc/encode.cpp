// encode.cpp -- turns two host tables into the engine's device layout.
//
// * Partition bucket of every row, computed exactly as the reference does
//   (core/components/data_mngr.h:150-202): std::hash of the cell in column
//   pred_index[0] (the LEFT column index of plan slot 0, used for both tables)
//   when slot 0 is an equality, plus the optional first-character prefix
//   hash.  libstdc++'s std::hash<std::string_view> is the same function as
//   std::hash<std::string>.
// * Equality columns: one joint dictionary per (left column, right column)
//   pair, so two cells are equal (equalities_kernel, device_func.cuh:39-52,
//   which compares up to the first NUL) iff their int32 codes are equal.
// * String columns of similarity predicates: symbols (a frequency-ordered
//   bijection of the bytes that occur, 0 reserved for padding), each string
//   starting on a 16-byte boundary of one arena and zero padded to the next
//   boundary; lengths are kept in a parallel array (structure of arrays) so
//   that a warp's length reads coalesce and string data stays aligned for
//   16-byte vector loads.
#include "encode.h"

#include <algorithm>
#include <climits>
#include <cstring>
#include <functional>
#include <numeric>
#include <string>
#include <string_view>
#include <unordered_map>

namespace hbx {

namespace {

inline std::string_view cell_full(const Column& c, int64_t i) {
  return std::string_view(c.ptr(i), (size_t)c.len(i));
}

inline std::string_view cell_c(const Column& c, int64_t i) {
  std::string_view s = cell_full(c, i);
  size_t z = s.find('\0');
  return z == std::string_view::npos ? s : s.substr(0, z);
}

void compute_buckets(const Table& t, int part_col, uint64_t n, int64_t prefix_idx,
                     std::vector<uint32_t>* out) {
  out->assign((size_t)t.n_rows, 0);
  std::hash<std::string_view> H;
  for (int64_t i = 0; i < t.n_rows; i++) {
    uint64_t b = 0;
    if (part_col >= 0) {
      uint64_t local = (uint64_t)H(cell_full(t.cols[(size_t)part_col], i)) % n;
      b = (b + local) % n;
    }
    if (prefix_idx != INT_MAX) {
      std::string_view s = cell_full(t.cols[(size_t)prefix_idx], i);
      if (s.size() > 2) {
        uint64_t two_d = ((uint64_t)H(s.substr(0, 1)) + b) % n;
        b = (b + two_d) % n;
      }
    }
    (*out)[(size_t)i] = (uint32_t)b;
  }
}

void check_col(const Table& t, int col, const char* side, const char* what) {
  if (col < 0 || col >= t.n_cols())
    fail(HBX_ERR_UNSUPPORTED, std::string(what) + " uses column " + std::to_string(col) +
                                  " which the " + side + " table does not have");
}

}  // namespace

Encoded encode_schema(const Plan& plan, const Table& left, const Table& right,
                      uint64_t n_partitions, int64_t prefix_idx) {
  if (n_partitions == 0) fail(HBX_ERR_INVALID_ARG, "n_partitions must be >= 1");
  if (n_partitions > (1ull << 20)) fail(HBX_ERR_UNSUPPORTED, "n_partitions above 2^20");
  if (left.n_rows > (int64_t)UINT32_MAX - 1 || right.n_rows > (int64_t)UINT32_MAX - 1)
    fail(HBX_ERR_UNSUPPORTED, "more than 2^32 - 2 rows in a table");
  Encoded E;
  E.n_partitions = n_partitions;
  E.prefix_idx = prefix_idx;
  E.L.n_rows = left.n_rows;
  E.R.n_rows = right.n_rows;

  // ---- partition key (data_mngr.h:150-202)
  if (!plan.pred_type.empty() && plan.pred_type[0] == 'e') E.part_col = plan.pred_index[0];
  if (left.n_cols() == 0 || right.n_cols() == 0) fail(HBX_ERR_UNSUPPORTED, "table without columns");
  if (E.part_col >= 0) {
    check_col(left, E.part_col, "left", "the partition key");
    check_col(right, E.part_col, "right", "the partition key");
  }
  if (prefix_idx != INT_MAX) {
    check_col(left, (int)prefix_idx, "left", "prefix_hash_pred_idx");
    check_col(right, (int)prefix_idx, "right", "prefix_hash_pred_idx");
  }

  // ---- columns the rules use; output ids are column 0 of each table
  for (auto& cr : plan.compiled) {
    for (auto& p : cr.eqs) {
      check_col(left, p.col_l, "left", "an equality");
      check_col(right, p.col_r, "right", "an equality");
    }
    for (auto& p : cr.sims) {
      check_col(left, p.col_l, "left", "a similarity predicate");
      check_col(right, p.col_r, "right", "a similarity predicate");
    }
  }

  // ---- equality slots (one joint dictionary each) and string slots
  auto eq_slot_of = [&](int cl, int crr) {
    for (size_t s = 0; s < E.eq_slots.size(); s++)
      if (E.eq_slots[s].first == cl && E.eq_slots[s].second == crr) return (int)s;
    E.eq_slots.emplace_back(cl, crr);
    return (int)E.eq_slots.size() - 1;
  };
  auto str_slot_of = [&](SideEnc& S, int col) {
    for (size_t s = 0; s < S.str_col.size(); s++)
      if (S.str_col[s] == col) return (int)s;
    S.str_col.push_back(col);
    return (int)S.str_col.size() - 1;
  };
  for (auto& cr : plan.compiled)
    for (auto& p : cr.eqs) eq_slot_of(p.col_l, p.col_r);
  for (auto& cr : plan.compiled)
    for (auto& p : cr.sims) {
      str_slot_of(E.L, p.col_l);
      str_slot_of(E.R, p.col_r);
    }
  for (auto& cr : plan.compiled) {
    RuleEnc re;
    for (auto& p : cr.eqs) re.eq_slot.push_back(eq_slot_of(p.col_l, p.col_r));
    for (auto& p : cr.sims) {
      re.sim_slot_l.push_back(str_slot_of(E.L, p.col_l));
      re.sim_slot_r.push_back(str_slot_of(E.R, p.col_r));
      re.thr.push_back(p.thr);
    }
    E.rules.push_back(std::move(re));
  }
  return E;
}

void encode_rows(const Table& left, const Table& right, Encoded* Ep) {
  Encoded& E = *Ep;
  const uint64_t n_partitions = E.n_partitions;
  for (SideEnc* S : {&E.L, &E.R}) {  // everything below is (re)built from scratch
    S->comp_codes.clear();
    S->arena.clear();
    S->str_off.clear();
    S->str_len.clear();
    S->str_maxlen.clear();
  }
  compute_buckets(left, E.part_col, n_partitions, E.prefix_idx, &E.L.bucket);
  compute_buckets(right, E.part_col, n_partitions, E.prefix_idx, &E.R.bucket);
  {
    std::vector<uint64_t> hl(n_partitions, 0), hr(n_partitions, 0);
    for (uint32_t b : E.L.bucket) hl[b]++;
    for (uint32_t b : E.R.bucket) hr[b]++;
    E.pairs_covered = 0;
    E.n_partitions_used = 0;
    for (uint64_t p = 0; p < n_partitions; p++) {
      E.pairs_covered += hl[p] * hr[p];
      if (hl[p] && hr[p]) E.n_partitions_used++;
    }
  }

  // ---- joint dictionaries: two cells are equal (equalities_kernel,
  // device_func.cuh:39-52, compares up to the first NUL) iff their codes are
  E.L.eq_codes.clear();
  E.R.eq_codes.clear();
  E.eq_card.clear();
  for (auto& slot : E.eq_slots) {
    std::unordered_map<std::string_view, int32_t> dict;
    dict.reserve((size_t)(left.n_rows + right.n_rows) / 4 + 16);
    auto enc_side = [&](const Table& t, int col, std::vector<int32_t>* out) {
      const Column& c = t.cols[(size_t)col];
      out->resize((size_t)t.n_rows);
      for (int64_t i = 0; i < t.n_rows; i++) {
        auto it = dict.emplace(cell_c(c, i), (int32_t)dict.size()).first;
        (*out)[(size_t)i] = it->second;
      }
    };
    E.L.eq_codes.emplace_back();
    E.R.eq_codes.emplace_back();
    enc_side(left, slot.first, &E.L.eq_codes.back());
    enc_side(right, slot.second, &E.R.eq_codes.back());
    E.eq_card.push_back((uint32_t)std::max<size_t>(dict.size(), 1));
  }

  // ---- the symbol alphabet of the string slots
  uint64_t freq[256] = {0};
  auto count_side = [&](const Table& t, const SideEnc& S) {
    for (int col : S.str_col) {
      const Column& c = t.cols[(size_t)col];
      for (int64_t i = 0; i < t.n_rows; i++)
        for (unsigned char ch : cell_c(c, i)) freq[ch]++;
    }
  };
  count_side(left, E.L);
  count_side(right, E.R);
  {
    std::vector<int> bytes;
    for (int b = 1; b < 256; b++)
      if (freq[b]) bytes.push_back(b);
    std::stable_sort(bytes.begin(), bytes.end(), [&](int a, int b) { return freq[a] > freq[b]; });
    E.sym_of_byte.fill(0);
    for (size_t k = 0; k < bytes.size(); k++) E.sym_of_byte[(size_t)bytes[k]] = (uint8_t)(k + 1);
    E.n_symbols = (uint32_t)bytes.size() + 1;
  }
  auto pack_side = [&](const Table& t, SideEnc& S) {
    uint64_t total = 0;
    for (int col : S.str_col) {
      const Column& c = t.cols[(size_t)col];
      for (int64_t i = 0; i < t.n_rows; i++) total += (cell_c(c, i).size() + 15) / 16 * 16;
    }
    total += 16;  // a zero block at the end: empty strings point there too
    if (total / 16 > UINT32_MAX) fail(HBX_ERR_UNSUPPORTED, "string arena above 64 GiB");
    S.arena.assign((size_t)total, 0);
    uint64_t pos = 0;
    for (int col : S.str_col) {
      const Column& c = t.cols[(size_t)col];
      std::vector<uint32_t> off((size_t)t.n_rows), len((size_t)t.n_rows);
      uint32_t mx = 0;
      for (int64_t i = 0; i < t.n_rows; i++) {
        std::string_view s = cell_c(c, i);
        off[(size_t)i] = (uint32_t)(pos / 16);
        len[(size_t)i] = (uint32_t)s.size();
        mx = std::max(mx, (uint32_t)s.size());
        uint8_t* dst = S.arena.data() + pos;
        for (size_t k = 0; k < s.size(); k++) dst[k] = E.sym_of_byte[(unsigned char)s[k]];
        pos += (s.size() + 15) / 16 * 16;
      }
      S.str_off.push_back(std::move(off));
      S.str_len.push_back(std::move(len));
      S.str_maxlen.push_back(mx);
    }
  };
  pack_side(left, E.L);
  pack_side(right, E.R);
}

bool rule_mixed_domain(const Encoded& E, RuleEnc* rp) {
  RuleEnc& re = *rp;
  const uint64_t n_partitions = E.n_partitions;
  re.radix.clear();
  re.part_key_begin.clear();
  re.composite = false;
  re.comp_index = -1;
  unsigned __int128 M = 1;
  for (int s : re.eq_slot) {
    re.radix.push_back(E.eq_card[(size_t)s]);
    M *= E.eq_card[(size_t)s];
  }
  const unsigned __int128 D = M * n_partitions;
  if (D > kMaxKeyDomain) return false;
  re.domain = (uint64_t)D;
  for (uint64_t p = 0; p <= n_partitions; p++) re.part_key_begin.push_back(p * (uint64_t)M);
  return true;
}

bool finish_rules(Encoded* Ep, bool allow_composite) {
  Encoded& E = *Ep;
  const uint64_t n_partitions = E.n_partitions;
  for (RuleEnc& re : E.rules) {
    // mixed-radix domain
    if (rule_mixed_domain(E, &re)) continue;
    if (!allow_composite) return false;
    // dense ids of the (bucket, codes...) tuples that occur, grouped by bucket
    re.composite = true;
    re.comp_index = (int)E.L.comp_codes.size();
    std::unordered_map<std::string, int32_t> ids;
    std::vector<uint32_t> id_bucket;
    std::string key;
    auto tuple_id = [&](const SideEnc& S, int64_t i) {
      key.clear();
      uint32_t b = S.bucket[(size_t)i];
      key.append((const char*)&b, 4);
      for (int s : re.eq_slot) key.append((const char*)&S.eq_codes[(size_t)s][(size_t)i], 4);
      auto it = ids.emplace(key, (int32_t)ids.size());
      if (it.second) id_bucket.push_back(b);
      return it.first->second;
    };
    std::vector<int32_t> tl((size_t)E.L.n_rows), tr((size_t)E.R.n_rows);
    for (int64_t i = 0; i < E.L.n_rows; i++) tl[(size_t)i] = tuple_id(E.L, i);
    for (int64_t i = 0; i < E.R.n_rows; i++) tr[(size_t)i] = tuple_id(E.R, i);
    std::vector<uint64_t> start(n_partitions + 1, 0);
    for (uint32_t b : id_bucket) start[b + 1]++;
    for (uint64_t p = 0; p < n_partitions; p++) start[p + 1] += start[p];
    std::vector<int32_t> remap(id_bucket.size());
    std::vector<uint64_t> cur(start.begin(), start.end() - 1);
    for (size_t k = 0; k < id_bucket.size(); k++) remap[k] = (int32_t)cur[id_bucket[k]]++;
    for (auto& v : tl) v = remap[(size_t)v];
    for (auto& v : tr) v = remap[(size_t)v];
    E.L.comp_codes.push_back(std::move(tl));
    E.R.comp_codes.push_back(std::move(tr));
    re.domain = std::max<uint64_t>(id_bucket.size(), 1);
    re.part_key_begin = start;
    if (re.domain > (1ull << 31)) fail(HBX_ERR_UNSUPPORTED, "join key domain too large");
  }
  return true;
}

Encoded encode(const Plan& plan, const Table& left, const Table& right, uint64_t n_partitions,
               int64_t prefix_idx) {
  Encoded E = encode_schema(plan, left, right, n_partitions, prefix_idx);
  encode_rows(left, right, &E);
  finish_rules(&E, true);
  return E;
}

}  // namespace hbx
