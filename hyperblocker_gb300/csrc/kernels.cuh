// kernels.cuh -- sm_103a device code of the blocking engine.
//
// Pipeline per run (all on one stream; the batched form is a CUDA graph):
//   1. k_keys_hist    join key of every row per rule (partition bucket and
//                     equality dictionary codes in mixed radix, or a dense
//                     composite id) + histogram of keys per side.
//   2. scan kernels   exclusive scans: row offsets per key, and work items
//                     per key (a work item = one left row x up to TR right rows
//                     of one candidate block).
//   3. k_scatter      rows grouped by key (counting sort) -> candidate blocks
//                     L_key x R_key.
//   4. k_peq_build    Peq bitmask table of every left string (built with
//                     __match_any), in device memory.
//   5. k_eval         persistent, warp-granular work stealing over the items
//                     of every rule: a warp filters an item's right rows
//                     (staged by bulk copies, the next item's copies in
//                     flight) against the first similarity predicate and
//                     queues the pairs that need a scan in a shared-memory
//                     ring; lanes take the next queued pair, of whatever
//                     item, as soon as theirs is decided (bit-parallel Jaro
//                     from the left string's table, exact early-fail bound),
//                     and go on with the rule's next predicate in the same
//                     lane; matches leave by warp-aggregated atomics.
//
// Semantics reproduced (reference = HyperBlocker):
//   * pairs are compared only inside a partition (data_mngr.h:150-216, the
//     bucket is part of every join key);
//   * a pair matches when some rule has all equalities true and all
//     similarities !(JW < (double)threshold) (global_func.cuh:120-167);
//   * Jaro match count m of device_func.cuh:54-132 equals the size of a
//     maximum matching between equal characters at distance <= h,
//     h = (min(len1, len2) + 1) / 2, whenever the shorter string has at most
//     256 bytes; longer pairs run the reference's own loop order (jaro_m_ref);
//   * the Jaro value is (float)(((double)(m/ls + m/ll) + 1.0) / 3.0) with IEEE
//     float quotients, and JW = fma((1 - j) * p, 0.1, j) clamped to 1 with an
//     uncapped common prefix p (device_func.cuh:210-231).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace hbx {
namespace dev {

constexpr int kMaxEq = 8;
constexpr int kMaxSim = 8;
constexpr int kWarpsPerCta = 8;
// words per symbol row of a Peq table for a left string of w 32-bit words
__host__ __device__ constexpr int row_words(int w) { return w <= 1 ? 1 : w <= 2 ? 2 : w <= 4 ? 4 : 8; }
constexpr float kDecisionMargin = 1e-4f;  // |approx JW - thr| below this -> exact path

// Count signature of a string: byte k (of 32) counts the string's symbols in
// bucket k, where the 31 most frequent symbols have a bucket each and the
// rest share the last one.  For any two strings a, b the Jaro match count
// (any matching between equal symbols) is at most
//     sum_k min(sig_a[k], sig_b[k]),
// and pooling symbols into one bucket only raises that sum, so the bound is
// exact.  A string longer than kSigMaxLen bytes, whose counts might not fit a
// byte, gets 0xff in every bucket: min() then takes the other side's count,
// which still bounds the matches from above.
constexpr uint32_t kSigBuckets = 32;
constexpr uint32_t kSigMaxLen = 255;
__host__ __device__ inline uint32_t sig_bucket(uint32_t sym) {  // sym >= 1
  return sym >= kSigBuckets ? kSigBuckets - 1 : sym - 1;
}

// Metadata of one string: where it is, how long, its first 16 symbols (0 past
// the end) and its count signature, so that one 64-byte record gives the
// length, the common prefix with another string (up to 16), the first chunk
// of a scan and an upper bound on the matches with any other string.
struct __align__(16) StrMeta {
  uint4 loc;     // {offset / 16, length, 0, 0}
  uint4 head;    // symbols 0-3, 4-7, 8-11, 12-15 (little endian)
  uint4 sig[2];  // bucket counts 0-15, 16-31, one byte each (little endian)
};

// Host form of the signature of a string of symbols.
inline void make_sig(const uint8_t* s, uint32_t len, uint4 out[2]) {
  uint32_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (len > kSigMaxLen) {
    for (int k = 0; k < 8; k++) w[k] = 0xffffffffu;
  } else {
    uint32_t c[kSigBuckets] = {0};
    for (uint32_t i = 0; i < len; i++)
      if (s[i]) c[sig_bucket(s[i])]++;
    for (uint32_t k = 0; k < kSigBuckets; k++) w[k / 4] |= c[k] << (8 * (k % 4));
  }
  out[0] = make_uint4(w[0], w[1], w[2], w[3]);
  out[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

struct Side {
  const uint32_t* bucket;
  const int32_t* eq_codes;    // [n_eq_slots][n_rows]
  const int32_t* comp_codes;  // [n_comp][n_rows]
  const uint8_t* arena;       // symbol strings, 16-byte aligned, zero padded
  const StrMeta* str_meta;    // [n_str_slots][n_rows]
  uint32_t n_rows;
};

// A rule evaluated as a member of a group (see Rule): its threshold on the
// group's first similarity column, the extra equality slots it needs beyond
// the group root's (bits of Rule::xslot), and its other similarity
// predicates in evaluation order.
constexpr uint32_t kMaxMembers = 8;
struct Member {
  float thr_first;
  uint32_t xmask;
  uint32_t n_rest;
  uint32_t rest_l[kMaxSim], rest_r[kMaxSim];
  float rest_thr[kMaxSim];
};

struct Rule {
  uint32_t n_eq, n_sim, composite, comp_index;
  uint32_t eq_slot[kMaxEq];
  uint32_t radix[kMaxEq];
  uint32_t sim_l[kMaxSim], sim_r[kMaxSim];
  float thr[kMaxSim];
  uint32_t domain;    // D: join keys
  // Left rows are grouped by (word class, key): the word class is the number
  // of 32-symbol words of the left string of the first similarity predicate
  // (1, 2, 3, 4, more).  Work items are ordered class by class, so warps that
  // run at the same time mostly run the same scan variant.
  uint32_t n_wclass;  // 1 (no split) or kWordClasses
  uint32_t wclass_slot;  // left string slot that decides the class
  uint32_t domain_l;  // n_wclass * D: left keys
  uint32_t* key_l;
  uint32_t* key_r;
  uint32_t* cnt_l;  // [domain_l]
  uint32_t* cnt_r;  // [domain]
  uint32_t* off_l;  // [domain_l]
  uint32_t* off_r;  // [domain]
  uint32_t* cur_l;
  uint32_t* cur_r;
  unsigned long long* item_off;  // [domain_l + 1]
  uint32_t* sorted_l;
  uint32_t* sorted_r;  // [n_rows + 4]: the tail pads 16-byte bulk copies
  // right-row string metadata of the first similarity predicate in sorted_r
  // order, so that a work item's metadata is one contiguous, 16-byte-aligned
  // block for a bulk copy into shared memory (null without similarities)
  StrMeta* sorted_meta_r;
  // Group evaluation.  The work items of this rule's join are evaluated for
  // n_members rules at once: member 0 is this rule, the others are rules whose
  // equality slots contain this rule's (their candidates are this join's
  // candidates whose extra slots xslot[] also hold) and whose similarity
  // predicates include this rule's first column (sim_l[0], sim_r[0]).  The
  // first column is filtered and scanned once per pair, at the smallest
  // threshold of the members still live, and decided per member from the
  // match count; members that pass go on with their other predicates, and
  // the pair matches when one member passes them all (OR across rules).
  // n_members == 0: the rule is a member of another rule's group and has no
  // work items of its own (its join still counts its pair-comparisons).
  uint32_t n_members;
  uint32_t n_xslots;
  uint32_t xslot[kMaxEq];
  float thr_min;  // smallest member threshold on the first column
  Member mem[kMaxMembers];
  // Groups with at most two extra slots: for each pattern of the extra slots
  // that hold (bit j: xslot[j]), the members still live and the smallest of
  // their first-column thresholds (fill_extras_table), so that the filter
  // looks them up instead of walking the members for every pair.
  uint32_t x_live[4];
  float x_thr[4];
};

// Host: fills Rule::x_live / x_thr from the members, with the device's
// live-threshold rule (the smallest threshold; NaN when any is NaN).
inline void fill_extras_table(Rule* g) {
  for (uint32_t eqm = 0; eqm < 4; eqm++) {
    uint32_t live = 0;
    float t = 3.0e38f;
    for (uint32_t k = 0; k < g->n_members; k++) {
      if (g->mem[k].xmask & ~eqm) continue;
      live |= 1u << k;
      const float u = g->mem[k].thr_first;
      t = (u != u || t != t) ? __builtin_nanf("") : (u < t ? u : t);
    }
    g->x_live[eqm] = live;
    g->x_thr[eqm] = t;
  }
}

// Host: a rule as the only member of its own group (the plain form, serving,
// and any rule no group takes in).
inline void make_singleton(Rule* d) {
  d->n_members = 1;
  d->n_xslots = 0;
  Member& m = d->mem[0];
  m = Member{};
  m.thr_first = d->n_sim ? d->thr[0] : 0.0f;
  m.xmask = 0;
  m.n_rest = d->n_sim > 1 ? d->n_sim - 1 : 0;
  for (uint32_t k = 1; k < d->n_sim; k++) {
    m.rest_l[k - 1] = d->sim_l[k];
    m.rest_r[k - 1] = d->sim_r[k];
    m.rest_thr[k - 1] = d->thr[k];
  }
  d->thr_min = m.thr_first;
  fill_extras_table(d);
}

constexpr uint32_t kWordClasses = 5;
constexpr uint32_t kMaxSegments = 8;
constexpr uint32_t kRingEntries = 64;
constexpr uint32_t kRingWords = 12;  // words per ring entry (three 16-byte records)

// Peq tables of the left strings, in device memory: one per (left string
// slot, left row), tab_words 32-bit words each; row `sym` (peq_s words) has
// bit j of word k set when a[32k + j] == sym.  Strings of 1 to fast_max
// symbols have a table; fast_max = 32 * peq_w <= 256.
struct PeqShape {
  uint32_t w;          // words the scans run on: 1, 2, 3, 4 or 8
  uint32_t s;          // words per symbol row: row_words(w)
  uint32_t tab_words;  // words per table (a multiple of 4: tables are 16-byte aligned)
  uint32_t fast_max;   // longest left string with a table
};

// Shape for left strings up to max_len symbols (capped at 256) over an
// alphabet of n_symbols symbols.
inline PeqShape peq_shape(uint32_t max_len, uint32_t n_symbols) {
  const uint32_t len = max_len < 1 ? 1 : (max_len > 256 ? 256 : max_len);
  const uint32_t w0 = (len + 31) / 32;
  PeqShape p;
  p.w = w0 <= 4 ? w0 : 8;
  p.s = (uint32_t)row_words((int)p.w);
  p.tab_words = (n_symbols * p.s + 3) / 4 * 4;
  p.fast_max = 32 * p.w;
  return p;
}

// Shared memory of one warp of k_eval, in 32-bit words: the ring of pairs
// waiting for a scan (kRingEntries x kRingWords), n_bufs staging buffers
// (while the warp filters one work item, the bulk copies of the next
// n_bufs - 1 fill the others) and one mbarrier per buffer.  A staging buffer holds the item's right-row
// metadata (tile_right StrMeta records), its right rows (tile_right + 8: a
// 16-byte-aligned copy starts up to 3 rows early and rounds up) and the
// metadata of its left string.  Every offset is a multiple of 4 words (16
// bytes) when tile_right is a multiple of 32.  A control block of
// kWarpCtlWords words follows.
constexpr uint32_t kMaxStageBufs = 4;
struct WarpLayout {
  uint32_t n_bufs, buf_off, buf_words, buf_rows_off, buf_lmeta_off, mbar_off, ctl_off, warp_words;
};
constexpr uint32_t kWarpCtlWords = 400;  // the warp's control block (kernels.cu: WarpCtl)

inline WarpLayout warp_layout(uint32_t tile_right, uint32_t n_bufs) {
  WarpLayout w;
  w.n_bufs = n_bufs < 1 ? 1 : (n_bufs > kMaxStageBufs ? kMaxStageBufs : n_bufs);
  const uint32_t meta_words = (uint32_t)(sizeof(StrMeta) / 4) * tile_right;
  w.buf_rows_off = meta_words;
  w.buf_lmeta_off = meta_words + (tile_right + 8 + 3) / 4 * 4;
  w.buf_words = w.buf_lmeta_off + (uint32_t)(sizeof(StrMeta) / 4);
  w.buf_off = kRingWords * kRingEntries;
  w.mbar_off = w.buf_off + w.n_bufs * w.buf_words;
  w.ctl_off = w.mbar_off + (2 * w.n_bufs + 3) / 4 * 4;
  w.warp_words = w.ctl_off + kWarpCtlWords;
  return w;
}

// The deepest staging (up to kMaxStageBufs buffers) that keeps two blocks of
// kWarpsPerCta warps on an SM within smem_cap bytes of shared memory; one
// buffer when none does (with one buffer the next item's copies start once
// the current item is filtered, and other warps cover their latency).
inline WarpLayout warp_layout_fit(uint32_t tile_right, size_t smem_cap) {
  for (uint32_t n = kMaxStageBufs; n > 1; n--) {
    const WarpLayout c = warp_layout(tile_right, n);
    if ((size_t)c.warp_words * 4 * kWarpsPerCta * 2 <= smem_cap) return c;
  }
  return warp_layout(tile_right, 1);
}

__host__ __device__ inline uint32_t word_class(uint32_t len) {
  const uint32_t w = (len + 31u) >> 5;
  return w == 0 ? 0u : (w > kWordClasses ? kWordClasses - 1 : w - 1);
}

struct Counters {
  unsigned long long out_count;
  unsigned long long comparisons;
  unsigned long long ambiguous;
  unsigned long long long_pairs;
  unsigned long long work_next;
  unsigned long long watchdog_trips;
  unsigned long long items_done;
  unsigned long long jw_word_ops;  // algorithmic work of the JW evaluations
  unsigned long long seen_overflow;  // nonzero: the duplicate set had no room (run repeats)
  unsigned long long passes;  // rule-level passes before de-duplication (plans with several rules)
  unsigned long long scans;       // pairs that reached a bit-parallel scan
  unsigned long long scan_steps;  // scan steps of 4 symbols
  unsigned long long items_total; // work items of the run (written by the join)
  unsigned long long scan_warp_steps;  // warp-level scan steps (any lane scanning)
  unsigned long long rest_scans;       // scans of predicates after a rule's or group's first
};

struct EvalParams {
  Side L, R;
  const Rule* rules;
  uint32_t n_rules;
  uint32_t n_symbols;
  const unsigned long long* rule_item_base;  // [n_rules + 1], global item space
  // Work list of the launch: every item (n_seg == 0, the batched form), or the
  // concatenation of item ranges [seg_begin[k], seg_end[k]) (the plain form:
  // one partition of one rule, one range per word class).
  uint32_t n_seg;
  unsigned long long seg_begin[kMaxSegments];
  unsigned long long seg_end[kMaxSegments];
  uint32_t tile_right;  // TR
  // shared-memory words per warp and offsets inside a warp's region (warp_layout)
  uint32_t warp_words, n_bufs, buf_off, buf_words, buf_rows_off, buf_lmeta_off, mbar_off, ctl_off;
  // Peq tables of the left strings (PeqShape): [left string slot][left row]
  const uint32_t* peq;
  uint32_t peq_w, tab_words, fast_max;
  uint32_t* out_l;
  uint32_t* out_r;
  unsigned long long capacity;
  Counters* ctr;
  unsigned long long watchdog_cycles;  // 0 = no budget
  // set of reported (left, right) keys when the plan has several rules, else null
  unsigned long long* seen;
  unsigned long long seen_mask;  // slots - 1 (a power of two minus one)
};

// Host: the shared-memory layout and Peq tables of a launch.
inline void set_layout(EvalParams* P, const WarpLayout& w, const PeqShape& s, const uint32_t* peq) {
  P->warp_words = w.warp_words;
  P->n_bufs = w.n_bufs;
  P->buf_off = w.buf_off;
  P->buf_words = w.buf_words;
  P->buf_rows_off = w.buf_rows_off;
  P->buf_lmeta_off = w.buf_lmeta_off;
  P->mbar_off = w.mbar_off;
  P->ctl_off = w.ctl_off;
  P->peq = peq;
  P->peq_w = s.w;
  P->tab_words = s.tab_words;
  P->fast_max = s.fast_max;
}

// ------------------------------------------------------------------ join
__global__ void k_keys_hist(Side S, const Rule* rules, uint32_t rule, int side);
__global__ void k_scatter(Side S, const Rule* rules, uint32_t rule, int side);
__global__ void k_scan_partial_u32(const uint32_t* in, uint32_t n, uint32_t* partial);
__global__ void k_scan_top_u32(uint32_t* partial, uint32_t nb);
__global__ void k_scan_final_u32(const uint32_t* in, uint32_t n, const uint32_t* partial,
                                 uint32_t* out);
__global__ void k_items_partial(const Rule* rules, uint32_t rule, uint32_t tile_right,
                                unsigned long long* partial, unsigned long long* comparisons);
__global__ void k_scan_top_u64(unsigned long long* partial, uint32_t nb);
__global__ void k_items_final(const Rule* rules, uint32_t rule, uint32_t tile_right,
                              const unsigned long long* partial);
__global__ void k_rule_base(const Rule* rules, uint32_t n_rules, unsigned long long* base,
                            unsigned long long* items_total);
// One launch for a run's resets: the counters and histograms to 0, the
// duplicate set (n_seen slots, may be 0) to empty.
__global__ void k_reset(Counters* ctr, uint32_t* counts, uint64_t n_counts,
                        unsigned long long* seen, uint64_t n_seen, unsigned long long* zero64,
                        uint64_t n_zero64);
// fused join (every rule's left key domain <= kFusedJoinMaxDomain); k_join_count
// and k_join_scatter run on grid (blocks, rules, 2 tables); k_join_count
// takes min(max domain, kSharedHistKeys) * 4 bytes of dynamic shared memory;
// k_join_scan runs 1024 threads per (chunk of kScanChunk keys, scan, rule):
// grid (nb = max domain / kScanChunk rounded up, 3, rules); sync holds
// rules * 3 * (nb + 1) words, zero before the launch (k_reset)
constexpr uint32_t kFusedJoinMaxDomain = 1u << 16;
constexpr uint32_t kSharedHistKeys = 8192;
__global__ void k_join_count(Side L, Side R, const Rule* rules);
__global__ void k_join_scan(const Rule* rules, uint32_t tile_right, uint32_t nb,
                            unsigned long long* sync, unsigned long long* comparisons,
                            Counters* ctr);
__global__ void k_join_scatter(Side L, Side R, const Rule* rules, uint32_t n_rules,
                               unsigned long long* rule_base, unsigned long long* items_total);
// ------------------------------------------------------------------ evaluation
// Peq tables of every left string of n_slots string slots (PeqShape).
__global__ void k_peq_build(Side L, uint32_t n_slots, PeqShape shape, uint32_t* peq);
// The evaluation kernel for masks of peq_w words (PeqShape::w): k_eval<W>
// (3 CTAs per SM, register-limited) or k_eval_wide<W> (2 CTAs per SM, more
// registers), or the same two over rule groups (k_eval_groups<W>,
// k_eval_groups_wide<W>: launches where some rule evaluates others).
using EvalKernel = void (*)(EvalParams);
EvalKernel eval_kernel(int wide, bool groups, uint32_t peq_w);
constexpr uint32_t kPeqWidths[] = {1, 2, 3, 4, 8};  // every PeqShape::w

constexpr uint32_t kScanChunk = 4096;  // elements per CTA in the scans (1024 threads x 4)

}  // namespace dev
}  // namespace hbx
