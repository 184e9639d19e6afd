// engine.cu -- device state and launch orchestration behind the C ABI.
//
// A session owns one plan's encoding of two tables on the GPU and runs the
// blocking pipeline of kernels.cu in one of two forms:
//   PLAIN    per partition, per rule: one evaluation launch, the way the
//            reference submits one blocking_kernel per partition
//            (host_producer.h:75-104, 199-203);
//   BATCHED  every rule x partition in one persistent work-stealing launch;
//            the whole run (counter reset, joins, launch) is captured once
//            into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <thread>
#include <utility>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <unistd.h>

#include "context.h"
#include "device_buffers.h"
#include "engine.h"
#include "encode.h"
#include "hbx_core.h"
#include "ingest.h"
#include "kernels.cuh"


namespace hbx {

struct RuleBufs {
  DBuf<uint32_t> key_l, key_r, off_l, off_r, sorted_l, sorted_r;
  DBuf<dev::StrMeta> sorted_meta_r;
  DBuf<unsigned long long> item_off;
  DBuf<uint32_t> part_u32;
  DBuf<unsigned long long> part_u64;
  uint32_t nb = 0;    // scan CTAs over the join key domain
  uint32_t nb_l = 0;  // scan CTAs over the left key domain (word classes x keys)
};

template <class T>
std::vector<T> flatten(const std::vector<std::vector<T>>& v, size_t n_rows) {
  std::vector<T> out;
  out.reserve(v.size() * n_rows);
  for (auto& x : v) out.insert(out.end(), x.begin(), x.end());
  return out;
}

}  // namespace hbx

struct hbx_session {
  hbx_ctx* ctx = nullptr;
  hbx::Encoded E;
  hbx::SideBufs L, R;
  std::vector<hbx::RuleBufs> rb;
  // the rules, each evaluated on its own (plain form, and every join), and
  // the same rules grouped for the batched form (group_rules)
  std::vector<hbx::dev::Rule> h_rules, h_groups;
  hbx::DBuf<hbx::dev::Rule> d_rules, d_groups;
  hbx::DBuf<unsigned long long> d_rule_base;
  hbx::DBuf<hbx::dev::Counters> d_ctr;
  hbx::dev::Counters* h_ctr = nullptr;  // page-locked copy of d_ctr (the context's), written by each run
  hbx::DBuf<uint32_t> out_l, out_r;
  hbx::DBuf<unsigned long long> seen;  // reported-pair set (plans with several rules)
  // key histograms and scatter cursors of every rule, one block: one memset
  hbx::DBuf<uint32_t> counts;
  hbx::DBuf<unsigned long long> scan_sync;  // fused join: chunk totals and tickets (k_join_scan)
  bool fused_join = false;  // every key domain small: join kernels covering all rules
  hbx::DBuf<uint32_t> bound_idx;              // per rule, n_partitions + 1 key indices
  hbx::DBuf<unsigned long long> bound_val;    // item_off at those keys
  hbx::dev::Side side_l{}, side_r{};
  uint32_t warp_words = 4;
  uint32_t tile_right = 128;
  hbx::dev::WarpLayout wl{};
  hbx::dev::PeqShape peq_shape{};
  hbx::DBuf<uint32_t> peq;  // Peq tables of the left strings [slot][row]
  int variant = 0;  // evaluation kernel: 0 = k_eval, 1 = k_eval_wide
  bool groups = false;  // some rule evaluates others in the batched form (h_groups)
  bool tuned = false;
  bool one_shot = false;  // runs once (hbx_block): no graph is captured
  // output slots to start with; a run needing more than cap_limit (the
  // caller's buffer, 0 = none) returns its count without growing and rerunning
  uint64_t out_hint = 1 << 16, cap_limit = 0;
  int blocks_per_sm = 1;
  size_t smem_bytes = 0;
  cudaGraphExec_t graph = nullptr;
  // the caller's device output (hbx_session_run), written by the kernels
  // directly; null: the session's own buffers
  uint32_t* ext_l = nullptr;
  uint32_t* ext_r = nullptr;
  uint64_t ext_cap = 0;
  const uint32_t* graph_out = nullptr;  // output the captured graph writes
  uint64_t graph_cap = 0;
  uint64_t seen_pairs = 1 << 16;  // distinct pairs the duplicate set is sized for
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;      // whole run
  cudaEvent_t ev_eval0 = nullptr, ev_eval1 = nullptr;  // join ends / evaluation ends
  hbx_stats stats{};
  ~hbx_session() {
    if (graph) cudaGraphExecDestroy(graph);
    for (cudaEvent_t e : {ev0, ev1, ev_eval0, ev_eval1})
      if (e) cudaEventDestroy(e);
  }
};

namespace hbx {

void raise_smem_limit(dev::EvalKernel kern, size_t bytes) {
  // The limit belongs to the kernel, process-wide: only ever raise it, so a
  // session needing less never lowers it under another live session.
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  cudaFuncAttributes fa;
  HBX_CUDA(cudaFuncGetAttributes(&fa, kern));
  if ((size_t)fa.maxDynamicSharedSizeBytes < bytes)
    HBX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

namespace {

constexpr int kThreads = dev::kWarpsPerCta * 32;

void launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) fail(HBX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int row_grid(uint64_t n, int n_sm) {
  uint64_t g = (n + 255) / 256;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)n_sm * 8));
}

// Tile shape and kernel variant of a session: right rows per work item
// (tile_right) and the evaluation kernel (0: 3 CTAs per SM, 1: 2 CTAs per SM
// with more registers).  Lays out each warp's shared memory
// (dev::warp_layout), uploads the rule descriptors, raises the kernel's
// shared-memory limit if needed and drops the graph.
void configure(hbx_session* S, uint32_t tile_right, int variant) {
  hbx_ctx* C = S->ctx;
  S->tile_right = std::min<uint32_t>(512, std::max<uint32_t>(32, (tile_right + 31) / 32 * 32));
  S->variant = variant ? 1 : 0;
  // two blocks per SM: the SM's shared memory less 1 KB the hardware keeps
  // per block
  const size_t smem_cap = std::min<size_t>(C->smem_optin * 2, C->smem_per_sm - 2048);
  const uint32_t cap_warp_words = (uint32_t)(C->smem_optin / 4 / dev::kWarpsPerCta) / 4 * 4;
  S->wl = dev::warp_layout_fit(S->tile_right, smem_cap);
  S->warp_words = S->wl.warp_words;
  if (S->warp_words > cap_warp_words) fail(HBX_ERR_INVALID_ARG, "tile_right too large");
  // every warp region lies inside the dynamic allocation
  S->smem_bytes = (size_t)S->warp_words * 4 * dev::kWarpsPerCta;
  HBX_CUDA(cudaMemcpyAsync(S->d_rules.p, S->h_rules.data(), S->h_rules.size() * sizeof(dev::Rule),
                           cudaMemcpyHostToDevice, C->stream));
  HBX_CUDA(cudaMemcpyAsync(S->d_groups.p, S->h_groups.data(), S->h_groups.size() * sizeof(dev::Rule),
                           cudaMemcpyHostToDevice, C->stream));
  HBX_CUDA(cudaStreamSynchronize(C->stream));
  for (bool g : {false, true}) raise_smem_limit(dev::eval_kernel(S->variant, g, S->peq_shape.w), S->smem_bytes);
  int bps = 0;
  HBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &bps, dev::eval_kernel(S->variant, S->groups, S->peq_shape.w), kThreads, S->smem_bytes));
  S->blocks_per_sm = std::max(1, bps);
  if (S->graph) {
    cudaGraphExecDestroy(S->graph);
    S->graph = nullptr;
  }
}

// Uploads the host encoding of both tables (the host ingest path).
uint64_t upload_host_encoding(hbx_session* S) {
  const Encoded& E = S->E;
  cudaStream_t st = S->ctx->stream;
  const uint32_t nL = (uint32_t)E.L.n_rows, nR = (uint32_t)E.R.n_rows;
  auto up_side = [&](const SideEnc& se, SideBufs& sb, uint32_t n) {
    sb.bucket.upload(se.bucket, st);
    sb.eq.upload(flatten(se.eq_codes, (size_t)n), st);
    sb.comp.upload(flatten(se.comp_codes, (size_t)n), st);
    sb.arena.upload(se.arena, st);
    // per string: {offset / 16, length}, first 16 symbols (0 past the end)
    std::vector<dev::StrMeta> meta;
    meta.reserve(se.str_off.size() * (size_t)n);
    for (size_t slot = 0; slot < se.str_off.size(); slot++)
      for (uint32_t i = 0; i < n; i++) {
        const uint32_t off = se.str_off[slot][i], len = se.str_len[slot][i];
        uint32_t w[4] = {0, 0, 0, 0};
        for (uint32_t k = 0; k < 16 && k < len; k++)
          w[k / 4] |= (uint32_t)se.arena[(size_t)off * 16 + k] << (8 * (k % 4));
        dev::StrMeta m;
        m.loc = make_uint4(off, len, 0, 0);
        m.head = make_uint4(w[0], w[1], w[2], w[3]);
        dev::make_sig(se.arena.data() + (size_t)off * 16, len, m.sig);
        meta.push_back(m);
      }
    sb.meta.upload(meta, st);
    HBX_CUDA(cudaStreamSynchronize(st));  // the host vector dies at scope end
  };
  up_side(E.L, S->L, nL);
  up_side(E.R, S->R, nR);
  uint64_t h2d = 0;
  for (const SideBufs* sb : {&S->L, &S->R})
    h2d += sb->bucket.n * 4 + sb->eq.n * 4 + sb->comp.n * 4 + sb->arena.n +
           sb->meta.n * sizeof(dev::StrMeta);
  return h2d;
}

std::vector<dev::Rule> group_rules(const std::vector<dev::Rule>& singles);

// Launches k with programmatic stream serialization: its blocks may start
// while the kernel before it on the stream finishes (they wait in
// dev::pdl_wait before reading its results), so a chain of short dependent
// kernels does not pay a full launch gap per kernel.
template <typename... KArgs, typename... Args>
void launch_dependent(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                      Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  HBX_CUDA(cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...));
}

// Chunks of kScanChunk keys in the largest left key domain of the session's
// rules (the fused join's scan grid).
uint32_t fused_chunks(const hbx_session* S) {
  uint32_t max_d = 1;
  for (const dev::Rule& d : S->h_rules) max_d = std::max(max_d, d.domain_l);
  return (max_d + dev::kScanChunk - 1) / dev::kScanChunk;
}

// Device state of a session whose side buffers hold the encoded tables.
void setup_session(hbx_session* S, uint64_t h2d_tables) {
  hbx_ctx* C = S->ctx;
  const Encoded& E = S->E;
  cudaStream_t st = C->stream;
  const uint32_t nL = (uint32_t)E.L.n_rows, nR = (uint32_t)E.R.n_rows;
  auto bind = [](const SideBufs& sb, dev::Side& ds, uint32_t n) {
    ds.bucket = sb.bucket.p;
    ds.eq_codes = sb.eq.p;
    ds.comp_codes = sb.comp.p;
    ds.arena = sb.arena.p;
    ds.str_meta = sb.meta.p;
    ds.n_rows = n;
  };
  bind(S->L, S->side_l, nL);
  bind(S->R, S->side_r, nR);

  // join state of every rule (independent of the tile shape)
  S->rb.clear();
  S->rb.resize(E.rules.size());
  S->h_rules.assign(E.rules.size(), dev::Rule{});
  for (size_t r = 0; r < E.rules.size(); r++) {
    const RuleEnc& re = E.rules[r];
    dev::Rule& d = S->h_rules[r];
    d.n_eq = (uint32_t)re.eq_slot.size();
    d.n_sim = (uint32_t)re.sim_slot_l.size();
    d.composite = re.composite ? 1u : 0u;
    d.comp_index = re.composite ? (uint32_t)re.comp_index : 0u;
    for (size_t e = 0; e < re.eq_slot.size(); e++) {
      d.eq_slot[e] = (uint32_t)re.eq_slot[e];
      d.radix[e] = re.radix[e];
    }
    for (size_t s = 0; s < re.sim_slot_l.size(); s++) {
      d.sim_l[s] = (uint32_t)re.sim_slot_l[s];
      d.sim_r[s] = (uint32_t)re.sim_slot_r[s];
      d.thr[s] = re.thr[s];
    }
    d.domain = (uint32_t)re.domain;
    // group left rows by the word class of the first similarity predicate's
    // string, unless that would make the left key domain too large
    const bool split = !re.sim_slot_l.empty() &&
                       re.domain * dev::kWordClasses <= (uint64_t)kMaxKeyDomain * 4;
    d.n_wclass = split ? dev::kWordClasses : 1u;
    d.wclass_slot = split ? (uint32_t)re.sim_slot_l[0] : 0u;
    d.domain_l = d.n_wclass * d.domain;
    dev::make_singleton(&d);
    RuleBufs& b = S->rb[r];
    b.key_l.alloc(nL);
    b.key_r.alloc(nR);
    b.off_l.alloc(d.domain_l);
    b.off_r.alloc(re.domain);
    b.sorted_l.alloc(nL);
    b.sorted_r.alloc((size_t)nR + 4);
    if (d.n_sim) b.sorted_meta_r.alloc(nR);
    b.item_off.alloc((size_t)d.domain_l + 1);
    b.nb = (uint32_t)((re.domain + dev::kScanChunk - 1) / dev::kScanChunk);
    b.nb_l = (uint32_t)((d.domain_l + dev::kScanChunk - 1) / dev::kScanChunk);
    b.part_u32.alloc(std::max(b.nb, b.nb_l));
    b.part_u64.alloc(b.nb_l);
    d.key_l = b.key_l.p;
    d.key_r = b.key_r.p;
    d.off_l = b.off_l.p;
    d.off_r = b.off_r.p;
    d.item_off = b.item_off.p;
    d.sorted_l = b.sorted_l.p;
    d.sorted_r = b.sorted_r.p;
    d.sorted_meta_r = d.n_sim ? b.sorted_meta_r.p : nullptr;
  }
  // histograms and cursors: [cnt_l | cur_l | cnt_r | cur_r] per rule
  {
    size_t total = 0;
    for (const dev::Rule& d : S->h_rules) total += 2ull * d.domain_l + 2ull * d.domain;
    S->counts.alloc(std::max<size_t>(total, 1));
    size_t pos = 0;
    S->fused_join = true;
    for (dev::Rule& d : S->h_rules) {
      d.cnt_l = S->counts.p + pos;
      d.cur_l = d.cnt_l + d.domain_l;
      d.cnt_r = d.cur_l + d.domain_l;
      d.cur_r = d.cnt_r + d.domain;
      pos += 2ull * d.domain_l + 2ull * d.domain;
      if (d.domain_l > dev::kFusedJoinMaxDomain) S->fused_join = false;
    }
    if (S->fused_join) S->scan_sync.alloc(E.rules.size() * 3 * (fused_chunks(S) + 1));
  }
  S->h_groups = group_rules(S->h_rules);
  S->groups = false;
  for (const dev::Rule& g : S->h_groups)
    if (g.n_members > 1) S->groups = true;
  S->d_rules.alloc(E.rules.size());
  S->d_groups.alloc(E.rules.size());
  S->d_rule_base.alloc(E.rules.size() + 1);
  S->d_ctr.alloc(1);
  // one page-locked counter block per context: its sessions run one at a time
  if (!C->h_ctr) HBX_CUDA(cudaHostAlloc(&C->h_ctr, sizeof(dev::Counters), cudaHostAllocPortable));
  S->h_ctr = static_cast<dev::Counters*>(C->h_ctr);
  // Peq tables of every left string slot, shaped for the longest left
  // string any similarity predicate reads (the shape picks the evaluation
  // kernel, so it comes before the configuration)
  {
    uint32_t mx = 1;
    for (const RuleEnc& re : E.rules)
      for (int sl : re.sim_slot_l) mx = std::max(mx, E.L.str_maxlen[(size_t)sl]);
    S->peq_shape = dev::peq_shape(mx, E.n_symbols);
  }
  const uint32_t tile = C->opts.tile_right > 0 ? (uint32_t)C->opts.tile_right : 128u;
  const int variant = C->opts.eval_variant > 0 ? C->opts.eval_variant - 1 : 1;
  configure(S, tile, variant);
  {
    const uint32_t n_slots = (uint32_t)E.L.str_maxlen.size();
    const size_t words = (size_t)n_slots * nL * S->peq_shape.tab_words;
    S->peq.alloc(std::max<size_t>(words, 4));
    if (words) {
      const uint64_t warps = (uint64_t)n_slots * nL;
      const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((warps + 7) / 8, (uint64_t)C->n_sm * 16));
      dev::k_peq_build<<<grid, 256, 0, st>>>(S->side_l, n_slots, S->peq_shape, S->peq.p);
      launch_check("k_peq_build");
    }
  }

  // partition boundaries of every rule's left key space, per word class
  // (plain form): entry (rule, class, p) = first left key of partition p
  std::vector<uint32_t> idx;
  for (size_t r = 0; r < E.rules.size(); r++)
    for (uint32_t c = 0; c < dev::kWordClasses; c++)
      for (uint64_t p = 0; p <= E.n_partitions; p++) {
        const uint32_t cc = std::min<uint32_t>(c, S->h_rules[r].n_wclass - 1);
        idx.push_back(cc * S->h_rules[r].domain + (uint32_t)E.rules[r].part_key_begin[p]);
      }
  S->bound_idx.upload(idx, st);
  S->bound_val.alloc(idx.size());
  // output slots (and the duplicate set, twice as many) for the caller's
  // capacity, but never more than the partitions can hold: a generous caller
  // buffer does not size device buffers by itself
  const uint64_t cap0 =
      std::max<uint64_t>(1 << 16, std::min<uint64_t>(S->out_hint, E.pairs_covered + 1));
  S->out_l.alloc(cap0);
  S->out_r.alloc(cap0);
  if (E.rules.size() > 1) {
    uint64_t slots = 1 << 17;
    while (slots < 2 * cap0) slots *= 2;  // load factor at most one half
    S->seen.alloc(slots);
  }
  HBX_CUDA(cudaEventCreate(&S->ev0));
  HBX_CUDA(cudaEventCreate(&S->ev1));
  HBX_CUDA(cudaEventCreate(&S->ev_eval0));
  HBX_CUDA(cudaEventCreate(&S->ev_eval1));
  uint64_t h2d = h2d_tables;
  h2d += S->d_rules.n * sizeof(dev::Rule) + S->bound_idx.n * 4;
  S->stats.h2d_bytes = h2d;
  HBX_CUDA(cudaStreamSynchronize(st));
  S->stats.pairs_covered = E.pairs_covered;
  S->stats.n_partitions_used = E.n_partitions_used;
}

// Groups of the batched form (dev::Rule, "Group evaluation"), from the
// rules in plan order, each a singleton: a rule joins the first group whose
// root's equality slots it contains (its candidates are a subset of the
// root's) and whose first similarity column it also tests, up to
// dev::kMaxMembers members and dev::kMaxEq distinct extra slots.  Rules are
// taken fewest equalities first, so roots are the coarsest joins.  A new root
// puts first, among its own similarity columns, the one that the most
// remaining rules could share.  Rules without similarity predicates stay on
// their own.  The result keeps every rule at its index; members get
// n_members = 0.
std::vector<dev::Rule> group_rules(const std::vector<dev::Rule>& singles) {
  std::vector<dev::Rule> g = singles;
  const size_t n = g.size();
  auto eqset = [&](size_t r) {
    std::vector<uint32_t> v(singles[r].eq_slot, singles[r].eq_slot + singles[r].n_eq);
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    return v;
  };
  auto contains = [](const std::vector<uint32_t>& big, const std::vector<uint32_t>& small) {
    return std::includes(big.begin(), big.end(), small.begin(), small.end());
  };
  auto has_col = [&](size_t r, uint32_t sl, uint32_t sr) {
    for (uint32_t k = 0; k < singles[r].n_sim; k++)
      if (singles[r].sim_l[k] == sl && singles[r].sim_r[k] == sr) return true;
    return false;
  };
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return singles[a].n_eq < singles[b].n_eq; });
  std::vector<int> root_of(n, -1);
  std::vector<size_t> roots;
  for (size_t oi = 0; oi < n; oi++) {
    const size_t r = order[oi];
    if (singles[r].n_sim == 0) continue;
    const std::vector<uint32_t> er = eqset(r);
    bool placed = false;
    for (size_t root : roots) {
      dev::Rule& G = g[root];
      if (G.n_members >= dev::kMaxMembers) continue;
      if (!contains(er, eqset(root)) || !has_col(r, G.sim_l[0], G.sim_r[0])) continue;
      // the extra slots this member needs, added to the group's list
      std::vector<uint32_t> er_root = eqset(root), extra;
      std::set_difference(er.begin(), er.end(), er_root.begin(), er_root.end(),
                          std::back_inserter(extra));
      uint32_t nx = G.n_xslots, xmask = 0;
      uint32_t xs[dev::kMaxEq];
      std::copy(G.xslot, G.xslot + G.n_xslots, xs);
      bool fits = true;
      for (uint32_t slot : extra) {
        uint32_t j = 0;
        while (j < nx && xs[j] != slot) j++;
        if (j == nx) {
          if (nx == (uint32_t)dev::kMaxEq) {
            fits = false;
            break;
          }
          xs[nx++] = slot;
        }
        xmask |= 1u << j;
      }
      if (!fits) continue;
      G.n_xslots = nx;
      std::copy(xs, xs + nx, G.xslot);
      dev::Member& M = G.mem[G.n_members++];
      M = dev::Member{};
      M.xmask = xmask;
      M.thr_first = -1e30f;
      const dev::Rule& R = singles[r];
      for (uint32_t k = 0; k < R.n_sim; k++) {
        if (R.sim_l[k] == G.sim_l[0] && R.sim_r[k] == G.sim_r[0]) {
          M.thr_first = std::max(M.thr_first, R.thr[k]);  // both must hold: the larger decides
        } else {
          M.rest_l[M.n_rest] = R.sim_l[k];
          M.rest_r[M.n_rest] = R.sim_r[k];
          M.rest_thr[M.n_rest] = R.thr[k];
          M.n_rest++;
        }
      }
      G.thr_min = std::min(G.thr_min, M.thr_first);
      g[r].n_members = 0;
      root_of[r] = (int)root;
      placed = true;
      break;
    }
    if (placed) continue;
    // a new root: its first column is the one most later rules could share
    dev::Rule& G = g[r];
    uint32_t best_k = 0, best_n = 0;
    for (uint32_t k = 0; k < G.n_sim; k++) {
      uint32_t cnt = 0;
      for (size_t oj = oi + 1; oj < n; oj++) {
        const size_t q = order[oj];
        if (singles[q].n_sim && contains(eqset(q), er) && has_col(q, G.sim_l[k], G.sim_r[k])) cnt++;
      }
      if (cnt > best_n) {
        best_n = cnt;
        best_k = k;
      }
    }
    if (best_k) {  // move that predicate to the front, the others keep their order
      const uint32_t sl = G.sim_l[best_k], sr = G.sim_r[best_k];
      const float t = G.thr[best_k];
      for (uint32_t k = best_k; k > 0; k--) {
        G.sim_l[k] = G.sim_l[k - 1];
        G.sim_r[k] = G.sim_r[k - 1];
        G.thr[k] = G.thr[k - 1];
      }
      G.sim_l[0] = sl;
      G.sim_r[0] = sr;
      G.thr[0] = t;
      if (G.n_wclass > 1) G.wclass_slot = sl;
    }
    dev::make_singleton(&G);
    roots.push_back(r);
  }
  for (dev::Rule& G : g)
    if (G.n_members) dev::fill_extras_table(&G);
  return g;
}

__global__ void k_gather_bounds(const dev::Rule* rules, uint32_t n_rules, uint32_t per_rule,
                                const uint32_t* idx, unsigned long long* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_rules * per_rule) return;
  out[i] = rules[i / per_rule].item_off[idx[i]];
}

// Enqueues counter reset + the joins of every rule, with the rule array
// `rules` (d_rules or d_groups: the same join state; in d_groups a group's
// first column may lead another predicate, and members have no items).
// Returns launches.
uint32_t enqueue_join(hbx_session* S, cudaStream_t st, const dev::Rule* rules) {
  uint32_t launches = 1;  // k_reset
  const uint64_t n_sync = S->fused_join ? S->scan_sync.n : 0;
  {  // counters, histograms, the duplicate set and the join scan's tickets, one launch
    const uint64_t n_seen = S->seen.p ? S->seen.n : 0;
    const uint64_t n = std::max<uint64_t>(std::max<uint64_t>(S->counts.n, n_seen), std::max<uint64_t>(n_sync, 32));
    dev::k_reset<<<row_grid(n, S->ctx->n_sm), 256, 0, st>>>(S->d_ctr.p, S->counts.p, S->counts.n,
                                                            S->seen.p, n_seen, S->scan_sync.p,
                                                            n_sync);
  }
  const uint32_t nL = S->side_l.n_rows, nR = S->side_r.n_rows;
  const int n_sm = S->ctx->n_sm;
  const uint32_t n_rules = (uint32_t)S->rb.size();
  if (S->fused_join) {
    uint32_t max_d = 1;
    for (const dev::Rule& d : S->h_rules) max_d = std::max(max_d, d.domain_l);
    const size_t smem = std::min<uint32_t>(max_d, dev::kSharedHistKeys) * sizeof(uint32_t);
    // rows per block row: each (rule, table) pair gets its own blocks
    const dim3 grid(row_grid(std::max(nL, nR), n_sm), n_rules, 2);
    const uint32_t nb = fused_chunks(S);
    unsigned long long* comparisons = &S->d_ctr.p->comparisons;
    launch_dependent(dev::k_join_count, grid, dim3(256), smem, st, S->side_l, S->side_r, rules);
    launch_dependent(dev::k_join_scan, dim3(nb, 3, n_rules), dim3(1024), 0, st, rules,
                     S->tile_right, nb, S->scan_sync.p, comparisons, S->d_ctr.p);
    launch_dependent(dev::k_join_scatter, grid, dim3(256), 0, st, S->side_l, S->side_r, rules,
                     n_rules, S->d_rule_base.p, &S->d_ctr.p->items_total);
    launch_check("join kernels");
    return launches + 3;
  }
  for (size_t r = 0; r < S->rb.size(); r++) {
    RuleBufs& b = S->rb[r];
    const uint32_t D = S->h_rules[r].domain;
    const uint32_t DL = S->h_rules[r].domain_l;
    if (nL) dev::k_keys_hist<<<row_grid(nL, n_sm), 256, 0, st>>>(S->side_l, rules, (uint32_t)r, 0);
    if (nR) dev::k_keys_hist<<<row_grid(nR, n_sm), 256, 0, st>>>(S->side_r, rules, (uint32_t)r, 1);
    dev::k_scan_partial_u32<<<b.nb_l, 1024, 0, st>>>(S->h_rules[r].cnt_l, DL, b.part_u32.p);
    dev::k_scan_top_u32<<<1, 1024, 0, st>>>(b.part_u32.p, b.nb_l);
    dev::k_scan_final_u32<<<b.nb_l, 1024, 0, st>>>(S->h_rules[r].cnt_l, DL, b.part_u32.p, b.off_l.p);
    dev::k_scan_partial_u32<<<b.nb, 1024, 0, st>>>(S->h_rules[r].cnt_r, D, b.part_u32.p);
    dev::k_scan_top_u32<<<1, 1024, 0, st>>>(b.part_u32.p, b.nb);
    dev::k_scan_final_u32<<<b.nb, 1024, 0, st>>>(S->h_rules[r].cnt_r, D, b.part_u32.p, b.off_r.p);
    dev::k_items_partial<<<b.nb_l, 1024, 0, st>>>(rules, (uint32_t)r, S->tile_right,
                                                  b.part_u64.p, &S->d_ctr.p->comparisons);
    dev::k_scan_top_u64<<<1, 1024, 0, st>>>(b.part_u64.p, b.nb_l);
    dev::k_items_final<<<b.nb_l, 1024, 0, st>>>(rules, (uint32_t)r, S->tile_right,
                                                b.part_u64.p);
    if (nL) dev::k_scatter<<<row_grid(nL, n_sm), 256, 0, st>>>(S->side_l, rules, (uint32_t)r, 0);
    if (nR) dev::k_scatter<<<row_grid(nR, n_sm), 256, 0, st>>>(S->side_r, rules, (uint32_t)r, 1);
    launches += 9 + (nL ? 2 : 0) + (nR ? 2 : 0);
  }
  dev::k_rule_base<<<1, 32, 0, st>>>(rules, n_rules, S->d_rule_base.p,
                                     &S->d_ctr.p->items_total);
  launches++;
  launch_check("join kernels");
  return launches;
}

// Output slots of the next run: the caller's buffer or the session's own.
uint64_t out_cap(const hbx_session* S) { return S->ext_l ? S->ext_cap : S->out_l.n; }

void drop_graph(hbx_session* S) {
  if (S->graph) {
    cudaGraphExecDestroy(S->graph);
    S->graph = nullptr;
  }
}

// The duplicate set holds at least 2 x `pairs` slots (load at most one half).
void fit_seen(hbx_session* S, uint64_t pairs) {
  if (!S->seen.p) return;
  uint64_t slots = S->seen.n;
  while (slots < 2 * pairs) slots *= 2;
  if (slots != S->seen.n) {
    S->seen.alloc(slots);
    drop_graph(S);
  }
}

dev::EvalParams eval_params(hbx_session* S, const dev::Rule* rules) {
  dev::EvalParams P{};
  P.L = S->side_l;
  P.R = S->side_r;
  P.rules = rules;
  P.n_rules = (uint32_t)S->rb.size();
  P.n_symbols = S->E.n_symbols;
  P.rule_item_base = S->d_rule_base.p;
  P.tile_right = S->tile_right;
  dev::set_layout(&P, S->wl, S->peq_shape, S->peq.p);
  P.out_l = S->ext_l ? S->ext_l : S->out_l.p;
  P.out_r = S->ext_l ? S->ext_r : S->out_r.p;
  P.capacity = out_cap(S);
  P.ctr = S->d_ctr.p;
  P.watchdog_cycles = S->ctx->opts.watchdog_cycles;
  P.seen = S->seen.p;
  P.seen_mask = S->seen.p ? S->seen.n - 1 : 0;
  return P;
}

void queue_counters(hbx_session* S, cudaStream_t st);

uint32_t enqueue_batched(hbx_session* S, cudaStream_t st) {
  // Inside stream capture a plain record would only be a capture dependency
  // marker; the external flag makes it an event-record node that can be
  // timed (the flag is refused outside capture).  The run's events (start,
  // join done, evaluation done, end) are all recorded by the run itself.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  HBX_CUDA(cudaStreamIsCapturing(st, &cap));
  const unsigned rec_flags =
      cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
  HBX_CUDA(cudaEventRecordWithFlags(S->ev0, st, rec_flags));
  // the batched form evaluates rule groups: one join's items for several rules
  uint32_t launches = enqueue_join(S, st, S->d_groups.p);
  dev::EvalParams P = eval_params(S, S->d_groups.p);
  P.n_seg = 0;  // every work item of every group
  const int grid = S->ctx->n_sm * S->blocks_per_sm;
  HBX_CUDA(cudaEventRecordWithFlags(S->ev_eval0, st, rec_flags));
  dev::eval_kernel(S->variant, S->groups, S->peq_shape.w)<<<grid, kThreads, S->smem_bytes, st>>>(P);
  launch_check("k_eval");
  HBX_CUDA(cudaEventRecordWithFlags(S->ev_eval1, st, rec_flags));
  // the counters travel back inside the run (graph nodes when captured)
  queue_counters(S, st);
  HBX_CUDA(cudaEventRecordWithFlags(S->ev1, st, rec_flags));
  return launches + 1;
}

void grow_output(hbx_session* S, uint64_t need) {
  uint64_t cap = S->out_l.n;
  while (cap < need) cap *= 2;
  S->out_l.alloc(cap);
  S->out_r.alloc(cap);
  if (S->seen.p) {
    uint64_t slots = S->seen.n;
    while (slots < 2 * cap) slots *= 2;  // load factor stays at or below one half
    if (slots != S->seen.n) S->seen.alloc(slots);
  }
  if (S->graph) {
    cudaGraphExecDestroy(S->graph);
    S->graph = nullptr;
  }
}

// Output pairs a repeated run must have room for: the distinct pairs of a
// run whose output overflowed, or (duplicate set full) its pass count.
uint64_t needed_capacity(const hbx_session* S, const dev::Counters& c) {
  uint64_t need = c.out_count;
  if (c.seen_overflow) need = std::max<uint64_t>(need, c.passes);
  return std::max<uint64_t>(need, S->out_l.n + 1);
}

// Queues the copy of the counters (with the run's work-item total) into the
// context's page-locked block (a graph node when captured).
void queue_counters(hbx_session* S, cudaStream_t st) {
  HBX_CUDA(cudaMemcpyAsync(S->h_ctr, S->d_ctr.p, sizeof(dev::Counters), cudaMemcpyDeviceToHost, st));
}

unsigned long long items_total(const hbx_session* S) { return S->h_ctr->items_total; }

dev::Counters read_counters(hbx_session* S, cudaStream_t st) {
  queue_counters(S, st);
  HBX_CUDA(cudaStreamSynchronize(st));
  return *S->h_ctr;
}

// One run into the session's own output buffers; returns the counters.
dev::Counters run_once(hbx_session* S, hbx_mode mode, cudaStream_t st, uint32_t* launches) {
  const bool use_graph = S->ctx->opts.use_graph != 0 && !S->one_shot;
  if (mode == HBX_MODE_BATCHED) {
    if (use_graph) {
      const uint32_t* out = S->ext_l ? S->ext_l : S->out_l.p;
      if (S->graph && (S->graph_out != out || S->graph_cap != out_cap(S))) drop_graph(S);
      if (!S->graph) {
        S->graph_out = out;
        S->graph_cap = out_cap(S);
        cudaGraph_t g = nullptr;
        HBX_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        uint32_t n = 0;
        try {
          n = enqueue_batched(S, st);
        } catch (...) {
          cudaStreamEndCapture(st, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        HBX_CUDA(cudaStreamEndCapture(st, &g));
        cudaError_t e = cudaGraphInstantiate(&S->graph, g, 0);
        cudaGraphDestroy(g);
        HBX_CUDA(e);
        S->stats.n_launches = n;
      }
      HBX_CUDA(cudaGraphLaunch(S->graph, st));
      *launches = S->stats.n_launches;
    } else {
      *launches = enqueue_batched(S, st);
    }
    HBX_CUDA(cudaStreamSynchronize(st));
    return *S->h_ctr;
  }
  // PLAIN: join, then one launch per (partition, rule)
  HBX_CUDA(cudaEventRecord(S->ev0, st));
  uint32_t n = enqueue_join(S, st, S->d_rules.p);
  const uint32_t n_rules = (uint32_t)S->rb.size();
  const uint32_t per_class = (uint32_t)S->E.n_partitions + 1;
  const uint32_t per_rule = per_class * dev::kWordClasses;
  const uint32_t total = n_rules * per_rule;
  k_gather_bounds<<<(total + 255) / 256, 256, 0, st>>>(S->d_rules.p, n_rules, per_rule,
                                                       S->bound_idx.p, S->bound_val.p);
  n++;
  launch_check("k_gather_bounds");
  std::vector<unsigned long long> bounds(total), base(n_rules + 1);
  HBX_CUDA(cudaMemcpyAsync(bounds.data(), S->bound_val.p, total * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, st));
  HBX_CUDA(cudaMemcpyAsync(base.data(), S->d_rule_base.p, (n_rules + 1) * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, st));
  HBX_CUDA(cudaStreamSynchronize(st));
  dev::EvalParams P = eval_params(S, S->d_rules.p);
  const int max_grid = S->ctx->n_sm * S->blocks_per_sm;
  HBX_CUDA(cudaEventRecord(S->ev_eval0, st));
  for (uint64_t p = 0; p < S->E.n_partitions; p++) {
    for (uint32_t r = 0; r < n_rules; r++) {
      // the partition's items: one range per word class
      P.n_seg = 0;
      unsigned long long n_items = 0;
      for (uint32_t c = 0; c < S->h_rules[r].n_wclass; c++) {
        const size_t k = (size_t)r * per_rule + (size_t)c * per_class + p;
        const unsigned long long b0 = base[r] + bounds[k], b1 = base[r] + bounds[k + 1];
        if (b1 <= b0) continue;
        P.seg_begin[P.n_seg] = b0;
        P.seg_end[P.n_seg] = b1;
        P.n_seg++;
        n_items += b1 - b0;
      }
      if (!n_items) continue;
      HBX_CUDA(cudaMemsetAsync(&S->d_ctr.p->work_next, 0, sizeof(unsigned long long), st));
      const unsigned long long ctas = (n_items + dev::kWarpsPerCta - 1) / dev::kWarpsPerCta;
      const int grid = (int)std::min<unsigned long long>(ctas, (unsigned long long)max_grid);
      dev::eval_kernel(S->variant, false, S->peq_shape.w)<<<grid, kThreads, S->smem_bytes, st>>>(P);
      n++;
      launch_check("k_eval (plain)");
    }
  }
  HBX_CUDA(cudaEventRecord(S->ev_eval1, st));
  *launches = n;
  S->stats.n_launches = n;
  queue_counters(S, st);
  HBX_CUDA(cudaEventRecord(S->ev1, st));
  HBX_CUDA(cudaStreamSynchronize(st));
  return *S->h_ctr;
}

// ---- tile-shape autotuner ---------------------------------------------------
// The first batched run of a session whose tile shape or kernel variant is
// left to the engine (hbx_opts.tile_right == 0 or eval_variant == 0) times
// each candidate (right rows per work item x evaluation kernel) on the
// session's own data and keeps the fastest.  Choices are cached in a JSON
// file (HBX_AUTOTUNE_CACHE, default $HOME/.cache/hbx_autotune.json) under a
// signature of the device and the workload's shape, so later sessions of the
// same shape skip the search.

std::string autotune_path() {
  if (const char* p = std::getenv("HBX_AUTOTUNE_CACHE")) return p;
  const char* home = std::getenv("HOME");
  return std::string(home ? home : "/tmp") + "/.cache/hbx_autotune.json";
}

std::string workload_signature(const hbx_session* S) {
  std::string sig = S->ctx->device_name;
  sig += "|k4";  // evaluation kernel generation: entries of earlier kernels do not apply
  auto bucket = [](uint64_t n) {  // power-of-two bucket
    uint32_t b = 0;
    while ((1ull << b) < n) b++;
    return b;
  };
  sig += "|L" + std::to_string(bucket(S->E.L.n_rows)) + "|R" + std::to_string(bucket(S->E.R.n_rows)) +
         "|P" + std::to_string(bucket(S->E.n_partitions)) + "|S" + std::to_string(S->E.n_symbols);
  for (const RuleEnc& re : S->E.rules) {
    sig += "|e" + std::to_string(re.eq_slot.size()) + "s" + std::to_string(re.sim_slot_l.size());
    if (!re.sim_slot_l.empty())
      sig += "w" + std::to_string((S->E.L.str_maxlen[(size_t)re.sim_slot_l[0]] + 31) / 32) + "d" +
             std::to_string(bucket(re.domain));
  }
  for (auto& ch : sig)
    if (ch == '"' || ch == '\\') ch = '_';
  return sig;
}

// The cache file holds one entry per line:  "<signature>": [tile_right, variant, ms],
std::map<std::string, std::string> read_autotune_file(const std::string& path) {
  std::map<std::string, std::string> m;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    const size_t a = line.find('"'), b = line.find("\": [");
    const size_t e = line.find(']', b == std::string::npos ? 0 : b);
    if (a == std::string::npos || b == std::string::npos || e == std::string::npos) continue;
    m[line.substr(a + 1, b - a - 1)] = line.substr(b + 4, e - b - 4);
  }
  return m;
}

// The file is read once per process and path; later lookups use the copy in
// memory, which every new choice updates before it is written back.
std::mutex g_tune_mu;
std::map<std::string, std::map<std::string, std::string>> g_tune_mem;  // path -> entries

std::map<std::string, std::string> load_autotune_cache(const std::string& path) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune_mem.find(path);
  if (it == g_tune_mem.end()) it = g_tune_mem.emplace(path, read_autotune_file(path)).first;
  return it->second;
}

void write_autotune_file(const std::string& path, const std::map<std::string, std::string>& m);

void save_autotune_cache(const std::string& path, const std::map<std::string, std::string>& m) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  std::map<std::string, std::string>& mem = g_tune_mem[path];
  for (auto& kv : m) mem[kv.first] = kv.second;
  write_autotune_file(path, mem);
}

void write_autotune_file(const std::string& path, const std::map<std::string, std::string>& m) {
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) {
    std::error_code ec;
    std::filesystem::create_directories(path.substr(0, slash), ec);
  }
  const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
  {
    std::ofstream f(tmp);
    if (!f) return;  // a cache that cannot be written is not an error
    f << "{\n";
    size_t k = 0;
    for (auto& kv : m) f << "  \"" << kv.first << "\": [" << kv.second << "]" << (++k < m.size() ? "," : "") << "\n";
    f << "}\n";
  }
  std::rename(tmp.c_str(), path.c_str());
}

// One batched run without a graph; returns its device time in ms.
// flush: when non-null, this buffer (larger than L2) is overwritten first,
// outside the timed region, so every candidate starts from a cold L2 the way a
// one-shot run or a run over inputs larger than L2 does.
float timed_batched_run(hbx_session* S, cudaStream_t st, DBuf<uint8_t>* flush = nullptr) {
  if (flush && flush->p) HBX_CUDA(cudaMemsetAsync(flush->p, 0, flush->n, st));
  enqueue_batched(S, st);  // records ev0 and ev1 itself
  HBX_CUDA(cudaEventSynchronize(S->ev1));
  float ms = 0;
  HBX_CUDA(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
  return ms;
}

void autotune(hbx_session* S, cudaStream_t st) {
  S->tuned = true;
  const hbx_opts& o = S->ctx->opts;
  if (o.tile_right > 0 && o.eval_variant > 0) return;
  const std::string path = autotune_path(), sig = workload_signature(S);
  std::map<std::string, std::string> cache = load_autotune_cache(path);
  auto hit = cache.find(sig);
  if (hit != cache.end()) {
    unsigned tr = 0;
    int v = 0;
    float ms = 0;
    if (std::sscanf(hit->second.c_str(), "%u, %d, %f", &tr, &v, &ms) == 3 && tr >= 32) {
      const uint32_t want_tr = o.tile_right > 0 ? (uint32_t)o.tile_right : tr;
      const int want_v = o.eval_variant > 0 ? o.eval_variant - 1 : v;
      if (want_tr != S->tile_right || (want_v ? 1 : 0) != S->variant) configure(S, want_tr, want_v);
      return;
    }
  }
  std::vector<uint32_t> tiles = {32, 64, 96, 128};
  std::vector<int> variants = {0, 1};
  if (o.tile_right > 0) tiles = {(uint32_t)o.tile_right};
  if (o.eval_variant > 0) variants = {o.eval_variant - 1};
  std::vector<std::pair<uint32_t, int>> cand;
  for (uint32_t tr : tiles)
    for (int v : variants) cand.emplace_back(tr, v);
  // interleaved rounds, best time per candidate: drifts of clock or cache
  // state hit every candidate alike; one round when runs are long
  std::vector<float> best_ms(cand.size(), 1e30f);
  DBuf<uint8_t> flush;
  {
    int l2 = 0;
    HBX_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, S->ctx->device));
    PoolScope scope(S->ctx->pool, st);
    flush.alloc((size_t)std::max(l2, 1 << 20) * 2);
  }
  for (int round = 0; round < 3; round++) {
    for (size_t k = 0; k < cand.size(); k++) {
      configure(S, cand[k].first, cand[k].second);
      float ms = timed_batched_run(S, st, &flush);
      const dev::Counters c = read_counters(S, st);
      if (S->ext_l ? (bool)c.seen_overflow : (c.out_count > S->out_l.n || c.seen_overflow)) {
        if (S->ext_l) {
          S->seen_pairs = std::max<uint64_t>(2 * S->seen_pairs, c.passes);
          fit_seen(S, S->seen_pairs);
        } else {
          grow_output(S, needed_capacity(S, c));
        }
        ms = timed_batched_run(S, st, &flush);
      }
      best_ms[k] = std::min(best_ms[k], ms);
    }
    if (*std::min_element(best_ms.begin(), best_ms.end()) >= 50.0f) break;
  }
  size_t bk = 0;
  for (size_t k = 1; k < cand.size(); k++)
    if (best_ms[k] < best_ms[bk]) bk = k;
  const uint32_t best_tr = cand[bk].first;
  const int best_v = cand[bk].second;
  const float best = best_ms[bk];
  configure(S, best_tr, best_v);
  char buf[64];
  std::snprintf(buf, sizeof buf, "%u, %d, %.4f", best_tr, best_v, best);
  cache[sig] = buf;
  save_autotune_cache(path, cache);
}

}  // namespace

// Encodes the tables (on the device unless hbx_opts.ingest asks for the host
// encoder, or only the host encoder is exact for the input) and builds the
// session's device state.  The similarity predicates of each rule run in the
// order the planner measures for this pair of tables (hbx_opts.pred_order),
// memoised on the plan.
void create_session(hbx_session* S, const hbx_plan* plan, const hbx_table* left,
                    const hbx_table* right, uint64_t n_partitions, int64_t prefix_idx) {
  hbx_ctx* C = S->ctx;
  const auto t0 = std::chrono::steady_clock::now();
  PoolScope scope(C->pool, C->stream);
  Plan ordered;
  const Plan* use = &plan->p;
  if (C->opts.pred_order == 0) {
    hbx_plan* mp = const_cast<hbx_plan*>(plan);
    const std::pair<uint64_t, uint64_t> key(left->uid, right->uid);
    std::vector<CompiledRule> order;
    bool have = false;
    {
      std::lock_guard<std::mutex> lock(mp->order_mu);
      auto it = mp->order_cache.find(key);
      if (it != mp->order_cache.end()) {
        order = it->second;
        have = true;
      }
    }
    ordered = plan->p;
    if (have) {
      ordered.compiled = std::move(order);
    } else {
      order_predicates(&ordered, left->t, right->t);
      std::lock_guard<std::mutex> lock(mp->order_mu);
      mp->order_cache[key] = ordered.compiled;
    }
    use = &ordered;
  }
  S->E = encode_schema(*use, left->t, right->t, n_partitions, prefix_idx);
  bool on_device = false;
  uint64_t h2d = 0;
  std::string why;
  if (C->opts.ingest == 0)
    on_device = device_encode(left, right, &S->E, &S->L, &S->R, C->n_sm, C->stream, &h2d, &why);
  if (!on_device) {
    encode_rows(left->t, right->t, &S->E);
    finish_rules(&S->E, true);
    h2d = upload_host_encoding(S);
  }
  setup_session(S, h2d);
  S->stats.ingest_on_device = on_device ? 1u : 0u;
  S->stats.ms_create =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void session_run(hbx_session* S, hbx_mode mode, cudaStream_t st) {
  HBX_CUDA(cudaSetDevice(S->ctx->device));
  if (!S->tuned && mode == HBX_MODE_BATCHED) autotune(S, st);

  uint32_t launches = 0;
  fit_seen(S, S->seen_pairs);
  for (int attempt = 0; attempt < 8; attempt++) {
    dev::Counters c = run_once(S, mode, st, &launches);  // returns with the stream idle
    float ms = 0, ms_join = 0, ms_eval = 0;
    HBX_CUDA(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
    HBX_CUDA(cudaEventElapsedTime(&ms_join, S->ev0, S->ev_eval0));
    HBX_CUDA(cudaEventElapsedTime(&ms_eval, S->ev_eval0, S->ev_eval1));
    S->stats.ms_last_run = ms;
    S->stats.ms_join = ms_join;
    S->stats.ms_eval = ms_eval;
    S->stats.jw_word_ops = c.jw_word_ops;
    S->stats.pair_comparisons = c.comparisons;
    S->stats.n_matches = c.out_count;
    S->stats.fma_ambiguous = c.ambiguous;
    S->stats.long_string_pairs = c.long_pairs;
    S->stats.n_launches = launches;
    S->stats.pairs_scanned = c.scans;
    S->stats.scan_steps = c.scan_steps;
    // a scan step is 4 characters over peq_shape.w 32-bit mask words, 3
    // operations per 32-bit word per character (6 per 64-bit word)
    S->stats.scan_word_ops = c.scan_steps * 4ull * 3ull * S->peq_shape.w;
    S->stats.scan_words = S->peq_shape.w;
    S->stats.scan_warp_steps = c.scan_warp_steps;
    S->stats.rest_scans = c.rest_scans;
    S->stats.tile_right = S->tile_right;
    S->stats.n_windows = 1;
    S->stats.eval_variant = (uint32_t)S->variant + 1;
    const unsigned long long total_items = items_total(S);  // copied with the counters
    S->stats.n_tiles = total_items;
    if (c.watchdog_trips) fail(HBX_ERR_WATCHDOG, "evaluation stopped by the watchdog budget");
    if (c.items_done != total_items)
      fail(HBX_ERR_CUDA, "evaluation finished " + std::to_string(c.items_done) + " of " +
                             std::to_string(total_items) + " work items");
    if (c.seen_overflow == 0)
      S->seen_pairs = std::max<uint64_t>(S->seen_pairs, c.out_count + c.out_count / 4);
    if (c.out_count <= out_cap(S) && c.seen_overflow == 0) return;
    if (S->ext_l) {
      // the caller's buffer: a result larger than it is only counted; a
      // full duplicate set is grown and the run repeated
      if (c.out_count > S->ext_cap || (c.seen_overflow && c.passes > S->ext_cap)) {
        S->stats.n_matches = c.seen_overflow ? std::max<uint64_t>(c.out_count, c.passes) : c.out_count;
        return;
      }
      S->seen_pairs = std::max<uint64_t>(2 * S->seen_pairs, c.passes);
      fit_seen(S, S->seen_pairs);
      continue;
    }
    const uint64_t need = needed_capacity(S, c);
    if (S->cap_limit && need > S->cap_limit) {
      // the caller's buffer is too small anyway: report the count (an upper
      // bound when the duplicate set overflowed) instead of running again
      S->stats.n_matches = c.seen_overflow ? std::max<uint64_t>(c.out_count, c.passes) : c.out_count;
      return;
    }
    grow_output(S, need);
  }
  fail(HBX_ERR_CAPACITY, "output kept growing");
}

void reserve_output(hbx_session* S, uint64_t pairs) {
  PoolScope scope(S->ctx->pool, S->ctx->stream);
  if (pairs > S->out_l.n) grow_output(S, pairs);
  S->seen_pairs = std::max<uint64_t>(S->seen_pairs, pairs);
}

void run_to_host(hbx_session* S, hbx_mode mode, std::vector<uint32_t>* l, std::vector<uint32_t>* r) {
  cudaStream_t st = S->ctx->stream;
  S->one_shot = true;  // no graph for a single run
  PoolScope scope(S->ctx->pool, st);
  session_run(S, mode, st);
  const uint64_t n = S->stats.n_matches;
  l->resize(n);
  r->resize(n);
  if (n) {
    HBX_CUDA(cudaMemcpyAsync(l->data(), S->out_l.p, n * 4, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaMemcpyAsync(r->data(), S->out_r.p, n * 4, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaStreamSynchronize(st));
  }
}

}  // namespace hbx

// ============================================================== C ABI (CUDA)
namespace {

// Copies bytes from src to dst with up to one thread per host core for
// large copies (the first touch of a caller's fresh pages and the copy
// itself both scale with threads; one thread copied C3's 4.1 GB of pairs at
// about 2.5 GB/s).
void parallel_copy(void* dst, const void* src, size_t bytes) {
  constexpr size_t kPerThread = 64ull << 20;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t n = std::min<size_t>(std::min<size_t>(hw, 32), (bytes + kPerThread - 1) / kPerThread);
  if (n <= 1) {
    std::memcpy(dst, src, bytes);
    return;
  }
  const size_t part = (bytes / n + 4095) / 4096 * 4096;
  auto copy_part = [=](size_t k) {
    const size_t a = k * part, z = std::min(bytes, a + part);
    if (a < z) std::memcpy(static_cast<char*>(dst) + a, static_cast<const char*>(src) + a, z - a);
  };
  std::vector<std::thread> th;
  size_t k = 1;
  try {
    for (; k < n && k * part < bytes; k++) th.emplace_back(copy_part, k);
  } catch (...) {
    // no thread for part k and later: this thread copies them
  }
  copy_part(0);
  for (size_t j = k; j < n; j++) copy_part(j);
  for (auto& t : th) t.join();
}

// Device -> caller's host memory through the context's two page-locked
// chunks: the copy of chunk i + 1 runs while the host threads move chunk i
// into place.  (Straight into a caller's pageable arrays the copy ran at
// 5.5 GB/s on GB300; through one staging buffer of the whole output it
// slowed from 190 to about 30 GB/s once the host had read that buffer.)
constexpr size_t kOutChunkBytes = 256ull << 20;
void copy_out(hbx_ctx* ctx, cudaStream_t st, void* const* dst, const void* const* src,
              const size_t* bytes, int n_arrays) {
  if (!ctx->h_out) {
    HBX_CUDA(cudaHostAlloc(&ctx->h_out, 2 * kOutChunkBytes, cudaHostAllocPortable));
    for (cudaEvent_t& e : ctx->h_out_ev)
      HBX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  struct Piece {
    char* dst;
    const char* src;
    size_t n;
  };
  std::vector<Piece> pieces;
  for (int a = 0; a < n_arrays; a++)
    for (size_t off = 0; off < bytes[a]; off += kOutChunkBytes)
      pieces.push_back({static_cast<char*>(dst[a]) + off, static_cast<const char*>(src[a]) + off,
                        std::min(kOutChunkBytes, bytes[a] - off)});
  char* slot[2] = {static_cast<char*>(ctx->h_out), static_cast<char*>(ctx->h_out) + kOutChunkBytes};
  auto issue = [&](size_t i) {
    HBX_CUDA(cudaMemcpyAsync(slot[i & 1], pieces[i].src, pieces[i].n, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaEventRecord(ctx->h_out_ev[i & 1], st));
  };
  try {
    if (!pieces.empty()) issue(0);
    for (size_t i = 0; i < pieces.size(); i++) {
      // slot (i + 1) & 1 last held piece i - 1, already moved into place
      if (i + 1 < pieces.size()) issue(i + 1);
      HBX_CUDA(cudaEventSynchronize(ctx->h_out_ev[i & 1]));
      parallel_copy(pieces[i].dst, slot[i & 1], pieces[i].n);
    }
  } catch (...) {
    cudaStreamSynchronize(st);  // no copy into the chunks is left running
    throw;
  }
}

hbx_status guard(hbx_ctx* ctx, const std::function<void()>& f) {
  try {
    f();
    if (ctx) ctx->err.clear();
    return HBX_OK;
  } catch (const hbx::Error& e) {
    if (ctx) ctx->err = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->err = "host out of memory";
    return HBX_ERR_OOM;
  } catch (const std::exception& e) {
    if (ctx) ctx->err = e.what();
    return HBX_ERR_INVALID_ARG;
  }
}

}  // namespace

extern "C" {

hbx_status hbx_ctx_create(int device, const hbx_opts* opts, hbx_ctx** out) {
  if (!out) return HBX_ERR_INVALID_ARG;
  *out = nullptr;
  auto ctx = std::make_unique<hbx_ctx>();
  ctx->opts.struct_size = sizeof(hbx_opts);
  ctx->opts.use_graph = 1;
  if (opts) {
    if (opts->struct_size != sizeof(hbx_opts)) return HBX_ERR_INVALID_ARG;
    if (opts->pred_order < 0 || opts->pred_order > 1) return HBX_ERR_INVALID_ARG;
    if (opts->eval_variant < 0 || opts->eval_variant > 2) return HBX_ERR_INVALID_ARG;
    if (opts->ingest < 0 || opts->ingest > 1) return HBX_ERR_INVALID_ARG;
    ctx->opts = *opts;
  }
  hbx_status s = guard(ctx.get(), [&] {
    int n = 0;
    HBX_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) hbx::fail(HBX_ERR_INVALID_ARG, "no such CUDA device");
    ctx->device = device;
    HBX_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    HBX_CUDA(cudaGetDeviceProperties(&prop, device));
    ctx->n_sm = prop.multiProcessorCount;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
    ctx->smem_per_sm = prop.sharedMemPerMultiprocessor;
    ctx->device_name = prop.name;
    HBX_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    HBX_CUDA(cudaMemPoolCreate(&ctx->pool, &props));
    uint64_t keep = UINT64_MAX;  // freed blocks stay in the pool for the next session
    HBX_CUDA(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  });
  if (s != HBX_OK) return s;
  *out = ctx.release();
  return HBX_OK;
}

hbx_status hbx_ctx_destroy(hbx_ctx* ctx) {
  if (!ctx) return HBX_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->h_ctr) cudaFreeHost(ctx->h_ctr);
  if (ctx->h_out) cudaFreeHost(ctx->h_out);
  for (cudaEvent_t e : ctx->h_out_ev)
    if (e) cudaEventDestroy(e);
  delete ctx;
  return HBX_OK;
}

const char* hbx_host_last_error(void);

const char* hbx_last_error(const hbx_ctx* ctx) {
  return ctx ? ctx->err.c_str() : hbx_host_last_error();
}

void hbx_internal_set_error(hbx_ctx* ctx, const char* msg) {
  if (ctx) ctx->err = msg ? msg : "";
}

hbx_status hbx_session_create(hbx_ctx* ctx, const hbx_plan* plan, const hbx_table* left,
                              const hbx_table* right, uint64_t n_partitions, int64_t prefix_idx,
                              hbx_session** out) {
  if (!ctx || !plan || !left || !right || !out) return HBX_ERR_INVALID_ARG;
  *out = nullptr;
  auto S = std::make_unique<hbx_session>();
  S->ctx = ctx;
  hbx_status st = guard(ctx, [&] {
    if (prefix_idx != INT_MAX && (prefix_idx < 0 || prefix_idx > INT_MAX))
      hbx::fail(HBX_ERR_INVALID_ARG, "prefix_idx out of range");
    HBX_CUDA(cudaSetDevice(ctx->device));
    hbx::create_session(S.get(), plan, left, right, n_partitions, prefix_idx);
  });
  if (st != HBX_OK) return st;
  *out = S.release();
  return HBX_OK;
}

hbx_status hbx_session_run(hbx_session* s, hbx_mode mode, hbx_pairs* out, void* stream) {
  if (!s || !out) return HBX_ERR_INVALID_ARG;
  if (mode != HBX_MODE_PLAIN && mode != HBX_MODE_BATCHED) return HBX_ERR_INVALID_ARG;
  return guard(s->ctx, [&] {
    cudaStream_t st = stream ? (cudaStream_t)stream : s->ctx->stream;
    hbx::PoolScope scope(s->ctx->pool, st);
    // the kernels write the caller's device buffers directly
    const bool ext = out->l_row && out->r_row && out->capacity > 0;
    s->ext_l = ext ? out->l_row : nullptr;
    s->ext_r = ext ? out->r_row : nullptr;
    s->ext_cap = ext ? out->capacity : 0;
    s->cap_limit = ext ? 0 : 1;  // no buffer: count only
    hbx::session_run(s, mode, st);
    const uint64_t n = s->stats.n_matches;
    out->n_required = n;
    out->n_written = 0;
    if (n > out->capacity) hbx::fail(HBX_ERR_CAPACITY, "output capacity below the match count");
    out->n_written = n;
  });
}

hbx_status hbx_session_stats(const hbx_session* s, hbx_stats* out) {
  if (!s || !out) return HBX_ERR_INVALID_ARG;
  *out = s->stats;
  return HBX_OK;
}

hbx_status hbx_session_destroy(hbx_session* s) {
  if (!s) return HBX_ERR_INVALID_ARG;
  cudaSetDevice(s->ctx->device);
  delete s;
  return HBX_OK;
}

hbx_status hbx_block(hbx_ctx* ctx, const hbx_plan* plan, const hbx_table* left,
                     const hbx_table* right, uint64_t n_partitions, int64_t prefix_idx,
                     hbx_mode mode, hbx_pairs* out, hbx_stats* stats, void* stream) {
  if (!ctx || !out) return HBX_ERR_INVALID_ARG;
  if (!plan || !left || !right) return HBX_ERR_INVALID_ARG;
  auto S = std::make_unique<hbx_session>();
  S->ctx = ctx;
  S->one_shot = true;
  // the caller's buffer sizes the device output; a larger result is only counted
  S->out_hint = out->capacity;
  S->cap_limit = std::max<uint64_t>(out->capacity, 1);
  hbx_session* s = S.get();
  hbx_status st = guard(ctx, [&] {
    if (prefix_idx != INT_MAX && (prefix_idx < 0 || prefix_idx > INT_MAX))
      hbx::fail(HBX_ERR_INVALID_ARG, "prefix_idx out of range");
    HBX_CUDA(cudaSetDevice(ctx->device));
    hbx::PoolScope scope(ctx->pool, ctx->stream);
    // the session is encoded on the context's stream (its creation ends with
    // that stream idle); the run and the copies go to the caller's stream
    hbx::create_session(s, plan, left, right, n_partitions, prefix_idx);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    hbx::session_run(s, mode, st);
    const uint64_t n = s->stats.n_matches;
    out->n_required = n;
    out->n_written = 0;
    if (stats) *stats = s->stats;
    if (n > out->capacity) hbx::fail(HBX_ERR_CAPACITY, "output capacity below the match count");
    if (n) {
      if (!out->l_row || !out->r_row) hbx::fail(HBX_ERR_INVALID_ARG, "null output pointer");
      void* dst[2] = {out->l_row, out->r_row};
      const void* src[2] = {s->out_l.p, s->out_r.p};
      const size_t bytes[2] = {n * 4, n * 4};
      copy_out(ctx, st, dst, src, bytes, 2);
    }
    out->n_written = n;
  });
  S.reset();
  return st;
}

// run_hyperblocker_exec's pipeline with the pairs kept on the device: one
// session run, the pairs sorted by (left row, right row), their id lines
// formatted and appended to path.
hbx_status hbx_internal_block_to_file(hbx_ctx* ctx, const hbx_plan* plan, const hbx_table* left,
                                      const hbx_table* right, uint64_t n_partitions,
                                      int64_t prefix_idx, hbx_mode mode, const char* path,
                                      hbx_stats* stats) {
  if (!ctx || !plan || !left || !right || !path) return HBX_ERR_INVALID_ARG;
  auto S = std::make_unique<hbx_session>();
  S->ctx = ctx;
  S->one_shot = true;
  hbx_session* s = S.get();
  hbx_status st = guard(ctx, [&] {
    if (prefix_idx != INT_MAX && (prefix_idx < 0 || prefix_idx > INT_MAX))
      hbx::fail(HBX_ERR_INVALID_ARG, "prefix_idx out of range");
    HBX_CUDA(cudaSetDevice(ctx->device));
    hbx::PoolScope scope(ctx->pool, ctx->stream);
    hbx::create_session(s, plan, left, right, n_partitions, prefix_idx);
    hbx::session_run(s, mode, ctx->stream);
    const uint64_t n = s->stats.n_matches;
    if (stats) *stats = s->stats;
    hbx::sort_pairs_device(ctx, s->out_l.p, s->out_r.p, n, (uint32_t)left->t.n_rows,
                           (uint32_t)right->t.n_rows);
    hbx::write_pairs_device(ctx, left->t, right->t, s->out_l.p, s->out_r.p, n, path);
  });
  S.reset();
  return st;
}

}  // extern "C"
