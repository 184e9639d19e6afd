// serve.cu -- the serving loop: one right table resident on the device,
// requests of left records answered with continuous batching (include/hbx.h,
// "serving").
//
// Resident state (built once by hbx_serve_open):
//   * the right table's columns that the plans read, encoded on the device
//     with the session ingest kernels: one dictionary per right equality
//     column, kept as an open-addressing lookup table (hash -> code, with the
//     representative row for an exact byte check); the right alphabet
//     (frequency ordered) and the symbol arenas + metadata of its strings;
//   * per rule of every plan, the right side of the equality join: right rows
//     grouped by join key (counting sort) with their string metadata in the
//     same order -- exactly what dev::Rule's right half holds for a session.
//
// Per batch (worker thread, one CUDA stream per batch slot):
//   * the admitted requests' records are concatenated (request q owns batch
//     rows [base_q, base_q + n_q)), copied once and encoded: each equality
//     cell becomes the resident code of the equal right cell, or -1 when no
//     right cell is equal (then the row joins nothing); string bytes become
//     resident symbols, bytes no right string contains become one reserved
//     symbol that equals no right symbol -- so every comparison the kernels
//     make gives the answer the raw bytes give;
//   * every (request, rule) pair is a rule instance: its left rows are the
//     request's rows grouped by join key; the right half is the resident one;
//   * one persistent k_eval launch runs all work items of all instances; the
//     pairs (batch row, right row) go back to the host and are split by the
//     requests' row ranges.  Instances of one request share the batch's
//     duplicate set (several rules of a plan), rows of different requests
//     never meet, so a result is the same in any batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "context.h"
#include "device_buffers.h"
#include "encode.h"
#include "hbx_core.h"
#include "ingest.h"
#include "kernels.cuh"
#include "std_hash.h"

namespace hbx {
namespace srv {

using Clock = std::chrono::steady_clock;

// ------------------------------------------------------------------ kernels

// Resident code of each left cell: the code of the right cell with the same
// bytes (up to the first NUL), or -1 when there is none.  The table holds one
// slot per distinct right hash (right collisions are refused at open), so a
// hash match with different bytes also means "no equal right cell".
__global__ void k_lookup(ing::ColDev lc, uint32_t n, const unsigned long long* keys,
                         const uint32_t* code, const uint32_t* rep, uint32_t mask, ing::ColDev rc,
                         int32_t* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int64_t a;
    const uint32_t len = ing::cell_len(lc, i, &a);
    unsigned long long h = std_hash_bytes(lc.bytes + a, len);
    if (h == ing::kEmpty) h = ing::kEmpty - 1;
    uint32_t slot = (uint32_t)(h ^ (h >> 32)) & mask;
    int32_t c = -1;
    for (uint32_t probe = 0; probe <= mask; probe++) {
      const unsigned long long k = keys[slot];
      if (k == ing::kEmpty) break;
      if (k == h) {
        int64_t b;
        const uint32_t lb = ing::cell_len(rc, rep[slot], &b);
        bool same = lb == len;
        for (uint32_t j = 0; same && j < len; j++) same = lc.bytes[a + j] == rc.bytes[b + j];
        if (same) c = (int32_t)code[slot];
        break;
      }
      slot = (slot + 1) & mask;
    }
    out[i] = c;
  }
}

// Left join key of the request rows [row0, row0 + n) for rule instance inst
// (word class x equality codes in mixed radix), counted per key; rows with an
// equality that has no resident partner get no key.
__global__ void k_keys(const dev::Rule* rules, uint32_t inst, dev::Side L, uint32_t row0,
                       uint32_t n, uint32_t* key_l) {
  const dev::Rule& R = rules[inst];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t row = row0 + i;
    uint32_t key = 0;
    bool ok = true;
    for (uint32_t e = 0; e < R.n_eq; e++) {
      const int32_t c = L.eq_codes[(size_t)R.eq_slot[e] * L.n_rows + row];
      ok = ok && c >= 0;
      key = key * R.radix[e] + (uint32_t)(c < 0 ? 0 : c);
    }
    if (!ok) {
      key_l[i] = 0xffffffffu;
      continue;
    }
    if (R.n_wclass > 1)
      key += R.domain * dev::word_class(L.str_meta[(size_t)R.wclass_slot * L.n_rows + row].loc.y);
    key_l[i] = key;
    atomicAdd(R.cnt_l + key, 1u);
  }
}

__global__ void k_scatter_left(const dev::Rule* rules, uint32_t inst, uint32_t row0, uint32_t n,
                               const uint32_t* key_l) {
  const dev::Rule& R = rules[inst];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t k = key_l[i];
    if (k == 0xffffffffu) continue;
    R.sorted_l[R.off_l[k] + atomicAdd(R.cur_l + k, 1u)] = row0 + i;
  }
}

// Request-side symbol of every byte: the resident symbol, or `unseen` for a
// byte no resident string contains.
__global__ void k_lut(const uint8_t* sym, uint32_t unseen, uint8_t* lut) {
  const uint32_t b = threadIdx.x;
  lut[b] = b == 0 ? 0 : (sym[b] ? sym[b] : (uint8_t)unseen);
}

// ------------------------------------------------------------------ host side

struct DevColumn {
  DBuf<uint8_t> bytes;
  DBuf<int64_t> off;
  uint32_t has_nul = 0;
  ing::ColDev view() const { return ing::ColDev{bytes.p, off.p, has_nul}; }
};

struct Dict {
  int rcol = -1;
  DBuf<unsigned long long> keys;
  DBuf<uint32_t> code, rep;
  uint32_t cap = 0, card = 0;
};

// One rule of one plan with its resident right-side join.
struct RuleT {
  dev::Rule d{};
  DBuf<uint32_t> key_r, cnt_r, off_r, cur_r, sorted_r;
  DBuf<dev::StrMeta> sorted_meta_r;
};

// A request: its records, and its progress through the batches.  Records
// are dispatched in row chunks; the result is delivered when the last chunk
// has come back.
struct Request {
  uint64_t id = 0;
  int32_t plan = 0;
  Table rows;
  uint32_t n = 0;
  Clock::time_point t_submit, t_admit;
  bool admitted = false;
  uint32_t next = 0;         // first row not dispatched yet
  uint32_t outstanding = 0;  // chunks in batches that have not come back
  std::vector<std::pair<uint32_t, uint32_t>> pairs;
  uint64_t comparisons = 0;
  uint32_t batch_requests = 0, batch_id = 0;
  hbx_status status = HBX_OK;
};

// Rows [r0, r1) of one request inside a batch.
struct Entry {
  Request* r = nullptr;
  uint32_t r0 = 0, r1 = 0;
  uint32_t n() const { return r1 - r0; }
};

struct Result {
  uint64_t id = 0;
  int32_t plan = 0;
  hbx_status status = HBX_OK;
  std::vector<uint32_t> l, r;
  uint64_t comparisons = 0;
  double ms_queued = 0, ms_total = 0;
  uint32_t batch_requests = 0, batch_id = 0;
};

struct Inst {
  DBuf<uint32_t> key_l, cnt_l, off_l, cur_l, sorted_l;
  DBuf<unsigned long long> item_off, part_u64;
  DBuf<uint32_t> part_u32;
  uint32_t nb_l = 0;
  uint32_t req = 0;  // entry index within the batch
};

// Page-locked host buffer that grows by powers of two.  A buffer it
// outgrows is kept until the slot closes: cudaFreeHost waits for the whole
// device, which would stall every other batch in flight (and the old buffer
// may still be the source or target of this slot's copies).  The kept
// buffers add up to less than the current one.
struct Pinned {
  void* p = nullptr;
  size_t n = 0;
  std::vector<void*> retired;
  Pinned() = default;
  Pinned(const Pinned&) = delete;
  Pinned& operator=(const Pinned&) = delete;
  ~Pinned() {
    if (p) cudaFreeHost(p);
    for (void* q : retired) cudaFreeHost(q);
  }
  void ensure(size_t bytes) {
    if (bytes <= n) return;
    size_t want = 1 << 16;
    while (want < bytes) want *= 2;
    void* q = nullptr;
    HBX_CUDA(cudaHostAlloc(&q, want, cudaHostAllocPortable));
    if (p) retired.push_back(p);
    p = q;
    n = want;
  }
};

// One batch in flight.
struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t ev_start = nullptr, ev_eval = nullptr, ev_out = nullptr;
  int state = 0;  // 0 idle, 1 evaluating, 2 copying pairs back
  uint32_t batch_id = 0;
  std::vector<Entry> ents;
  std::vector<uint32_t> base;  // first batch row of each entry (+ total)
  uint64_t est = 0;
  uint32_t n_rows = 0;
  std::vector<DevColumn> cols;  // per needed left column
  SideBufs L;
  dev::Side side_l{};
  std::vector<Inst> inst;
  std::vector<dev::Rule> h_rules;
  DBuf<dev::Rule> d_rules;
  DBuf<unsigned long long> d_base, d_cmp, seen;
  DBuf<dev::Counters> d_ctr;
  DBuf<uint32_t> out_l, out_r;
  uint64_t capacity = 0;
  uint64_t cmp_first = 0;  // comparisons counted by the first evaluation pass
  dev::PeqShape shape{};   // Peq tables of this batch's left strings
  DBuf<uint32_t> peq;
  Pinned stage, h_out, h_ctr;  // h_ctr: Counters + total items + comparisons per instance
  ~Slot() {
    release();  // buffers return to the pool on this slot's stream first
    for (cudaEvent_t e : {ev_start, ev_eval, ev_out})
      if (e) cudaEventDestroy(e);
    if (st) cudaStreamDestroy(st);
  }
  void release() {
    ents.clear();
    base.clear();
    cols.clear();
    L = SideBufs{};
    inst.clear();
    h_rules.clear();
    d_rules.reset();
    d_base.reset();
    d_cmp.reset();
    seen.reset();
    d_ctr.reset();
    out_l.reset();
    out_r.reset();
    peq.reset();
    capacity = 0;
    state = 0;
  }
};

}  // namespace srv
}  // namespace hbx

using namespace hbx;
using namespace hbx::srv;

struct hbx_server {
  hbx_ctx* ctx = nullptr;
  hbx_serve_opts opts{};
  // resident table
  uint32_t n_right = 0;
  std::vector<std::pair<int, int>> pairs;  // equality slots: (left column, right column)
  std::vector<int> pair_dict;
  std::vector<Dict> dicts;
  std::vector<int> lstr, rstr;  // string slots: left columns / right columns
  std::map<int, DevColumn> rcols;
  SideBufs R;
  dev::Side side_r{};
  DBuf<uint8_t> sym, lut;
  uint32_t n_symbols = 1;  // for the kernel: resident alphabet + the unseen symbol
  std::vector<std::unique_ptr<RuleT>> rules;
  std::vector<std::vector<int>> plan_rules;
  std::vector<int> left_cols;  // left columns any plan reads
  int left_cols_min = 0;
  bool any_multi_rule = false;
  uint64_t resident_bytes = 0;
  // kernel configuration
  uint32_t tile_right = 128;
  int variant = 1;
  dev::WarpLayout wl{};
  size_t smem_bytes = 0;
  int blocks_per_sm = 1;
  // queue and results
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<std::unique_ptr<Request>> active;  // submitted, result not delivered yet
  std::deque<Result> done;
  Result current;
  bool stopping = false;
  bool failed = false;
  std::string err;
  std::thread worker;
  std::vector<std::unique_ptr<Slot>> slots;
  uint64_t budget = 0, in_use = 0, peak = 0;
  uint32_t next_batch = 0;
  hbx_serve_stats st{};
};

namespace hbx {
namespace srv {
namespace {

constexpr int kThreads = dev::kWarpsPerCta * 32;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

uint32_t next_pow2_at_least(uint64_t n, uint32_t lo) {
  uint64_t c = lo;
  while (c < n) c <<= 1;
  if (c > (1ull << 31)) fail(HBX_ERR_UNSUPPORTED, "resident table too large for its dictionary");
  return (uint32_t)c;
}

void upload_column(const Column& c, DevColumn* d, cudaStream_t st) {
  d->bytes.alloc(std::max<size_t>(c.bytes.size(), 16));
  d->off.alloc(c.off.size());
  if (!c.bytes.empty())
    HBX_CUDA(cudaMemcpyAsync(d->bytes.p, c.bytes.data(), c.bytes.size(), cudaMemcpyHostToDevice, st));
  HBX_CUDA(cudaMemcpyAsync(d->off.p, c.off.data(), c.off.size() * sizeof(int64_t),
                           cudaMemcpyHostToDevice, st));
  d->has_nul = c.has_nul ? 1u : 0u;
}

// Symbol arenas + metadata of string columns (slot-major), as device_encode.
void pack_strings(const std::vector<const DevColumn*>& cols, const std::vector<uint64_t>& col_bytes,
                  uint32_t n, const uint8_t* sym, SideBufs* B, int n_sm, cudaStream_t st,
                  unsigned long long* maxlen) {
  const size_t ns = cols.size();
  uint64_t bound = 16;
  for (uint64_t b : col_bytes) bound += b + 15ull * n;
  bound = (bound + 15) / 16 * 16;
  if (bound / 16 > UINT32_MAX) fail(HBX_ERR_UNSUPPORTED, "string arena above 64 GiB");
  B->arena.alloc(bound);
  HBX_CUDA(cudaMemsetAsync(B->arena.p, 0, bound, st));
  B->meta.alloc(std::max<size_t>(ns * n, 1));
  if (!ns || !n) return;
  if ((uint64_t)ns * n > UINT32_MAX) fail(HBX_ERR_UNSUPPORTED, "more than 2^32 strings");
  DBuf<uint32_t> units, off16;
  units.alloc(ns * n);
  off16.alloc(ns * n);
  for (size_t s = 0; s < ns; s++)
    ing::k_units<<<grid_for(n, n_sm), 256, 0, st>>>(cols[s]->view(), n, units.p + s * n);
  scan_u32(units.p, (uint32_t)(ns * n), off16.p, st);
  for (size_t s = 0; s < ns; s++)
    ing::k_pack<<<grid_for((uint64_t)n * 32, n_sm), 256, 0, st>>>(
        cols[s]->view(), n, off16.p + s * n, sym, B->arena.p, B->meta.p + s * n, maxlen + s);
  check_launch("serving string arenas");
}

void open_server(hbx_server* S, const hbx_plan* const* plans, int32_t n_plans, const hbx_table* right) {
  hbx_ctx* C = S->ctx;
  cudaStream_t st = C->stream;
  PoolScope scope(C->pool, st);
  const Table& TR = right->t;
  if (TR.n_rows > (int64_t)(1u << 30)) fail(HBX_ERR_UNSUPPORTED, "resident table above 2^30 rows");
  const uint32_t nR = (uint32_t)TR.n_rows;
  S->n_right = nR;
  pin_table(right);

  // ---- slots of all plans
  auto pair_of = [&](int cl, int cr) {
    for (size_t k = 0; k < S->pairs.size(); k++)
      if (S->pairs[k].first == cl && S->pairs[k].second == cr) return (int)k;
    S->pairs.emplace_back(cl, cr);
    return (int)S->pairs.size() - 1;
  };
  auto slot_of = [](std::vector<int>& v, int col) {
    for (size_t k = 0; k < v.size(); k++)
      if (v[k] == col) return (int)k;
    v.push_back(col);
    return (int)v.size() - 1;
  };
  struct Pending {
    std::vector<int> eq_pair, sim_l, sim_r;
    std::vector<float> thr;
  };
  std::vector<std::vector<Pending>> per_plan((size_t)n_plans);
  for (int32_t p = 0; p < n_plans; p++) {
    if (!plans[p]) fail(HBX_ERR_INVALID_ARG, "null plan");
    const Plan& P = plans[p]->p;
    if (P.compiled.empty()) fail(HBX_ERR_INVALID_ARG, "a plan without rules");
    if (P.compiled.size() > 1) S->any_multi_rule = true;
    for (const CompiledRule& cr : P.compiled) {
      Pending pr;
      for (const Pred& e : cr.eqs) {
        if (e.col_r >= TR.n_cols()) fail(HBX_ERR_UNSUPPORTED, "an equality uses a column the resident table does not have");
        pr.eq_pair.push_back(pair_of(e.col_l, e.col_r));
        S->left_cols_min = std::max(S->left_cols_min, e.col_l + 1);
      }
      for (const Pred& s : cr.sims) {
        if (s.col_r >= TR.n_cols()) fail(HBX_ERR_UNSUPPORTED, "a similarity uses a column the resident table does not have");
        pr.sim_l.push_back(slot_of(S->lstr, s.col_l));
        pr.sim_r.push_back(slot_of(S->rstr, s.col_r));
        pr.thr.push_back(s.thr);
        S->left_cols_min = std::max(S->left_cols_min, s.col_l + 1);
      }
      if (pr.eq_pair.size() > (size_t)dev::kMaxEq || pr.sim_l.size() > (size_t)dev::kMaxSim)
        fail(HBX_ERR_UNSUPPORTED, "too many predicates in a rule");
      per_plan[(size_t)p].push_back(pr);
    }
  }
  for (auto& pr : S->pairs) slot_of(S->left_cols, pr.first);
  for (int c : S->lstr) slot_of(S->left_cols, c);

  // ---- resident columns
  for (auto& pr : S->pairs)
    if (!S->rcols.count(pr.second)) upload_column(TR.cols[(size_t)pr.second], &S->rcols[pr.second], st);
  for (int c : S->rstr)
    if (!S->rcols.count(c)) upload_column(TR.cols[(size_t)c], &S->rcols[c], st);

  const size_t n_sum = ing::kSumFixed + 1 + S->rstr.size();
  DBuf<unsigned long long> sum;
  sum.alloc(n_sum);
  HBX_CUDA(cudaMemsetAsync(sum.p, 0, n_sum * sizeof(unsigned long long), st));

  // ---- dictionaries of the right equality columns
  std::vector<DBuf<int32_t>> codes_of_col;
  std::map<int, int> dict_of_col;
  for (auto& pr : S->pairs) {
    if (dict_of_col.count(pr.second)) continue;
    dict_of_col[pr.second] = (int)S->dicts.size();
    S->dicts.emplace_back();
    Dict& D = S->dicts.back();
    D.rcol = pr.second;
    D.cap = next_pow2_at_least(2ull * nR, 1024);
    D.keys.alloc(D.cap);
    D.rep.alloc(D.cap);
    D.code.alloc(D.cap);
    HBX_CUDA(cudaMemsetAsync(D.keys.p, 0xff, (size_t)D.cap * 8, st));
    HBX_CUDA(cudaMemsetAsync(D.rep.p, 0xff, (size_t)D.cap * 4, st));
    DBuf<uint32_t> row_slot, occ;
    row_slot.alloc(std::max<uint32_t>(nR, 1));
    occ.alloc(D.cap);
    codes_of_col.emplace_back();
    codes_of_col.back().alloc(std::max<uint32_t>(nR, 1));
    const ing::ColDev rc = S->rcols[pr.second].view();
    if (nR)
      ing::k_dict_insert<<<grid_for(nR, C->n_sm), 256, 0, st>>>(rc, nR, 0, D.keys.p, D.rep.p,
                                                                 D.cap - 1, row_slot.p, sum.p,
                                                                 kDictSeed);
    ing::k_occupied<<<grid_for(D.cap, C->n_sm), 256, 0, st>>>(D.keys.p, D.cap, occ.p);
    scan_u32(occ.p, D.cap, D.code.p, st);
    if (nR)
      ing::k_dict_assign<<<grid_for(nR, C->n_sm), 256, 0, st>>>(
          rc, nR, 0, row_slot.p, D.code.p, D.rep.p, rc, rc, nR, codes_of_col.back().p, sum.p);
    ing::k_scan_total<<<1, 32, 0, st>>>(D.code.p, occ.p, D.cap, 0, sum.p + ing::kSumFixed);
    check_launch("serving dictionary");
    unsigned long long card = 0, flags = 0;
    HBX_CUDA(cudaMemcpyAsync(&card, sum.p + ing::kSumFixed, 8, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaMemcpyAsync(&flags, sum.p + ing::kSumFlags, 8, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaStreamSynchronize(st));
    if (flags)
      fail(HBX_ERR_UNSUPPORTED, "two distinct cells of a resident equality column share a 64-bit hash");
    D.card = (uint32_t)std::max<unsigned long long>(card, 1);
  }
  for (auto& pr : S->pairs) S->pair_dict.push_back(dict_of_col[pr.second]);
  S->R.eq.alloc(std::max<size_t>(S->pairs.size() * (size_t)nR, 1));
  for (size_t k = 0; k < S->pairs.size(); k++)
    if (nR)
      HBX_CUDA(cudaMemcpyAsync(S->R.eq.p + k * nR, codes_of_col[(size_t)S->pair_dict[k]].p,
                               (size_t)nR * 4, cudaMemcpyDeviceToDevice, st));

  // ---- resident alphabet, arenas, string metadata
  DBuf<unsigned long long> bhist;
  bhist.alloc(256);
  S->sym.alloc(256);
  S->lut.alloc(256);
  HBX_CUDA(cudaMemsetAsync(bhist.p, 0, 256 * 8, st));
  for (int c : S->rstr) {
    const Column& col = TR.cols[(size_t)c];
    const uint64_t work = col.has_nul ? nR : (col.bytes.size() + 15) / 16;
    if (nR) ing::k_byte_hist<<<grid_for(work, C->n_sm, 4), 256, 0, st>>>(S->rcols[c].view(), nR, bhist.p);
  }
  ing::k_symbol_map<<<1, 256, 0, st>>>(bhist.p, S->sym.p, sum.p);
  unsigned long long ns = 1;
  HBX_CUDA(cudaMemcpyAsync(&ns, sum.p + ing::kSumSymbols, 8, cudaMemcpyDeviceToHost, st));
  HBX_CUDA(cudaStreamSynchronize(st));
  const uint32_t unseen = ns < 256 ? (uint32_t)ns : 0u;  // 0: every byte value occurs
  S->n_symbols = (uint32_t)ns + (ns < 256 ? 1u : 0u);
  k_lut<<<1, 256, 0, st>>>(S->sym.p, unseen, S->lut.p);
  {
    std::vector<const DevColumn*> cols;
    std::vector<uint64_t> bytes;
    for (int c : S->rstr) {
      cols.push_back(&S->rcols[c]);
      bytes.push_back(TR.cols[(size_t)c].bytes.size());
    }
    pack_strings(cols, bytes, nR, S->sym.p, &S->R, C->n_sm, st, sum.p + ing::kSumFixed + 1);
  }
  S->R.bucket.alloc(std::max<uint32_t>(nR, 1));
  HBX_CUDA(cudaMemsetAsync(S->R.bucket.p, 0, (size_t)std::max<uint32_t>(nR, 1) * 4, st));
  S->R.comp.alloc(1);
  S->side_r = dev::Side{S->R.bucket.p, S->R.eq.p, S->R.comp.p, S->R.arena.p, S->R.meta.p, nR};

  // ---- kernel configuration
  S->tile_right = S->opts.tile_right > 0 ? (uint32_t)S->opts.tile_right : 128u;
  S->tile_right = std::min<uint32_t>(512, std::max<uint32_t>(32, (S->tile_right + 31) / 32 * 32));
  S->variant = S->opts.eval_variant == 1 ? 0 : 1;
  const size_t smem_cap = std::min<size_t>(C->smem_optin, 200 * 1024);
  const uint32_t cap_warp_words = (uint32_t)(smem_cap / 4 / dev::kWarpsPerCta) / 4 * 4;
  S->wl = dev::warp_layout_fit(S->tile_right, smem_cap);
  if (S->wl.warp_words > cap_warp_words) fail(HBX_ERR_INVALID_ARG, "tile_right too large");
  S->smem_bytes = (size_t)S->wl.warp_words * 4 * dev::kWarpsPerCta;

  // ---- rules and their resident right-side joins
  for (int32_t p = 0; p < n_plans; p++) {
    S->plan_rules.emplace_back();
    for (const Pending& pr : per_plan[(size_t)p]) {
      auto T = std::make_unique<RuleT>();
      dev::Rule& d = T->d;
      d.n_eq = (uint32_t)pr.eq_pair.size();
      d.n_sim = (uint32_t)pr.sim_l.size();
      uint64_t D = 1;
      for (size_t e = 0; e < pr.eq_pair.size(); e++) {
        d.eq_slot[e] = (uint32_t)pr.eq_pair[e];
        d.radix[e] = S->dicts[(size_t)S->pair_dict[(size_t)pr.eq_pair[e]]].card;
        D *= d.radix[e];
        if (D > kMaxKeyDomain)
          fail(HBX_ERR_UNSUPPORTED, "a served rule's equality key domain is above 2^24");
      }
      for (size_t s = 0; s < pr.sim_l.size(); s++) {
        d.sim_l[s] = (uint32_t)pr.sim_l[s];
        d.sim_r[s] = (uint32_t)pr.sim_r[s];
        d.thr[s] = pr.thr[s];
      }
      d.domain = (uint32_t)D;
      d.n_wclass = (d.n_sim && D * dev::kWordClasses <= (1ull << 22)) ? dev::kWordClasses : 1u;
      d.wclass_slot = d.n_sim ? d.sim_l[0] : 0u;
      d.domain_l = d.n_wclass * d.domain;
      dev::make_singleton(&d);
      // right half of the join: rows grouped by key, metadata in that order
      T->key_r.alloc(std::max<uint32_t>(nR, 1));
      T->cnt_r.alloc(D);
      T->off_r.alloc(D);
      T->cur_r.alloc(D);
      T->sorted_r.alloc((size_t)nR + 4);
      HBX_CUDA(cudaMemsetAsync(T->cnt_r.p, 0, D * 4, st));
      HBX_CUDA(cudaMemsetAsync(T->cur_r.p, 0, D * 4, st));
      HBX_CUDA(cudaMemsetAsync(T->sorted_r.p, 0, ((size_t)nR + 4) * 4, st));
      if (d.n_sim) T->sorted_meta_r.alloc(std::max<uint32_t>(nR, 1));
      d.key_r = T->key_r.p;
      d.cnt_r = T->cnt_r.p;
      d.off_r = T->off_r.p;
      d.cur_r = T->cur_r.p;
      d.sorted_r = T->sorted_r.p;
      d.sorted_meta_r = d.n_sim ? T->sorted_meta_r.p : nullptr;
      DBuf<dev::Rule> tmp;
      tmp.alloc(1);
      HBX_CUDA(cudaMemcpyAsync(tmp.p, &d, sizeof d, cudaMemcpyHostToDevice, st));
      if (nR) dev::k_keys_hist<<<grid_for(nR, C->n_sm), 256, 0, st>>>(S->side_r, tmp.p, 0, 1);
      scan_u32(T->cnt_r.p, (uint32_t)D, T->off_r.p, st);
      if (nR) dev::k_scatter<<<grid_for(nR, C->n_sm), 256, 0, st>>>(S->side_r, tmp.p, 0, 1);
      check_launch("serving right join");
      HBX_CUDA(cudaStreamSynchronize(st));  // tmp and d (host) are read by the copies above
      S->plan_rules.back().push_back((int)S->rules.size());
      S->rules.push_back(std::move(T));
    }
  }
  // a request batch's longest left string picks the mask width: the grid is
  // sized by the width with the fewest resident blocks
  S->blocks_per_sm = 1 << 20;
  for (uint32_t w : dev::kPeqWidths) {
    const dev::EvalKernel kern = dev::eval_kernel(S->variant, false, w);
    raise_smem_limit(kern, S->smem_bytes);
    int bps = 0;
    HBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, kThreads, S->smem_bytes));
    S->blocks_per_sm = std::max(1, std::min(S->blocks_per_sm, bps));
  }
  HBX_CUDA(cudaStreamSynchronize(st));

  uint64_t rb = S->R.eq.n * 4 + S->R.arena.n + S->R.meta.n * sizeof(dev::StrMeta) + S->R.bucket.n * 4;
  for (auto& kv : S->rcols) rb += kv.second.bytes.n + kv.second.off.n * 8;
  for (auto& D : S->dicts) rb += (uint64_t)D.cap * 16;
  for (auto& T : S->rules)
    rb += (T->key_r.n + T->cnt_r.n + T->off_r.n + T->cur_r.n + T->sorted_r.n) * 4 +
          T->sorted_meta_r.n * sizeof(dev::StrMeta);
  S->resident_bytes = rb;

  // ---- budget and batch slots
  size_t free_b = 0, total_b = 0;
  HBX_CUDA(cudaMemGetInfo(&free_b, &total_b));
  S->budget = S->opts.budget_bytes ? S->opts.budget_bytes : (uint64_t)free_b / 2;
  const int n_slots = S->opts.max_inflight > 0 ? S->opts.max_inflight : 2;
  for (int k = 0; k < n_slots; k++) {
    auto sl = std::make_unique<Slot>();
    HBX_CUDA(cudaStreamCreateWithFlags(&sl->st, cudaStreamNonBlocking));
    HBX_CUDA(cudaEventCreate(&sl->ev_start));
    HBX_CUDA(cudaEventCreate(&sl->ev_eval));
    HBX_CUDA(cudaEventCreate(&sl->ev_out));
    S->slots.push_back(std::move(sl));
  }
  S->st.budget_bytes = S->budget;
  S->st.resident_bytes = S->resident_bytes;
}

// Device memory rows [r0, r1) of a request need while their batch is in
// flight (upper bound).
uint64_t estimate(const hbx_server* S, const Table& t, int32_t plan, uint32_t r0, uint32_t r1) {
  const uint64_t n = r1 - r0;
  uint64_t b = 0;
  auto bytes = [&](int c) {
    const Column& col = t.cols[(size_t)c];
    return (uint64_t)(col.off[r1] - col.off[r0]);
  };
  for (int c : S->left_cols) b += bytes(c) + 8 * (n + 1) + 16;
  for (int c : S->lstr) b += bytes(c) + 15 * n + 16 + 40 * n;  // arena, metadata, scan
  // Peq tables, at most 8 words per symbol row
  b += 4ull * ((8ull * S->n_symbols + 3) / 4 * 4) * n * S->lstr.size() + 16;
  b += sizeof(dev::StrMeta) * n * S->lstr.size() + 4 * n * S->pairs.size();
  for (int r : S->plan_rules[(size_t)plan]) {
    const dev::Rule& d = S->rules[(size_t)r]->d;
    b += 12ull * n + 20ull * d.domain_l + 64 + 8 * ((d.domain_l + dev::kScanChunk - 1) / dev::kScanChunk + 1);
  }
  b += 16 * n + (S->any_multi_rule ? 64 * n : 0) + 4096;  // output share (grows if needed)
  return b;
}

void launch_batch(hbx_server* S, Slot& B) {
  hbx_ctx* C = S->ctx;
  cudaStream_t st = B.st;
  PoolScope scope(C->pool, st);
  const size_t nq = B.ents.size();
  B.base.assign(nq + 1, 0);
  for (size_t q = 0; q < nq; q++) B.base[q + 1] = B.base[q] + B.ents[q].n();
  const uint32_t N = B.base[nq];
  B.n_rows = N;
  HBX_CUDA(cudaEventRecord(B.ev_start, st));

  // ---- stage the needed left columns (one pinned buffer) and copy them
  const size_t nc = S->left_cols.size();
  std::vector<uint64_t> bytes_c(nc, 0), boff(nc), ooff(nc);
  uint64_t total = 0;
  for (size_t k = 0; k < nc; k++) {
    for (auto& e : B.ents) {
      const Column& col = e.r->rows.cols[(size_t)S->left_cols[k]];
      bytes_c[k] += (uint64_t)(col.off[e.r1] - col.off[e.r0]);
    }
    boff[k] = total;
    total += (bytes_c[k] + 15) / 16 * 16;
  }
  for (size_t k = 0; k < nc; k++) {
    ooff[k] = total;
    total += 8ull * (N + 1);
  }
  B.stage.ensure(total);
  uint8_t* h = (uint8_t*)B.stage.p;
  B.cols.clear();
  B.cols.resize(nc);
  for (size_t k = 0; k < nc; k++) {
    const int c = S->left_cols[k];
    uint64_t pos = 0;
    int64_t* off = (int64_t*)(h + ooff[k]);
    off[0] = 0;
    uint32_t row = 0;
    bool nul = false;
    for (auto& e : B.ents) {
      const Column& col = e.r->rows.cols[(size_t)c];
      const int64_t a = col.off[e.r0], len = col.off[e.r1] - a;
      if (len) std::memcpy(h + boff[k] + pos, col.bytes.data() + a, (size_t)len);
      for (uint32_t i = 0; i < e.n(); i++) off[row + i + 1] = (int64_t)pos + col.off[e.r0 + i + 1] - a;
      pos += (uint64_t)len;
      row += e.n();
      nul = nul || col.has_nul;
    }
    DevColumn& d = B.cols[k];
    d.bytes.alloc(std::max<uint64_t>(bytes_c[k], 16));
    d.off.alloc((size_t)N + 1);
    if (bytes_c[k])
      HBX_CUDA(cudaMemcpyAsync(d.bytes.p, h + boff[k], bytes_c[k], cudaMemcpyHostToDevice, st));
    HBX_CUDA(cudaMemcpyAsync(d.off.p, off, 8ull * (N + 1), cudaMemcpyHostToDevice, st));
    d.has_nul = nul ? 1u : 0u;
  }
  auto col_index = [&](int c) {
    for (size_t k = 0; k < nc; k++)
      if (S->left_cols[k] == c) return k;
    return (size_t)0;
  };
  // Peq tables shaped for the batch's longest left string (bytes bound symbols)
  int64_t max_len = 1;
  for (size_t sl = 0; sl < S->lstr.size(); sl++)
    for (auto& e : B.ents) {
      const Column& col = e.r->rows.cols[(size_t)S->lstr[sl]];
      for (uint32_t i = e.r0; i < e.r1; i++)
        max_len = std::max<int64_t>(max_len, col.off[i + 1] - col.off[i]);
    }
  B.shape = dev::peq_shape((uint32_t)std::min<int64_t>(max_len, 1 << 20), S->n_symbols);

  // ---- encode the batch against the resident dictionaries and alphabet
  B.L.eq.alloc(std::max<size_t>(S->pairs.size() * (size_t)N, 1));
  for (size_t k = 0; k < S->pairs.size(); k++) {
    const Dict& D = S->dicts[(size_t)S->pair_dict[k]];
    k_lookup<<<grid_for(N, C->n_sm), 256, 0, st>>>(
        B.cols[col_index(S->pairs[k].first)].view(), N, D.keys.p, D.code.p, D.rep.p, D.cap - 1,
        S->rcols.at(S->pairs[k].second).view(), B.L.eq.p + k * N);
  }
  {
    std::vector<const DevColumn*> cols;
    std::vector<uint64_t> nb;
    for (int c : S->lstr) {
      cols.push_back(&B.cols[col_index(c)]);
      nb.push_back(bytes_c[col_index(c)]);
    }
    DBuf<unsigned long long> mx;
    mx.alloc(std::max<size_t>(S->lstr.size(), 1));
    HBX_CUDA(cudaMemsetAsync(mx.p, 0, mx.n * 8, st));
    pack_strings(cols, nb, N, S->lut.p, &B.L, C->n_sm, st, mx.p);
  }
  B.L.comp.alloc(1);
  B.side_l = dev::Side{nullptr, B.L.eq.p, B.L.comp.p, B.L.arena.p, B.L.meta.p, N};
  {
    const uint32_t n_slots = (uint32_t)S->lstr.size();
    const size_t words = (size_t)n_slots * N * B.shape.tab_words;
    B.peq.alloc(std::max<size_t>(words, 4));
    if (words) {
      const uint64_t warps = (uint64_t)n_slots * N;
      const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((warps + 7) / 8, (uint64_t)C->n_sm * 16));
      dev::k_peq_build<<<grid, 256, 0, st>>>(B.side_l, n_slots, B.shape, B.peq.p);
    }
  }
  check_launch("serving batch encode");

  // ---- rule instances: (request, rule of its plan)
  B.inst.clear();
  B.h_rules.clear();
  for (size_t q = 0; q < nq; q++)
    for (int r : S->plan_rules[(size_t)B.ents[q].r->plan]) {
      const dev::Rule& t = S->rules[(size_t)r]->d;
      B.inst.emplace_back();
      Inst& I = B.inst.back();
      I.req = (uint32_t)q;
      const uint32_t n = B.ents[q].n();
      I.key_l.alloc(std::max<uint32_t>(n, 1));
      I.cnt_l.alloc(t.domain_l);
      I.off_l.alloc(t.domain_l);
      I.cur_l.alloc(t.domain_l);
      I.sorted_l.alloc(std::max<uint32_t>(n, 1));
      I.item_off.alloc((size_t)t.domain_l + 1);
      I.nb_l = (t.domain_l + dev::kScanChunk - 1) / dev::kScanChunk;
      I.part_u32.alloc(I.nb_l);
      I.part_u64.alloc(I.nb_l);
      HBX_CUDA(cudaMemsetAsync(I.cnt_l.p, 0, (size_t)t.domain_l * 4, st));
      HBX_CUDA(cudaMemsetAsync(I.cur_l.p, 0, (size_t)t.domain_l * 4, st));
      dev::Rule d = t;
      d.key_l = I.key_l.p;
      d.cnt_l = I.cnt_l.p;
      d.off_l = I.off_l.p;
      d.cur_l = I.cur_l.p;
      d.item_off = I.item_off.p;
      d.sorted_l = I.sorted_l.p;
      B.h_rules.push_back(d);
    }
  const uint32_t ni = (uint32_t)B.inst.size();
  B.d_rules.alloc(ni);
  HBX_CUDA(cudaMemcpyAsync(B.d_rules.p, B.h_rules.data(), ni * sizeof(dev::Rule),
                           cudaMemcpyHostToDevice, st));
  B.d_base.alloc(ni + 1);
  B.d_cmp.alloc(ni);
  B.d_ctr.alloc(1);
  HBX_CUDA(cudaMemsetAsync(B.d_cmp.p, 0, ni * 8ull, st));
  HBX_CUDA(cudaMemsetAsync(B.d_ctr.p, 0, sizeof(dev::Counters), st));
  for (uint32_t i = 0; i < ni; i++) {
    const Inst& I = B.inst[i];
    const dev::Rule& t = B.h_rules[i];
    const uint32_t row0 = B.base[I.req], n = B.ents[I.req].n();
    if (n) k_keys<<<grid_for(n, C->n_sm), 256, 0, st>>>(B.d_rules.p, i, B.side_l, row0, n, I.key_l.p);
    dev::k_scan_partial_u32<<<I.nb_l, 1024, 0, st>>>(I.cnt_l.p, t.domain_l, I.part_u32.p);
    dev::k_scan_top_u32<<<1, 1024, 0, st>>>(I.part_u32.p, I.nb_l);
    dev::k_scan_final_u32<<<I.nb_l, 1024, 0, st>>>(I.cnt_l.p, t.domain_l, I.part_u32.p, I.off_l.p);
    dev::k_items_partial<<<I.nb_l, 1024, 0, st>>>(B.d_rules.p, i, S->tile_right, I.part_u64.p,
                                                  B.d_cmp.p + i);
    dev::k_scan_top_u64<<<1, 1024, 0, st>>>(I.part_u64.p, I.nb_l);
    dev::k_items_final<<<I.nb_l, 1024, 0, st>>>(B.d_rules.p, i, S->tile_right, I.part_u64.p);
    if (n) k_scatter_left<<<grid_for(n, C->n_sm), 256, 0, st>>>(B.d_rules.p, i, row0, n, I.key_l.p);
  }
  dev::k_rule_base<<<1, 32, 0, st>>>(B.d_rules.p, ni, B.d_base.p, nullptr);
  check_launch("serving batch join");

  B.capacity = std::max<uint64_t>(1 << 16, 2ull * N);
  B.out_l.alloc(B.capacity);
  B.out_r.alloc(B.capacity);
  if (S->any_multi_rule) {
    uint64_t slots = 1 << 16;
    while (slots < 2 * B.capacity) slots *= 2;
    B.seen.alloc(slots);
  }
  B.cmp_first = 0;
  B.h_ctr.ensure(sizeof(dev::Counters) + 8 + 8ull * ni);
}

// The evaluation launch of a batch and the copy of its counters.
void launch_eval(hbx_server* S, Slot& B) {
  cudaStream_t st = B.st;
  const uint32_t ni = (uint32_t)B.inst.size();
  if (B.seen.p) HBX_CUDA(cudaMemsetAsync(B.seen.p, 0xff, B.seen.n * 8, st));
  dev::EvalParams P{};
  P.L = B.side_l;
  P.R = S->side_r;
  P.rules = B.d_rules.p;
  P.n_rules = ni;
  P.n_symbols = S->n_symbols;
  P.rule_item_base = B.d_base.p;
  P.n_seg = 0;
  P.tile_right = S->tile_right;
  dev::set_layout(&P, S->wl, B.shape, B.peq.p);
  P.out_l = B.out_l.p;
  P.out_r = B.out_r.p;
  P.capacity = B.capacity;
  P.ctr = B.d_ctr.p;
  P.watchdog_cycles = 0;
  P.seen = B.seen.p;
  P.seen_mask = B.seen.p ? B.seen.n - 1 : 0;
  const int grid = S->ctx->n_sm * S->blocks_per_sm;
  dev::eval_kernel(S->variant, false, B.shape.w)<<<grid, kThreads, S->smem_bytes, st>>>(P);
  check_launch("serving k_eval");
  uint8_t* h = (uint8_t*)B.h_ctr.p;
  HBX_CUDA(cudaMemcpyAsync(h, B.d_ctr.p, sizeof(dev::Counters), cudaMemcpyDeviceToHost, st));
  HBX_CUDA(cudaMemcpyAsync(h + sizeof(dev::Counters), B.d_base.p + ni, 8, cudaMemcpyDeviceToHost, st));
  HBX_CUDA(cudaMemcpyAsync(h + sizeof(dev::Counters) + 8, B.d_cmp.p, 8ull * ni,
                           cudaMemcpyDeviceToHost, st));
  HBX_CUDA(cudaEventRecord(B.ev_eval, st));
  B.state = 1;
}

// Delivers a request whose rows have all come back (caller holds the lock).
void deliver(hbx_server* S, Request* r, Clock::time_point now) {
  std::sort(r->pairs.begin(), r->pairs.end());
  Result res;
  res.id = r->id;
  res.plan = r->plan;
  res.status = r->status;
  if (r->status == HBX_OK) {
    res.l.reserve(r->pairs.size());
    res.r.reserve(r->pairs.size());
    for (auto& pr : r->pairs) {
      res.l.push_back(pr.first);
      res.r.push_back(pr.second);
    }
  }
  res.comparisons = r->comparisons;
  res.ms_queued = r->admitted ? ms_between(r->t_submit, r->t_admit) : 0.0;
  res.ms_total = ms_between(r->t_submit, now);
  res.batch_requests = r->batch_requests;
  res.batch_id = r->batch_id;
  S->done.push_back(std::move(res));
  S->st.requests_done++;
  for (size_t k = 0; k < S->active.size(); k++)
    if (S->active[k].get() == r) {
      S->active.erase(S->active.begin() + (long)k);
      break;
    }
  S->cv_done.notify_all();
}

// A batch failed: its requests fail (their other chunks are not dispatched).
void fail_batch(hbx_server* S, Slot& B, hbx_status status, const std::string& why) {
  const auto now = Clock::now();
  std::lock_guard<std::mutex> lock(S->mu);
  S->err = why;
  for (auto& e : B.ents) {
    Request* r = e.r;
    r->status = status;
    r->next = r->n;
    r->outstanding--;
  }
  for (auto& e : B.ents)
    if (e.r->outstanding == 0) {
      Request* r = e.r;
      e.r = nullptr;
      bool live = false;
      for (auto& a : S->active) live = live || a.get() == r;
      if (live) deliver(S, r, now);
    }
  S->in_use -= B.est;
}

// Advances one batch; returns true when something happened.
bool progress(hbx_server* S, Slot& B) {
  if (B.state == 1) {
    const cudaError_t q = cudaEventQuery(B.ev_eval);
    if (q == cudaErrorNotReady) return false;
    HBX_CUDA(q);
    const uint8_t* h = (const uint8_t*)B.h_ctr.p;
    dev::Counters c;
    std::memcpy(&c, h, sizeof c);
    unsigned long long total_items = 0;
    std::memcpy(&total_items, h + sizeof c, 8);
    if (c.items_done != total_items)
      fail(HBX_ERR_CUDA, "serving batch finished " + std::to_string(c.items_done) + " of " +
                             std::to_string(total_items) + " work items");
    if (c.out_count > B.capacity || c.seen_overflow) {
      // grow and evaluate again (the join is unchanged)
      PoolScope scope(S->ctx->pool, B.st);
      uint64_t cap = B.capacity;
      const uint64_t need = c.seen_overflow ? std::max<uint64_t>(c.out_count, c.passes) : c.out_count;
      while (cap < need || cap == B.capacity) cap *= 2;
      B.capacity = cap;
      B.out_l.alloc(cap);
      B.out_r.alloc(cap);
      if (B.seen.p) {
        uint64_t slots = B.seen.n;
        while (slots < 2 * cap) slots *= 2;
        B.seen.alloc(slots);
      }
      HBX_CUDA(cudaMemsetAsync(B.d_ctr.p, 0, sizeof(dev::Counters), B.st));
      launch_eval(S, B);
      return true;
    }
    const uint64_t n = c.out_count;
    B.h_out.ensure(std::max<uint64_t>(8 * n, 16));
    uint32_t* ho = (uint32_t*)B.h_out.p;
    if (n) {
      HBX_CUDA(cudaMemcpyAsync(ho, B.out_l.p, 4 * n, cudaMemcpyDeviceToHost, B.st));
      HBX_CUDA(cudaMemcpyAsync(ho + n, B.out_r.p, 4 * n, cudaMemcpyDeviceToHost, B.st));
    }
    HBX_CUDA(cudaEventRecord(B.ev_out, B.st));
    B.capacity = n;  // from here on: the number of pairs copied back
    B.state = 2;
    return true;
  }
  if (B.state == 2) {
    const cudaError_t q = cudaEventQuery(B.ev_out);
    if (q == cudaErrorNotReady) return false;
    HBX_CUDA(q);
    float ms = 0;
    HBX_CUDA(cudaEventElapsedTime(&ms, B.ev_start, B.ev_eval));
    const uint64_t n = B.capacity;
    const uint32_t* ho = (const uint32_t*)B.h_out.p;
    const size_t nq = B.ents.size();
    const uint8_t* h = (const uint8_t*)B.h_ctr.p;
    const auto now = Clock::now();
    std::lock_guard<std::mutex> lock(S->mu);
    for (uint64_t k = 0; k < n; k++) {
      const uint32_t l = ho[k];
      const size_t q = (size_t)(std::upper_bound(B.base.begin(), B.base.end(), l) - B.base.begin()) - 1;
      const Entry& e = B.ents[q];
      e.r->pairs.emplace_back(l - B.base[q] + e.r0, ho[n + k]);
    }
    uint64_t cmp_all = 0;
    for (size_t i = 0; i < B.inst.size(); i++) {
      uint64_t v;
      std::memcpy(&v, h + sizeof(dev::Counters) + 8 + 8 * i, 8);
      B.ents[B.inst[i].req].r->comparisons += v;
      cmp_all += v;
    }
    for (auto& e : B.ents) {
      Request* r = e.r;
      r->batch_requests = std::max<uint32_t>(r->batch_requests, (uint32_t)nq);
      r->batch_id = B.batch_id;
      r->outstanding--;
      if (r->outstanding == 0 && r->next == r->n) deliver(S, r, now);
    }
    S->st.batches++;
    S->st.rows += B.n_rows;
    S->st.pair_comparisons += cmp_all;
    S->st.n_pairs += n;
    S->st.ms_device += ms;
    S->in_use -= B.est;
    B.release();
    return true;
  }
  return false;
}

// Requests waiting longer than this go ahead of shorter ones.
constexpr double kAgingMs = 200.0;

void worker_loop(hbx_server* S) {
  cudaSetDevice(S->ctx->device);
  const uint64_t max_rows = S->opts.max_batch_rows > 0 ? (uint64_t)S->opts.max_batch_rows : 4096u;
  for (;;) {
    bool progressed = false;
    for (auto& sp : S->slots) {
      Slot& B = *sp;
      if (B.state == 0) continue;
      try {
        progressed |= progress(S, B);
      } catch (const Error& e) {
        cudaStreamSynchronize(B.st);
        fail_batch(S, B, e.status, e.what());
        B.release();
        progressed = true;
      }
    }
    Slot* idle = nullptr;
    for (auto& sp : S->slots)
      if (sp->state == 0) {
        idle = sp.get();
        break;
      }
    std::vector<Entry> ents;
    uint64_t est = 0;
    {
      std::unique_lock<std::mutex> lock(S->mu);
      if (idle) {
        // shortest remaining work first (rows not yet dispatched), except that
        // requests waiting past kAgingMs go first, oldest first
        const auto now = Clock::now();
        std::vector<Request*> cand;
        for (auto& r : S->active)
          if (r->next < r->n) cand.push_back(r.get());
        std::sort(cand.begin(), cand.end(), [&](const Request* x, const Request* y) {
          const bool ax = ms_between(x->t_submit, now) > kAgingMs;
          const bool ay = ms_between(y->t_submit, now) > kAgingMs;
          if (ax != ay) return ax;
          if (ax) return x->t_submit < y->t_submit;
          const uint32_t rx = x->n - x->next, ry = y->n - y->next;
          if (rx != ry) return rx < ry;
          return x->t_submit < y->t_submit;
        });
        uint64_t rows = 0;
        for (Request* r : cand) {
          const uint32_t take = (uint32_t)std::min<uint64_t>(r->n - r->next, max_rows - rows);
          if (take == 0) break;
          const uint64_t e = estimate(S, r->rows, r->plan, r->next, r->next + take);
          if (S->in_use + est + e > S->budget && !(S->in_use == 0 && ents.empty())) break;
          ents.push_back(Entry{r, r->next, r->next + take});
          r->next += take;
          r->outstanding++;
          if (!r->admitted) {
            r->admitted = true;
            r->t_admit = now;
          }
          rows += take;
          est += e;
        }
        S->in_use += est;
        S->peak = std::max(S->peak, S->in_use);
        S->st.peak_bytes = S->peak;
      }
      bool busy = false;
      for (auto& sp : S->slots) busy = busy || sp->state != 0;
      if (ents.empty() && !busy) {
        if (S->stopping && S->active.empty()) return;
        if (!progressed) S->cv_work.wait_for(lock, std::chrono::milliseconds(2));
        continue;
      }
    }
    if (!ents.empty()) {
      Slot& B = *idle;
      B.ents = std::move(ents);
      B.est = est;
      B.batch_id = S->next_batch++;
      try {
        launch_batch(S, B);
        launch_eval(S, B);
      } catch (const Error& e) {
        cudaStreamSynchronize(B.st);
        fail_batch(S, B, e.status, e.what());
        B.release();
      }
      progressed = true;
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

}  // namespace
}  // namespace srv
}  // namespace hbx

// ============================================================== C ABI
extern "C" {

hbx_status hbx_serve_open(hbx_ctx* ctx, const hbx_plan* const* plans, int32_t n_plans,
                          const hbx_table* right, const hbx_serve_opts* opts, hbx_server** out) {
  if (!ctx || !plans || n_plans <= 0 || !right || !out) return HBX_ERR_INVALID_ARG;
  *out = nullptr;
  auto S = std::make_unique<hbx_server>();
  S->ctx = ctx;
  S->opts.struct_size = sizeof(hbx_serve_opts);
  if (opts) {
    if (opts->struct_size != sizeof(hbx_serve_opts)) return HBX_ERR_INVALID_ARG;
    if (opts->max_inflight < 0 || opts->max_batch_rows < 0 || opts->eval_variant < 0 ||
        opts->eval_variant > 2 || opts->tile_right < 0)
      return HBX_ERR_INVALID_ARG;
    S->opts = *opts;
  }
  try {
    HBX_CUDA(cudaSetDevice(ctx->device));
    open_server(S.get(), plans, n_plans, right);
  } catch (const Error& e) {
    ctx->err = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    ctx->err = "host out of memory";
    return HBX_ERR_OOM;
  }
  hbx_server* s = S.get();
  s->worker = std::thread([s] { worker_loop(s); });
  *out = S.release();
  return HBX_OK;
}

hbx_status hbx_serve_submit(hbx_server* s, uint64_t req_id, int32_t plan, const hbx_columns* left) {
  if (!s || !left) return HBX_ERR_INVALID_ARG;
  auto r = std::make_unique<Request>();
  r->id = req_id;
  r->plan = plan;
  r->t_submit = Clock::now();
  uint64_t need = 0;
  try {
    if (plan < 0 || plan >= (int32_t)s->plan_rules.size()) fail(HBX_ERR_INVALID_ARG, "no such plan");
    r->rows = table_from_columns(left);
    if (r->rows.n_cols() < s->left_cols_min)
      fail(HBX_ERR_INVALID_ARG, "the request has fewer columns than its plans read");
    if (r->rows.n_rows > (int64_t)(1u << 30)) fail(HBX_ERR_UNSUPPORTED, "request above 2^30 rows");
    r->n = (uint32_t)r->rows.n_rows;
    // the largest chunk the request can be dispatched in must fit the budget
    const uint64_t max_rows = s->opts.max_batch_rows > 0 ? (uint64_t)s->opts.max_batch_rows : 4096u;
    need = estimate(s, r->rows, plan, 0, (uint32_t)std::min<uint64_t>(r->n, max_rows));
  } catch (const Error& e) {
    std::lock_guard<std::mutex> lock(s->mu);
    s->err = e.what();
    return e.status;
  }
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->stopping) {
    s->err = "the server is closing";
    return HBX_ERR_INVALID_ARG;
  }
  if (need > s->budget) {
    s->err = "request needs " + std::to_string(need) + " bytes of device memory; the budget is " +
             std::to_string(s->budget);
    return HBX_ERR_CAPACITY;
  }
  Request* raw = r.get();
  s->active.push_back(std::move(r));
  if (raw->n == 0) {
    deliver(s, raw, Clock::now());  // nothing to evaluate
  } else {
    s->cv_work.notify_one();
  }
  return HBX_OK;
}

hbx_status hbx_serve_poll(hbx_server* s, int32_t timeout_ms, hbx_serve_result* out) {
  if (!s || !out) return HBX_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lock(s->mu);
  auto ready = [&] { return !s->done.empty(); };
  if (timeout_ms < 0)
    s->cv_done.wait(lock, ready);
  else if (!s->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), ready))
    return HBX_ERR_TIMEOUT;
  s->current = std::move(s->done.front());
  s->done.pop_front();
  const Result& r = s->current;
  out->req_id = r.id;
  out->status = r.status;
  out->plan = r.plan;
  out->n_pairs = r.l.size();
  out->l_row = r.l.data();
  out->r_row = r.r.data();
  out->pair_comparisons = r.comparisons;
  out->ms_queued = r.ms_queued;
  out->ms_total = r.ms_total;
  out->batch_requests = r.batch_requests;
  out->batch_id = r.batch_id;
  return HBX_OK;
}

hbx_status hbx_serve_get_stats(const hbx_server* s, hbx_serve_stats* out) {
  if (!s || !out) return HBX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(const_cast<hbx_server*>(s)->mu);
  *out = s->st;
  return HBX_OK;
}

hbx_status hbx_serve_close(hbx_server* s) {
  if (!s) return HBX_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stopping = true;
    s->cv_work.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(s->ctx->device);
  for (auto& sl : s->slots) cudaStreamSynchronize(sl->st);
  delete s;
  return HBX_OK;
}

const char* hbx_serve_last_error(const hbx_server* s) {
  if (!s) return "";
  std::lock_guard<std::mutex> lock(const_cast<hbx_server*>(s)->mu);
  return s->err.c_str();
}

}  // extern "C"
