// static_scratch.cu -- hbx_block_static: the blocking pipeline with no device
// memory allocation of its own.
//
// Some callers cannot call cudaMalloc: an application whose device memory is
// carved up up-front by another runtime or a memory pool it does not share,
// a process running under a fixed device-memory budget, or a latency-critical
// loop that cannot afford cudaMalloc/cudaFree, which may synchronize the whole
// device.  For them this entry point runs the same kernels as hbx_block (the
// device encoder of the tables, the equality join, the Jaro-Winkler
// evaluation and the duplicate set), but every buffer they need -- the
// columns the plan reads, the encoded tables and the encoder's temporaries,
// the join's histograms, offsets and sorted rows, the counters and the
// duplicate set -- is carved out of one file-scope device array of
// kStaticScratchBytes (64 MiB).  The caller passes
// the tables and the output buffers; nothing here calls cudaMalloc, cudaFree,
// or any other allocating routine (no streams, events or graphs are created).
//
// Costs and limits, stated for the caller:
//   * every GPU that loads libhbx.so holds the 64 MiB array until the process
//     exits;
//   * an input whose columns, encoding, join state and duplicate set do not
//     fit is refused with HBX_ERR_INVALID_ARG (the encoding is refused while
//     the encoder places it, the rest before any join work);
//   * every call shares the one array and keeps the previous call's contents
//     (whatever must start at zero is cleared by the call itself), so calls
//     whose work overlaps on the GPU -- from several host threads, or on
//     several streams without ordering between them -- race and corrupt each
//     other;
//   * the first call on a device looks up the array's device address (once
//     per device and CUDA context, with that device current).  A later call
//     that finds another context current on the device (after
//     cudaDeviceReset, say, which reloads the module and may move the array)
//     looks it up again;
//   * a call cannot be captured into a CUDA graph: it copies from pageable
//     host memory and synchronizes its stream.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "device_buffers.h"
#include "encode.h"
#include "hbx_core.h"
#include "ingest.h"
#include "kernels.cuh"

namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;
constexpr int kMaxDevices = 64;

// The scratch.  In host code this name is only a stand-in for the symbol, not
// a device address: kernels get the address cudaGetSymbolAddress returns.
static __device__ __align__(256) unsigned char g_scratch[kStaticScratchBytes];

// The array's address on each device, with the id of the CUDA context it
// was looked up in (0: the id could not be read; the address is then looked
// up on every call, which allocates nothing once the module is loaded).
struct ScratchAddr {
  unsigned char* addr = nullptr;
  unsigned long long ctx_id = 0;
};
std::mutex g_mu;
ScratchAddr g_scratch_addr[kMaxDevices];
thread_local std::string g_static_err;

#define HBX_STATIC_CUDA(expr)                                                              \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      ::hbx::fail(HBX_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));       \
  } while (0)

// Id of the current CUDA context (cuCtxGetCurrent + cuCtxGetId through the
// runtime's driver entry points, so no link against the driver library); 0
// when it cannot be read.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool resolved = false;
  if (!resolved) {  // under g_mu
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = (GetId)f;
    resolved = true;
  }
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c) return 0;
  if (get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the scratch on `device`, which is current: looked up
// once per device and context.
unsigned char* scratch_on(int device) {
  std::lock_guard<std::mutex> lock(g_mu);
  const unsigned long long ctx = current_context_id();
  ScratchAddr& a = g_scratch_addr[device];
  if (!a.addr || ctx == 0 || a.ctx_id != ctx) {
    void* p = nullptr;
    HBX_STATIC_CUDA(cudaGetSymbolAddress(&p, g_scratch));
    a.addr = (unsigned char*)p;
    a.ctx_id = ctx;
  }
  return a.addr;
}

// Bump allocation of 256-byte aligned pieces of the scratch.  A first pass
// with base == nullptr only measures.
struct Carve {
  unsigned char* base;
  size_t used = 0;
  template <class T>
  T* take(size_t count) {
    used = (used + 255) / 256 * 256;
    T* p = base ? (T*)(base + used) : nullptr;
    used += std::max<size_t>(count, 1) * sizeof(T);
    return p;
  }
};

struct Layout {
  hbx::dev::Side L{}, R{};
  std::vector<hbx::dev::Rule> rules;
  std::vector<uint32_t> nb, nb_l;
  hbx::dev::Rule* d_rules = nullptr;
  unsigned long long* rule_base = nullptr;
  hbx::dev::Counters* ctr = nullptr;
  unsigned long long* seen = nullptr;
  unsigned long long seen_slots = 0;
  uint32_t* part_u32 = nullptr;
  unsigned long long* part_u64 = nullptr;
  hbx::dev::WarpLayout wl{};
  hbx::dev::PeqShape shape{};
  uint32_t* peq = nullptr;
  uint32_t tile_right = 128;
};

// Places the join state, the Peq tables and the counters after the encoded
// tables (c.used starts past them); with c.base == nullptr it only measures.
// The duplicate set (plans with several rules) is placed last by place_seen.
void place(Carve& c, const hbx::Encoded& E, size_t smem_cap, Layout* Y) {
  namespace dev = hbx::dev;
  const uint32_t nL = (uint32_t)E.L.n_rows, nR = (uint32_t)E.R.n_rows;
  uint32_t max_len = 1;
  Y->rules.assign(E.rules.size(), dev::Rule{});
  Y->nb.assign(E.rules.size(), 0);
  Y->nb_l.assign(E.rules.size(), 0);
  uint32_t max_nb = 1;
  for (size_t r = 0; r < E.rules.size(); r++) {
    const hbx::RuleEnc& re = E.rules[r];
    dev::Rule& d = Y->rules[r];
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
      max_len = std::max(max_len, E.L.str_maxlen[(size_t)re.sim_slot_l[s]]);
    }
    d.domain = (uint32_t)re.domain;
    const bool split = !re.sim_slot_l.empty() &&
                       re.domain * dev::kWordClasses <= (uint64_t)hbx::kMaxKeyDomain * 4;
    d.n_wclass = split ? dev::kWordClasses : 1u;
    d.wclass_slot = split ? (uint32_t)re.sim_slot_l[0] : 0u;
    d.domain_l = d.n_wclass * d.domain;
    dev::make_singleton(&d);
    d.key_l = c.take<uint32_t>(nL);
    d.key_r = c.take<uint32_t>(nR);
    d.cnt_l = c.take<uint32_t>(d.domain_l);
    d.cnt_r = c.take<uint32_t>(d.domain);
    d.off_l = c.take<uint32_t>(d.domain_l);
    d.off_r = c.take<uint32_t>(d.domain);
    d.cur_l = c.take<uint32_t>(d.domain_l);
    d.cur_r = c.take<uint32_t>(d.domain);
    d.item_off = c.take<unsigned long long>((size_t)d.domain_l + 1);
    d.sorted_l = c.take<uint32_t>(nL);
    d.sorted_r = c.take<uint32_t>((size_t)nR + 4);
    d.sorted_meta_r = d.n_sim ? c.take<dev::StrMeta>(nR) : nullptr;
    Y->nb[r] = (d.domain + dev::kScanChunk - 1) / dev::kScanChunk;
    Y->nb_l[r] = (d.domain_l + dev::kScanChunk - 1) / dev::kScanChunk;
    max_nb = std::max(max_nb, std::max(Y->nb[r], Y->nb_l[r]));
  }
  Y->wl = dev::warp_layout_fit(Y->tile_right, smem_cap);
  if ((size_t)Y->wl.warp_words * 4 * dev::kWarpsPerCta > smem_cap)
    hbx::fail(HBX_ERR_INVALID_ARG, "tile_right too large");
  Y->shape = dev::peq_shape(max_len, E.n_symbols);
  Y->peq = c.take<uint32_t>(std::max<size_t>((size_t)E.L.str_maxlen.size() * nL * Y->shape.tab_words, 4));
  Y->part_u32 = c.take<uint32_t>(max_nb);
  Y->part_u64 = c.take<unsigned long long>(max_nb);
  Y->d_rules = c.take<dev::Rule>(E.rules.size());
  Y->rule_base = c.take<unsigned long long>(E.rules.size() + 1);
  Y->ctr = c.take<dev::Counters>(1);
}

// Slots of the duplicate set: twice the distinct pairs the call can report
// (at most the caller's capacity, and at most the pairs the partitions hold),
// rounded up to a power of two, but no more than what is left of the
// scratch after the other buffers (`used` bytes).  A set that fills up
// stops the run with HBX_ERR_CAPACITY (seen_overflow).
unsigned long long seen_slots_for(const hbx::Encoded& E, uint64_t capacity, size_t used) {
  if (E.rules.size() <= 1) return 0;
  const uint64_t pairs = std::min<uint64_t>(capacity, E.pairs_covered);
  unsigned long long slots = 1024;
  while (slots < 2 * pairs) slots *= 2;
  const size_t left = kStaticScratchBytes > used + 256 ? kStaticScratchBytes - used - 256 : 0;
  while (slots > 1024 && slots * 8 > left) slots /= 2;
  return slots;
}

void place_seen(Carve& c, Layout* Y, unsigned long long slots) {
  Y->seen_slots = slots;
  Y->seen = slots ? c.take<unsigned long long>(slots) : nullptr;
}

void run_static(int device, const hbx_plan* plan, const hbx_table* left, const hbx_table* right,
                uint64_t n_partitions, int64_t prefix_idx, hbx_pairs* out, cudaStream_t st,
                hbx_stats* stats) {
  namespace dev = hbx::dev;
  int n_dev = 0;
  HBX_STATIC_CUDA(cudaGetDeviceCount(&n_dev));
  if (device < 0 || device >= n_dev || device >= kMaxDevices)
    hbx::fail(HBX_ERR_INVALID_ARG, "no such CUDA device");
  if (prefix_idx != INT_MAX && (prefix_idx < 0 || prefix_idx > INT_MAX))
    hbx::fail(HBX_ERR_INVALID_ARG, "prefix_idx out of range");
  if (out->capacity && (!out->l_row || !out->r_row))
    hbx::fail(HBX_ERR_INVALID_ARG, "null output pointer");
  int n_sm = 0, smem_optin = 0;
  HBX_STATIC_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device));
  HBX_STATIC_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  const size_t smem_cap = std::min<size_t>((size_t)smem_optin, 200 * 1024);

  int prev = 0;
  HBX_STATIC_CUDA(cudaGetDevice(&prev));
  HBX_STATIC_CUDA(cudaSetDevice(device));
  struct Restore {
    int d;
    ~Restore() { cudaSetDevice(d); }
  } restore{prev};
  unsigned char* const base = scratch_on(device);
  // Once work is queued on the scratch, a failure waits for the stream before
  // it returns, so the scratch is free again when the call returns.
  struct DrainOnError {
    cudaStream_t st;
    bool armed = false;
    ~DrainOnError() {
      if (armed) cudaStreamSynchronize(st);
    }
  } drain{st};

  // The tables are encoded on the device, into the front of the scratch: the
  // device encoder's buffers come from an arena over it (the columns the plan
  // reads, then the encoded sides; an input they do not fit is refused there)
  hbx::Encoded E = hbx::encode_schema(plan->p, left->t, right->t, n_partitions, prefix_idx);
  hbx::DevArena arena;
  arena.base = base;
  arena.cap = kStaticScratchBytes;
  hbx::SideBufs SL, SR;
  uint64_t h2d = 0;
  {
    hbx::ArenaScope in_scratch(&arena);
    std::string why;
    drain.armed = true;
    if (!hbx::device_encode(left, right, &E, &SL, &SR, n_sm, st, &h2d, &why, /*pin=*/false))
      hbx::fail(HBX_ERR_UNSUPPORTED, "the device encoder cannot take this input: " + why);
  }
  const uint32_t nL = (uint32_t)E.L.n_rows, nR = (uint32_t)E.R.n_rows;
  Layout Y;
  Y.L = dev::Side{SL.bucket.p, SL.eq.p, SL.comp.p, SL.arena.p, SL.meta.p, nL};
  Y.R = dev::Side{SR.bucket.p, SR.eq.p, SR.comp.p, SR.arena.p, SR.meta.p, nR};

  // the join state, Peq tables and counters after the encoded tables
  Carve measure{nullptr};
  measure.used = arena.used;
  place(measure, E, smem_cap, &Y);
  if (measure.used > kStaticScratchBytes)
    hbx::fail(HBX_ERR_INVALID_ARG,
              "input needs " + std::to_string(measure.used) + " bytes of device scratch for its "
              "encoding and join state; the static scratch holds " +
              std::to_string(kStaticScratchBytes));
  const unsigned long long seen_slots = seen_slots_for(E, out->capacity, measure.used);
  place_seen(measure, &Y, seen_slots);
  if (measure.used > kStaticScratchBytes)
    hbx::fail(HBX_ERR_INVALID_ARG,
              "input needs " + std::to_string(measure.used) + " bytes of device scratch; the "
              "static scratch holds " + std::to_string(kStaticScratchBytes));
  Carve carve{base};
  carve.used = arena.used;
  place(carve, E, smem_cap, &Y);
  place_seen(carve, &Y, seen_slots);

  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (bytes) HBX_STATIC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    h2d += bytes;
  };
  up(Y.d_rules, Y.rules.data(), Y.rules.size() * sizeof(dev::Rule));

  // counters, histograms, cursors and the duplicate set start from zero/empty
  HBX_STATIC_CUDA(cudaMemsetAsync(Y.ctr, 0, sizeof(dev::Counters), st));
  if (Y.seen) HBX_STATIC_CUDA(cudaMemsetAsync(Y.seen, 0xff, Y.seen_slots * 8, st));
  auto grid_for = [&](uint32_t n) {
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)n_sm * 8));
  };
  for (size_t r = 0; r < Y.rules.size(); r++) {
    const dev::Rule& d = Y.rules[r];
    HBX_STATIC_CUDA(cudaMemsetAsync(d.cnt_l, 0, d.domain_l * 4, st));
    HBX_STATIC_CUDA(cudaMemsetAsync(d.cnt_r, 0, d.domain * 4, st));
    HBX_STATIC_CUDA(cudaMemsetAsync(d.cur_l, 0, d.domain_l * 4, st));
    HBX_STATIC_CUDA(cudaMemsetAsync(d.cur_r, 0, d.domain * 4, st));
    const uint32_t ru = (uint32_t)r;
    if (nL) dev::k_keys_hist<<<grid_for(nL), 256, 0, st>>>(Y.L, Y.d_rules, ru, 0);
    if (nR) dev::k_keys_hist<<<grid_for(nR), 256, 0, st>>>(Y.R, Y.d_rules, ru, 1);
    dev::k_scan_partial_u32<<<Y.nb_l[r], 1024, 0, st>>>(d.cnt_l, d.domain_l, Y.part_u32);
    dev::k_scan_top_u32<<<1, 1024, 0, st>>>(Y.part_u32, Y.nb_l[r]);
    dev::k_scan_final_u32<<<Y.nb_l[r], 1024, 0, st>>>(d.cnt_l, d.domain_l, Y.part_u32, d.off_l);
    dev::k_scan_partial_u32<<<Y.nb[r], 1024, 0, st>>>(d.cnt_r, d.domain, Y.part_u32);
    dev::k_scan_top_u32<<<1, 1024, 0, st>>>(Y.part_u32, Y.nb[r]);
    dev::k_scan_final_u32<<<Y.nb[r], 1024, 0, st>>>(d.cnt_r, d.domain, Y.part_u32, d.off_r);
    dev::k_items_partial<<<Y.nb_l[r], 1024, 0, st>>>(Y.d_rules, ru, Y.tile_right, Y.part_u64,
                                                     &Y.ctr->comparisons);
    dev::k_scan_top_u64<<<1, 1024, 0, st>>>(Y.part_u64, Y.nb_l[r]);
    dev::k_items_final<<<Y.nb_l[r], 1024, 0, st>>>(Y.d_rules, ru, Y.tile_right, Y.part_u64);
    if (nL) dev::k_scatter<<<grid_for(nL), 256, 0, st>>>(Y.L, Y.d_rules, ru, 0);
    if (nR) dev::k_scatter<<<grid_for(nR), 256, 0, st>>>(Y.R, Y.d_rules, ru, 1);
  }
  dev::k_rule_base<<<1, 32, 0, st>>>(Y.d_rules, (uint32_t)Y.rules.size(), Y.rule_base, nullptr);
  const uint32_t n_slots = (uint32_t)E.L.str_maxlen.size();
  if (n_slots && nL)
    dev::k_peq_build<<<grid_for((uint32_t)std::min<uint64_t>((uint64_t)n_slots * nL * 32, 1u << 30)), 256, 0,
                       st>>>(Y.L, n_slots, Y.shape, Y.peq);
  HBX_STATIC_CUDA(cudaGetLastError());

  dev::EvalParams P{};
  P.L = Y.L;
  P.R = Y.R;
  P.rules = Y.d_rules;
  P.n_rules = (uint32_t)Y.rules.size();
  P.n_symbols = E.n_symbols;
  P.rule_item_base = Y.rule_base;
  P.n_seg = 0;
  P.tile_right = Y.tile_right;
  dev::set_layout(&P, Y.wl, Y.shape, Y.peq);
  P.out_l = out->l_row;
  P.out_r = out->r_row;
  P.capacity = out->capacity;
  P.ctr = Y.ctr;
  P.seen = Y.seen;
  P.seen_mask = Y.seen ? Y.seen_slots - 1 : 0;
  const size_t smem = (size_t)Y.wl.warp_words * 4 * dev::kWarpsPerCta;
  const dev::EvalKernel kern = dev::eval_kernel(1, false, Y.shape.w);
  {
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    cudaFuncAttributes fa;
    HBX_STATIC_CUDA(cudaFuncGetAttributes(&fa, kern));
    if ((size_t)fa.maxDynamicSharedSizeBytes < smem)
      HBX_STATIC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  int bps = 0;
  HBX_STATIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, dev::kWarpsPerCta * 32, smem));
  kern<<<n_sm * std::max(1, bps), dev::kWarpsPerCta * 32, smem, st>>>(P);
  HBX_STATIC_CUDA(cudaGetLastError());

  dev::Counters c{};
  unsigned long long total_items = 0;
  HBX_STATIC_CUDA(cudaMemcpyAsync(&c, Y.ctr, sizeof c, cudaMemcpyDeviceToHost, st));
  HBX_STATIC_CUDA(cudaMemcpyAsync(&total_items, Y.rule_base + Y.rules.size(), 8,
                                  cudaMemcpyDeviceToHost, st));
  HBX_STATIC_CUDA(cudaStreamSynchronize(st));
  drain.armed = false;  // the stream is idle
  if (c.items_done != total_items) hbx::fail(HBX_ERR_CUDA, "evaluation did not finish its work");
  out->n_required = c.seen_overflow ? std::max<uint64_t>(c.out_count, c.passes) : c.out_count;
  out->n_written = 0;
  if (stats) {
    *stats = hbx_stats{};
    stats->tile_right = Y.tile_right;
    stats->eval_variant = 2;
    stats->pairs_covered = E.pairs_covered;
    stats->pair_comparisons = c.comparisons;
    stats->n_matches = c.out_count;
    stats->fma_ambiguous = c.ambiguous;
    stats->long_string_pairs = c.long_pairs;
    stats->n_tiles = total_items;
    stats->n_partitions_used = E.n_partitions_used;
    stats->jw_word_ops = c.jw_word_ops;
    stats->pairs_scanned = c.scans;
    stats->scan_steps = c.scan_steps;
    stats->scan_word_ops = c.scan_steps * 4ull * 3ull * Y.shape.w;
    stats->scan_words = Y.shape.w;
    stats->scan_warp_steps = c.scan_warp_steps;
    stats->rest_scans = c.rest_scans;
    stats->h2d_bytes = h2d;  // bytes copied to the device by this call
    stats->ingest_on_device = 1;
    stats->n_windows = 1;
  }
  if (c.seen_overflow)
    hbx::fail(HBX_ERR_CAPACITY,
              "the duplicate set (" + std::to_string(Y.seen_slots) + " slots, sized from the "
              "output capacity and the pairs the partitions hold, within the 64 MiB scratch) "
              "filled up; at least " + std::to_string(out->n_required) + " output slots needed");
  if (c.out_count > out->capacity)
    hbx::fail(HBX_ERR_CAPACITY, "output capacity below the match count");
  out->n_written = c.out_count;
}

}  // namespace

extern "C" {

const char* hbx_static_last_error(void) { return g_static_err.c_str(); }

hbx_status hbx_block_static(int device, const hbx_plan* plan, const hbx_table* left,
                            const hbx_table* right, uint64_t n_partitions, int64_t prefix_idx,
                            hbx_pairs* out, void* stream, hbx_stats* stats) {
  if (!plan || !left || !right || !out) return HBX_ERR_INVALID_ARG;
  try {
    run_static(device, plan, left, right, n_partitions, prefix_idx, out, (cudaStream_t)stream,
               stats);
    g_static_err.clear();
    return HBX_OK;
  } catch (const hbx::Error& e) {
    g_static_err = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    g_static_err = "host out of memory";
    return HBX_ERR_OOM;
  } catch (const std::exception& e) {
    g_static_err = e.what();
    return HBX_ERR_INVALID_ARG;
  }
}

}  // extern "C"
