// kernels.cu -- sm_103a kernels of the blocking engine (see kernels.cuh).
#include "kernels.cuh"
#include "bitscan.cuh"

namespace hbx {
namespace dev {

constexpr unsigned kFull = 0xffffffffu;

// =====================================================================
// Join: keys, histograms, scans, scatter
// =====================================================================

__device__ __forceinline__ uint32_t row_key(const Side& S, const Rule& R, uint32_t row) {
  if (R.composite) return (uint32_t)S.comp_codes[(size_t)R.comp_index * S.n_rows + row];
  uint32_t key = S.bucket[row];
  for (uint32_t e = 0; e < R.n_eq; e++)
    key = key * R.radix[e] + (uint32_t)S.eq_codes[(size_t)R.eq_slot[e] * S.n_rows + row];
  return key;
}

__global__ void k_keys_hist(Side S, const Rule* rules, uint32_t rule, int side) {
  const Rule& R = rules[rule];
  uint32_t* keys = side ? R.key_r : R.key_l;
  uint32_t* cnt = side ? R.cnt_r : R.cnt_l;
  const bool split = !side && R.n_wclass > 1;
  for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < S.n_rows;
       row += gridDim.x * blockDim.x) {
    uint32_t k = row_key(S, R, row);
    if (split) k += R.domain * word_class(S.str_meta[(size_t)R.wclass_slot * S.n_rows + row].loc.y);
    keys[row] = k;
    atomicAdd(cnt + k, 1u);
  }
}

// A right row's metadata as the join stores it in sorted_meta_r: the string
// metadata of the rule's first similarity column, with the row's dictionary
// codes of the group's first two extra equality slots in loc.z and loc.w
// (unused words of the string record), so that the filter compares them
// from the staged copy.
__device__ __forceinline__ StrMeta sorted_meta(const Side& S, const Rule& Q, const StrMeta* meta_in,
                                               uint32_t row) {
  StrMeta m = meta_in[row];
  if (Q.n_xslots > 0) m.loc.z = (uint32_t)S.eq_codes[(size_t)Q.xslot[0] * S.n_rows + row];
  if (Q.n_xslots > 1) m.loc.w = (uint32_t)S.eq_codes[(size_t)Q.xslot[1] * S.n_rows + row];
  return m;
}

__global__ void k_scatter(Side S, const Rule* rules, uint32_t rule, int side) {
  const Rule& R = rules[rule];
  if (!R.n_members) return;  // evaluated in another rule's group: no items of its own
  const uint32_t* keys = side ? R.key_r : R.key_l;
  const uint32_t* off = side ? R.off_r : R.off_l;
  uint32_t* cur = side ? R.cur_r : R.cur_l;
  uint32_t* sorted = side ? R.sorted_r : R.sorted_l;
  StrMeta* meta_out = side ? R.sorted_meta_r : nullptr;
  const StrMeta* meta_in = S.str_meta + (size_t)R.sim_r[0] * S.n_rows;
  for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < S.n_rows;
       row += gridDim.x * blockDim.x) {
    const uint32_t k = keys[row];
    const uint32_t pos = off[k] + atomicAdd(cur + k, 1u);
    sorted[pos] = row;
    if (meta_out) meta_out[pos] = sorted_meta(S, R, meta_in, row);
  }
}

// Block-wide exclusive scan of 4 values per thread (1024 threads).
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* s_warp, T* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = (lane < (int)(blockDim.x >> 5)) ? s_warp[lane] : T(0);
    T z = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(kFull, z, o);
      if (lane >= o) z += y;
    }
    s_warp[lane] = z - w;  // exclusive prefix of warp sums
    if (lane == 31) *total = z;
  }
  __syncthreads();
  const T r = s_warp[warp] + x - v;
  __syncthreads();
  return r;
}

__global__ void k_scan_partial_u32(const uint32_t* in, uint32_t n, uint32_t* partial) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk + threadIdx.x * 4u;
  uint32_t v = 0;
  for (int k = 0; k < 4; k++)
    if (base + k < n) v += in[base + k];
  block_excl_scan<uint32_t>(v, s_warp, &s_total);
  if (threadIdx.x == 0) partial[blockIdx.x] = s_total;
}

template <typename T>
__device__ void scan_top(T* partial, uint32_t nb) {
  __shared__ T s_warp[32];
  __shared__ T s_total;
  T carry = 0;
  for (uint32_t b0 = 0; b0 < nb; b0 += blockDim.x) {
    const uint32_t i = b0 + threadIdx.x;
    const T v = i < nb ? partial[i] : T(0);
    const T ex = block_excl_scan<T>(v, s_warp, &s_total);
    if (i < nb) partial[i] = carry + ex;
    carry += s_total;
    __syncthreads();
  }
}

__global__ void k_scan_top_u32(uint32_t* partial, uint32_t nb) { scan_top<uint32_t>(partial, nb); }
__global__ void k_scan_top_u64(unsigned long long* partial, uint32_t nb) {
  scan_top<unsigned long long>(partial, nb);
}

__global__ void k_scan_final_u32(const uint32_t* in, uint32_t n, const uint32_t* partial,
                                 uint32_t* out) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_total;
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk + threadIdx.x * 4u;
  uint32_t v[4];
  uint32_t sum = 0;
  for (int k = 0; k < 4; k++) {
    v[k] = (base + k < n) ? in[base + k] : 0u;
    sum += v[k];
  }
  uint32_t ex = block_excl_scan<uint32_t>(sum, s_warp, &s_total) + partial[blockIdx.x];
  for (int k = 0; k < 4; k++) {
    if (base + k < n) out[base + k] = ex;
    ex += v[k];
  }
}

// Work items of left key j (word class j / D, join key j % D).
__device__ __forceinline__ unsigned long long key_items(const Rule& R, uint32_t j,
                                                        uint32_t tile_right,
                                                        unsigned long long* pairs) {
  const uint32_t nl = R.cnt_l[j], nr = R.cnt_r[j % R.domain];
  *pairs = (unsigned long long)nl * nr;
  if (!nl || !nr) return 0;
  return (unsigned long long)nl * ((nr + tile_right - 1) / tile_right);
}

__global__ void k_items_partial(const Rule* rules, uint32_t rule, uint32_t tile_right,
                                unsigned long long* partial, unsigned long long* comparisons) {
  __shared__ unsigned long long s_warp[32];
  __shared__ unsigned long long s_total;
  const Rule& R = rules[rule];
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk + threadIdx.x * 4u;
  unsigned long long v = 0, pr = 0;
  for (int k = 0; k < 4; k++)
    if (base + k < R.domain_l) {
      unsigned long long p;
      v += key_items(R, (uint32_t)(base + k), tile_right, &p);
      pr += p;
    }
  block_excl_scan<unsigned long long>(v, s_warp, &s_total);
  if (threadIdx.x == 0) partial[blockIdx.x] = s_total;
  __shared__ unsigned long long s_pairs;
  block_excl_scan<unsigned long long>(pr, s_warp, &s_pairs);
  if (threadIdx.x == 0 && s_pairs) atomicAdd(comparisons, s_pairs);
}

__global__ void k_items_final(const Rule* rules, uint32_t rule, uint32_t tile_right,
                              const unsigned long long* partial) {
  __shared__ unsigned long long s_warp[32];
  __shared__ unsigned long long s_total;
  const Rule& R = rules[rule];
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk + threadIdx.x * 4u;
  unsigned long long v[4], sum = 0, p;
  for (int k = 0; k < 4; k++) {
    v[k] = (base + k < R.domain_l) ? key_items(R, (uint32_t)(base + k), tile_right, &p) : 0ull;
    sum += v[k];
  }
  unsigned long long ex =
      block_excl_scan<unsigned long long>(sum, s_warp, &s_total) + partial[blockIdx.x];
  for (int k = 0; k < 4; k++) {
    if (base + k < R.domain_l) R.item_off[base + k] = ex;
    ex += v[k];
    if (base + k + 1 == R.domain_l) R.item_off[R.domain_l] = ex;
  }
}

// Programmatic dependent launch: a kernel launched with the programmatic
// stream serialization attribute (launch_dependent) may start while the
// kernel before it still runs; it waits here before it reads anything that
// kernel writes (every write of the earlier grid is visible after the wait).
// Without the attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Lets the next kernel in the stream start its blocks (they wait in
// pdl_wait); called once every block of this grid has started.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }

// ---- fused join for small key domains (every rule's left key domain at most
// kFusedJoinMaxDomain): one launch for keys + histograms, one for offsets +
// work items, one for the scatter, each covering every rule and both
// tables.  The row kernels run one block row per (rule, table)
// (blockIdx.y = rule, blockIdx.z = table), so the rules' and tables'
// dependent load -> atomic -> store chains run side by side.

// Keys and key histograms of every rule for both tables; histograms of
// domains up to kSharedHistKeys are kept per block in shared memory.
__global__ void k_join_count(Side L, Side R, const Rule* rules) {
  extern __shared__ uint32_t s_cnt[];
  pdl_trigger();
  pdl_wait();  // the histograms are cleared (k_reset)
  const int side = blockIdx.z;
  const Side& S = side ? R : L;
  if ((unsigned long long)blockIdx.x * blockDim.x >= S.n_rows) return;  // whole block
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
  const Rule& Q = rules[blockIdx.y];
  const uint32_t D = side ? Q.domain : Q.domain_l;
  uint32_t* keys = side ? Q.key_r : Q.key_l;
  uint32_t* cnt = side ? Q.cnt_r : Q.cnt_l;
  const bool split = !side && Q.n_wclass > 1;
  const bool sh = D <= kSharedHistKeys;
  if (sh) {
    for (uint32_t k = threadIdx.x; k < D; k += blockDim.x) s_cnt[k] = 0;
    __syncthreads();
  }
  for (uint32_t row = t0; row < S.n_rows; row += stride) {
    uint32_t k = row_key(S, Q, row);
    if (split) k += Q.domain * word_class(S.str_meta[(size_t)Q.wclass_slot * S.n_rows + row].loc.y);
    keys[row] = k;
    atomicAdd(sh ? s_cnt + k : cnt + k, 1u);
  }
  if (sh) {
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < D; k += blockDim.x)
      if (s_cnt[k]) atomicAdd(cnt + k, s_cnt[k]);
  }
}

// The three independent scans of every rule -- row offsets per left key
// (y = 0), row offsets per right key (y = 1), work items per left key with
// the rule's pair-comparison count (y = 2) -- in chunks of kScanChunk keys,
// one block of 1024 threads per (chunk, y, rule), in one launch.  A block
// takes its chunk from a ticket counter of its (y, rule) when it starts,
// publishes the chunk's total (flag bit kScanFlag set) before it reads
// anything of the other chunks, then adds the totals of the chunks before
// its own: those blocks took their tickets earlier, so they are running or
// done, and every wait ends (bounded all the same: a wait that gives up
// counts a watchdog trip, which fails the run).
__device__ __forceinline__ uint32_t join_scan_domain(const Rule& Q, uint32_t y) {
  return y == 1 ? Q.domain : Q.domain_l;
}

// The value of key k (< D): its row count, or its work items (y = 2, with
// the key's pair comparisons added to *pairs).
__device__ __forceinline__ unsigned long long join_scan_value(const Rule& Q, uint32_t y,
                                                              uint32_t tile_right, uint32_t k,
                                                              unsigned long long* pairs) {
  if (y == 2) {
    unsigned long long p = 0;
    const unsigned long long v = key_items(Q, k, tile_right, &p);
    *pairs += p;
    return v;
  }
  return (y == 1 ? Q.cnt_r : Q.cnt_l)[k];
}

constexpr unsigned long long kScanFlag = 1ull << 63;
constexpr uint32_t kScanWaitPolls = 1u << 20;

__global__ void k_join_scan(const Rule* rules, uint32_t tile_right, uint32_t nb,
                            unsigned long long* sync, unsigned long long* comparisons,
                            Counters* ctr) {
  __shared__ unsigned long long s_w64[32];
  __shared__ unsigned long long s_t64, s_base;
  __shared__ uint32_t s_chunk;
  pdl_trigger();
  pdl_wait();  // the histograms are complete (k_join_count)
  const uint32_t y = blockIdx.y, r = blockIdx.z;
  // sync: per (rule, y) nb chunk totals, then one ticket counter each
  unsigned long long* totals = sync + ((size_t)r * 3 + y) * nb;
  unsigned long long* ticket = sync + (size_t)gridDim.z * 3 * nb + (size_t)r * 3 + y;
  if (threadIdx.x == 0) s_chunk = (uint32_t)atomicAdd(ticket, 1ull);
  __syncthreads();
  const uint32_t c = s_chunk;
  const Rule& Q = rules[r];
  const uint32_t D = join_scan_domain(Q, y);
  if ((unsigned long long)c * kScanChunk >= D) return;
  const uint32_t b = c * kScanChunk + threadIdx.x * 4u;
  unsigned long long v[4], pairs = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) v[k] = b + k < D ? join_scan_value(Q, y, tile_right, b + k, &pairs) : 0ull;
  unsigned long long ex = block_excl_scan<unsigned long long>(v[0] + v[1] + v[2] + v[3], s_w64, &s_t64);
  const unsigned long long chunk_total = s_t64;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicExch(totals + c, chunk_total | kScanFlag);
  }
  if (threadIdx.x < 32) {  // the chunks before this one: at most 15
    unsigned long long t = 0;
    for (uint32_t j = threadIdx.x; j < c; j += 32) {
      unsigned long long f = 0;
      uint32_t polls = 0;
      while (!((f = atomicAdd(totals + j, 0ull)) & kScanFlag) && ++polls < kScanWaitPolls)
        __nanosleep(64);
      if (!(f & kScanFlag)) atomicAdd(&ctr->watchdog_trips, 1ull);
      t += f & ~kScanFlag;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(kFull, t, o);
    if (threadIdx.x == 0) s_base = t;
  }
  __syncthreads();
  const unsigned long long base = s_base;
  ex += base;
  if (y == 2) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (b + k < D) Q.item_off[b + k] = ex;
      ex += v[k];
    }
    if ((unsigned long long)(c + 1) * kScanChunk >= D && threadIdx.x == 0)
      Q.item_off[D] = base + chunk_total;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) pairs += __shfl_xor_sync(kFull, pairs, o);
    if ((threadIdx.x & 31) == 0 && pairs) atomicAdd(comparisons, pairs);
  } else {
    uint32_t* off = y == 1 ? Q.off_r : Q.off_l;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (b + k < D) off[b + k] = (uint32_t)ex;
      ex += v[k];
    }
  }
}

// Rows of every rule grouped by key (counting-sort scatter, right rows with
// their first similarity column's metadata), and the rules' item bases.
__global__ void k_join_scatter(Side L, Side R, const Rule* rules, uint32_t n_rules,
                               unsigned long long* rule_base, unsigned long long* items_total) {
  pdl_trigger();
  pdl_wait();  // offsets and work items are complete (k_join_scan)
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0) {
    unsigned long long acc = 0;
    for (uint32_t r = 0; r < n_rules; r++) {
      rule_base[r] = acc;
      // a rule evaluated in another rule's group has no items of its own
      if (rules[r].n_members) acc += rules[r].item_off[rules[r].domain_l];
    }
    rule_base[n_rules] = acc;
    if (items_total) *items_total = acc;
  }
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
  const Rule& Q = rules[blockIdx.y];
  if (!Q.n_members) return;  // evaluated in another rule's group: counted, never enumerated
  if (blockIdx.z == 0) {
    for (uint32_t row = t0; row < L.n_rows; row += stride) {
      const uint32_t k = Q.key_l[row];
      Q.sorted_l[Q.off_l[k] + atomicAdd(Q.cur_l + k, 1u)] = row;
    }
  } else {
    const StrMeta* meta_in = R.str_meta + (size_t)Q.sim_r[0] * R.n_rows;
    for (uint32_t row = t0; row < R.n_rows; row += stride) {
      const uint32_t k = Q.key_r[row];
      const uint32_t pos = Q.off_r[k] + atomicAdd(Q.cur_r + k, 1u);
      Q.sorted_r[pos] = row;
      if (Q.sorted_meta_r) Q.sorted_meta_r[pos] = sorted_meta(R, Q, meta_in, row);
    }
  }
}

__global__ void k_rule_base(const Rule* rules, uint32_t n_rules, unsigned long long* base,
                            unsigned long long* items_total) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    unsigned long long acc = 0;
    for (uint32_t r = 0; r < n_rules; r++) {
      base[r] = acc;
      if (rules[r].n_members) acc += rules[r].item_off[rules[r].domain_l];
    }
    base[n_rules] = acc;
    if (items_total) *items_total = acc;
  }
}

__global__ void k_reset(Counters* ctr, uint32_t* counts, uint64_t n_counts,
                        unsigned long long* seen, uint64_t n_seen, unsigned long long* zero64,
                        uint64_t n_zero64) {
  // launched in stream order (after the previous run); lets the join's first
  // kernel start its blocks early
  pdl_trigger();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  constexpr uint64_t kCtrWords = sizeof(Counters) / 8;
  for (uint64_t i = t0; i < kCtrWords; i += stride) reinterpret_cast<unsigned long long*>(ctr)[i] = 0;
  for (uint64_t i = t0; i < n_counts; i += stride) counts[i] = 0;
  for (uint64_t i = t0; i < n_seen; i += stride) seen[i] = ~0ull;
  for (uint64_t i = t0; i < n_zero64; i += stride) zero64[i] = 0ull;
}

// =====================================================================
// Jaro-Winkler
// =====================================================================

// One symbol row of a Peq table in device memory (plain loads: they need
// fewer registers around the scan than the read-only path's).
template <int S>
__device__ __forceinline__ void load_row(const uint32_t* row, uint32_t (&pe)[S]) {
  if constexpr (S == 1) {
    pe[0] = *row;
  } else if constexpr (S == 2) {
    const uint2 v = *reinterpret_cast<const uint2*>(row);
    pe[0] = v.x;
    pe[1] = v.y;
  } else if constexpr (S == 4) {
    const uint4 v = *reinterpret_cast<const uint4*>(row);
    pe[0] = v.x;
    pe[1] = v.y;
    pe[2] = v.z;
    pe[3] = v.w;
  } else {
    const uint4 v = *reinterpret_cast<const uint4*>(row);
    const uint4 u = *reinterpret_cast<const uint4*>(row + 4);
    pe[0] = v.x;
    pe[1] = v.y;
    pe[2] = v.z;
    pe[3] = v.w;
    pe[4] = u.x;
    pe[5] = u.y;
    pe[6] = u.z;
    pe[7] = u.w;
  }
}

// The reference's Jaro loops (device_func.cuh:71-111) on symbol strings, with
// position 256 usable like any other (the reference's uint16_t idx[256] is
// indexed at 256 there).  Used for pairs whose left string is longer than the
// fast path handles and for the cross-rule duplicate check.
__device__ __noinline__ uint32_t jaro_m_ref(const uint8_t* s1, uint32_t l1, const uint8_t* s2,
                                            uint32_t l2) {
  const uint8_t* s = s1;
  const uint8_t* t = s2;
  uint32_t ls = l1, lt = l2;
  if (l1 > l2) {
    s = s2;
    t = s1;
    ls = l2;
    lt = l1;
  }
  const uint32_t h = (ls + 1u) / 2u;
  uint32_t used[9];
#pragma unroll
  for (int k = 0; k < 9; k++) used[k] = 0;
  uint32_t m = 0;
  for (uint32_t i = 0; i < h; i++) {
    const uint8_t ti = t[i];
    for (uint32_t j = 0; j <= i + h; j++) {
      if (j >= 256) break;
      const uint8_t sj = j < ls ? s[j] : (uint8_t)0;
      if (sj == ti && !((used[j >> 5] >> (j & 31)) & 1u)) {
        used[j >> 5] |= 1u << (j & 31);
        m++;
        break;
      }
    }
  }
  const uint32_t to = (ls + h < lt) ? ls + h : lt;
  for (uint32_t i = h; i < to; i++) {
    const uint8_t ti = t[i];
    for (uint32_t j = i - h; j < ls; j++) {
      if (j > 256) break;
      if (s[j] == ti && !((used[j >> 5] >> (j & 31)) & 1u)) {
        used[j >> 5] |= 1u << (j & 31);
        m++;
        break;
      }
    }
  }
  return m;
}

// Common prefix of two 16-byte-aligned, zero-padded symbol strings, capped at mn.
__device__ __forceinline__ uint32_t prefix_len(const uint8_t* a, const uint8_t* b, uint32_t mn) {
  const uint4* ap = reinterpret_cast<const uint4*>(a);
  const uint4* bp = reinterpret_cast<const uint4*>(b);
  for (uint32_t k = 0; k < mn; k += 16) {
    const uint4 x = __ldg(ap + (k >> 4));
    const uint4 y = __ldg(bp + (k >> 4));
    const uint32_t d[4] = {x.x ^ y.x, x.y ^ y.y, x.z ^ y.z, x.w ^ y.w};
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (d[q]) return min(mn, k + 4u * q + ((uint32_t)(__ffs(d[q]) - 1) >> 3));
  }
  return mn;
}

// Exact threshold decision with the reference's arithmetic.  Returns pass.
__device__ __noinline__ bool jw_exact(uint32_t m, uint32_t ls, uint32_t ll, uint32_t p, float thr,
                                      unsigned long long* ambiguous) {
  float jf;
  if (ls == 0 || ll == 0) {
    jf = (ls == 0 && ll == 0) ? 1.0f : 0.0f;
  } else if (m == 0) {
    jf = 0.0f;
  } else {
    const float md = (float)m;
    const float q = __fadd_rn(__fdiv_rn(md, (float)ls), __fdiv_rn(md, (float)ll));
    const double t = __dadd_rn((double)q, 1.0);
    jf = __double2float_rn(__ddiv_rn(t, 3.0));
  }
  const double j = (double)jf;
  const double a = __dmul_rn(__dsub_rn(1.0, j), (double)p);
  double jw_fma = __fma_rn(a, 0.1, j);
  double jw_sep = __dadd_rn(j, __dmul_rn(a, 0.1));
  jw_fma = jw_fma > 1.0 ? 1.0 : jw_fma;
  jw_sep = jw_sep > 1.0 ? 1.0 : jw_sep;
  const double t = (double)thr;
  const bool fail_fma = jw_fma < t;
  const bool fail_sep = jw_sep < t;
  if (fail_fma != fail_sep) atomicAdd(ambiguous, 1ull);
  return !fail_fma;
}

// Decision from the match count m and the common prefix p: a float estimate
// settles every pair whose JW lies farther than kDecisionMargin from the
// threshold (the estimate's error is below 2e-6); the rest take the exact path.
__device__ __forceinline__ bool jw_decide(uint32_t m, uint32_t ls, uint32_t ll, uint32_t p,
                                          float thr, unsigned long long* ambiguous) {
  const float fm = (float)m;
  const float ja = m ? (__fdividef(fm, (float)ls) + __fdividef(fm, (float)ll) + 1.0f) * (1.0f / 3.0f)
                     : 0.0f;
  const float jwa = ja + (1.0f - ja) * (0.1f * (float)p);
  if (jwa >= thr + kDecisionMargin) return true;
  if (jwa < thr - kDecisionMargin) return false;
  return jw_exact(m, ls, ll, p, thr, ambiguous);
}

// Smallest match count that can still reach the threshold, lowered by a
// safety margin: every m below the returned value gives JW < thr exactly.
// JW >= thr needs j >= (thr - c) / (1 - c) with c = 0.1 p, and
// j = (m/ls + m/ll + 1) / 3.  JW grows with m by at least
// 0.1 * (1/ls) / 3 >= 1.3e-4 per match (c <= 0.9, shorter length ls <= 256 on
// the path that uses this), so staying 0.05 matches below the real-valued
// bound keeps a 6.5e-6 gap, far above the float rounding of j (6e-8) and of
// this computation (< 3e-4 matches).  p >= 10 reaches 1.0: no bound.  A NaN
// threshold never fails a pair in the reference, so it gives no bound either.
__device__ __forceinline__ int m_need_lo(uint32_t ls, uint32_t ll, uint32_t p, float thr) {
  if (p >= 10u) return 0;
  const float c = 0.1f * (float)p;
  // every quotient here is __fdividef (at most 2 ulp off): the relative error
  // of mr stays below 1e-6, under 3e-4 matches for ls <= 256, far inside the
  // 0.05 margin below
  const float jn = __fdividef(thr - c, 1.0f - c);
  // m = (3 jn - 1) / (1/ls + 1/ll) = (3 jn - 1) ls ll / (ls + ll): one
  // quotient, each factor within an ulp or two, so the bound's error stays
  // far inside the margin below as well
  const float mr = __fdividef((3.0f * jn - 1.0f) * (float)ls * (float)ll, (float)ls + (float)ll);
  const float v = ceilf(mr - 0.05f);
  if (!(v > 0.0f)) return 0;
  return v > 1.0e6f ? 1000000 : (int)v;
}

// Slow exact similarity check of one pair (any lengths).  Out of line and
// with plain pointer/scalar arguments only: passing the kernel parameters by
// reference would copy them into local memory for the whole kernel.
__device__ __noinline__ bool sim_pass_slow(const uint8_t* a, uint32_t la, const uint8_t* b,
                                           uint32_t lb, float thr, Counters* ctr) {
  if (la == 0 || lb == 0) return jw_exact(0, la, lb, 0, thr, &ctr->ambiguous);
  const uint32_t mn = min(la, lb);
  if (mn > 256) atomicAdd(&ctr->long_pairs, 1ull);
  const uint32_t m = jaro_m_ref(a, la, b, lb);
  const uint32_t p = prefix_len(a, b, mn);
  return jw_exact(m, mn, max(la, lb), p, thr, &ctr->ambiguous);
}

// The match count and common prefix of one pair by the reference's own
// loops (any lengths; 0 and 0 when a string is empty), for decisions against
// several thresholds.  Out of line like sim_pass_slow.
__device__ __noinline__ void sim_m_slow(const uint8_t* a, uint32_t la, const uint8_t* b,
                                        uint32_t lb, Counters* ctr, uint32_t* m, uint32_t* p) {
  *m = 0;
  *p = 0;
  if (la == 0 || lb == 0) return;
  const uint32_t mn = min(la, lb);
  if (mn > 256) atomicAdd(&ctr->long_pairs, 1ull);
  *m = jaro_m_ref(a, la, b, lb);
  *p = prefix_len(a, b, mn);
}

// Threshold decision on one similarity column of a pair from its match
// count m and common prefix p (la, lb: left and right lengths); an empty
// string takes the reference's rule for empty strings (device_func.cuh:65-69).
__device__ __forceinline__ bool decide(uint32_t m, uint32_t la, uint32_t lb, uint32_t p, float thr,
                                       unsigned long long* ambiguous) {
  if (la == 0 || lb == 0) return jw_exact(0, la, lb, 0, thr, ambiguous);
  return jw_decide(m, min(la, lb), max(la, lb), p, thr, ambiguous);
}

// Members of `live` whose threshold on the group's first column the pair
// reaches.
__device__ __forceinline__ uint32_t first_pass(const Rule* R, uint32_t live, uint32_t m,
                                               uint32_t la, uint32_t lb, uint32_t p,
                                               unsigned long long* ambiguous) {
  uint32_t out = 0;
  for (uint32_t x = live; x; x &= x - 1) {
    const uint32_t k = (uint32_t)__ffs(x) - 1u;
    if (decide(m, la, lb, p, R->mem[k].thr_first, ambiguous)) out |= 1u << k;
  }
  return out;
}

// Does a member of `pass` have no predicate left (the pair matches)?
__device__ __forceinline__ bool member_done(const Rule* R, uint32_t pass) {
  for (uint32_t x = pass; x; x &= x - 1)
    if (R->mem[__ffs(x) - 1].n_rest == 0) return true;
  return false;
}

// Smallest first-column threshold of the live members: the threshold the
// filters and the scan's early stop use.  A NaN threshold never fails a pair
// (the reference compares JW < thr), so it makes the bound NaN: no bound.
__device__ __forceinline__ float live_thr(const Rule* R, uint32_t live) {
  float t = 3.0e38f;
  for (uint32_t x = live; x; x &= x - 1) {
    const float u = R->mem[__ffs(x) - 1].thr_first;
    t = (u != u || t != t) ? __int_as_float(0x7fc00000) : fminf(t, u);
  }
  return t;
}

__device__ __forceinline__ uint32_t find_key(const unsigned long long* item_off, uint32_t domain,
                                             unsigned long long local) {
  uint32_t lo = 0, hi = domain;  // item_off[lo] <= local < item_off[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (item_off[mid] <= local)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Algorithmic work of one Jaro-Winkler evaluation (one pair, one similarity
// predicate) in 64-bit word operations, the per-unit figure the roofline uses:
// 6 per scanned character per 64-bit word of the shorter string (Peq lookup,
// window AND, ANDNOT matched, lowest-bit isolate x2, OR) over
// to = min(ls + h, ll) characters, the prefix compare in 32-bit steps and 16
// for the count and the formula.  It is counted for every evaluation, also
// for pairs the bound settles without a scan.
__device__ __forceinline__ unsigned long long jw_eval_ops(uint32_t ls, uint32_t ll) {
  const uint32_t h = (ls + 1u) >> 1;
  const uint32_t to = min(ls + h, ll);
  return 6ull * to * ((ls + 63u) >> 6) + 2ull * ((ls + 3u) >> 2) + 16ull;
}

// One character step of the bit-parallel match count: x = the unmatched
// positions of the left string equal to `sym` inside the window; the lowest
// one becomes matched; the window [i - h, i + h] moves one position right
// (and only grows while i < h).
template <int W, int S>
__device__ __forceinline__ void bp_step(const uint32_t* __restrict__ tab, uint32_t sym,
                                        uint32_t (&win)[W], uint32_t (&mt)[W], uint32_t grow) {
  uint32_t pe[S];
  load_row<S>(tab + sym * S, pe);
  bp_update<W, S>(pe, win, mt, grow);
}

// First report of a pair?  With several rules a pair can match more than one
// of them (the reference stops at the first rule that passes,
// global_func.cuh:161-165); a device hash set of emitted (left, right) keys
// keeps exactly one report.  Open addressing with linear probing over
// seen_mask + 1 slots (all ones = empty).  The set is sized for a load of at
// most one half, where probe runs stay far below kMaxProbes; a run past it
// means the set is too small for this run's distinct pairs: seen_overflow is
// set, the host repeats the run with a set sized from the pass count
// (Counters::passes, an upper bound on the distinct pairs).  Reports whose
// probe run reaches kCheckProbe look at the overflow flag first and give up
// once it is set, so an overflowing run costs a few probes per report; runs
// of a set sized as intended rarely get that far and never read the flag.
constexpr unsigned long long kMaxProbes = 4096;
constexpr unsigned long long kCheckProbe = 8;
__device__ __forceinline__ bool first_report(const EvalParams& P, uint32_t lrow, uint32_t rrow) {
  const unsigned long long key = ((unsigned long long)lrow << 32) | rrow;
  unsigned long long h = key * 0x9E3779B97F4A7C15ull;
  h ^= h >> 29;
  for (unsigned long long probe = 0; probe <= P.seen_mask && probe < kMaxProbes; probe++) {
    if (probe == kCheckProbe && *(volatile unsigned long long*)&P.ctr->seen_overflow) return false;
    const unsigned long long slot = (h + probe) & P.seen_mask;
    const unsigned long long prev = atomicCAS(P.seen + slot, ~0ull, key);
    if (prev == ~0ull) return true;
    if (prev == key) return false;
  }
  atomicAdd(&P.ctr->seen_overflow, 1ull);
  return false;
}

// Writes up to one match per lane to the output with one atomic per warp
// (after the duplicate set, when the launch has one).
__device__ __forceinline__ void flush_pairs(const EvalParams& P, bool pass, uint32_t lrow,
                                            uint32_t rrow, int lane) {
  if (P.seen) {
    const unsigned cm = __ballot_sync(kFull, pass);
    if (!cm) return;
    if (lane == 0) atomicAdd(&P.ctr->passes, (unsigned long long)__popc(cm));
    if (pass) pass = first_report(P, lrow, rrow);
  }
  const unsigned pm = __ballot_sync(kFull, pass);
  if (!pm) return;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(&P.ctr->out_count, (unsigned long long)__popc(pm));
  base = __shfl_sync(kFull, base, 0);
  if (pass) {
    const unsigned long long pos = base + __popc(pm & ((1u << lane) - 1u));
    if (pos < P.capacity) {
      P.out_l[pos] = lrow;
      P.out_r[pos] = rrow;
    }
  }
}

// Upper bound on the Jaro matches of two strings from their count signatures
// (dev::StrMeta): sum over buckets of the smaller count.
__device__ __forceinline__ uint32_t sig_bound(const uint4& a0, const uint4& a1, const uint4& b0,
                                              const uint4& b1) {
  constexpr unsigned kOnes = 0x01010101u;
  uint32_t s = 0;
  s = __dp4a(__vminu4(a0.x, b0.x), kOnes, s);
  s = __dp4a(__vminu4(a0.y, b0.y), kOnes, s);
  s = __dp4a(__vminu4(a0.z, b0.z), kOnes, s);
  s = __dp4a(__vminu4(a0.w, b0.w), kOnes, s);
  s = __dp4a(__vminu4(a1.x, b1.x), kOnes, s);
  s = __dp4a(__vminu4(a1.y, b1.y), kOnes, s);
  s = __dp4a(__vminu4(a1.z, b1.z), kOnes, s);
  s = __dp4a(__vminu4(a1.w, b1.w), kOnes, s);
  return s;
}

// Common prefix of two 16-symbol little-endian heads; 16 when they agree.
__device__ __forceinline__ uint32_t prefix16(const uint4& a, const uint4& b) {
  const uint32_t d[4] = {a.x ^ b.x, a.y ^ b.y, a.z ^ b.z, a.w ^ b.w};
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (d[k]) return 4u * k + ((uint32_t)(__ffs(d[k]) - 1) >> 3);
  return 16u;
}

// Per-lane work counts of the evaluation loop, summed into Counters at exit:
// algorithmic JW word operations (every evaluation, scanned or not), pairs
// that reached a bit-parallel scan, and scan steps (4 symbols each).
struct WorkTally {
  unsigned long long ops;
  uint32_t scans, steps;
  uint32_t wsteps;  // warp-level scan steps (counted by lane 0)
  uint32_t rest;    // scans of predicates after the first (advance_rule / advance_group)
};

// Does the left string of length la have a Peq table (PeqShape)?
__device__ __forceinline__ bool has_table(const EvalParams& P, uint32_t la) {
  return la > 0u && la <= P.fast_max;
}

__device__ __forceinline__ const uint32_t* peq_table(const EvalParams& P, uint32_t slot,
                                                     uint32_t lrow) {
  return P.peq + ((size_t)slot * P.L.n_rows + lrow) * P.tab_words;
}

// Ring of pairs waiting for a scan, kRingEntries entries of three 16-byte
// records per warp:
//   {right row, right offset / 16, right length, tag}
//   {first 16 symbols of the right string}
//   {left row, left length | Peq slot << 9 | rule << 16, left offset / 16,
//   threshold bits} for a plain entry (its left string has a Peq table:
//   length <= 256; slot 127 = read it from the rule; plans hold at most 64
//   rules), with the threshold its need was computed for; {left row, left
//   length, left offset / 16, rule} for a kAdvance entry.
// tag = need | p << 10 | s << 15 | kAdvance? | live << 19 | member << 27.
// A plain entry waits for the scan of its group's first column: `live` holds
// the members whose extra equalities hold, need the matches the smallest of
// their thresholds needs and p the common prefix (or kPrefixUnknown).  A
// kAdvance entry passed the first column (live = the members that passed):
// the lane that takes it goes on with predicate s of member `member`.
constexpr uint32_t kRing = kRingEntries;
constexpr uint32_t kPrefixUnknown = 31u;  // common prefix longer than 16: measured at the scan
constexpr uint32_t kAdvance = 1u << 18;

__device__ __forceinline__ uint32_t ring_tag(uint32_t need, uint32_t p, uint32_t s, uint32_t live,
                                             uint32_t member) {
  return need | (p << 10) | (s << 15) | (live << 19) | (member << 27);
}
__device__ __forceinline__ uint32_t tag_live(uint32_t t) { return (t >> 19) & 0xffu; }
__device__ __forceinline__ uint32_t tag_member(uint32_t t) { return (t >> 27) & 7u; }
__device__ __forceinline__ uint32_t tag_s(uint32_t t) { return (t >> 15) & 7u; }

// Bit-parallel scan state of one lane: the pair's Peq table and right
// string, the symbols in hand (cur) and the next 16 (nxt), the window and
// matched masks, lengths, position, common prefix, the mismatches it can
// still afford and the threshold.
template <int W>
struct Scan {
  const uint32_t* tab;
  const uint8_t* b;
  uint4 cur, nxt;
  uint32_t win[W], mt[W];
  uint32_t ls, ll, i, n_iter, h, p;
  int allowed;
  float thr;
};

// Starts the scan of a pair (la, lb: lengths; p: common prefix or
// kPrefixUnknown; need: matches the threshold needs).  false = decided
// (fails) without a scan.
template <int W>
__device__ __forceinline__ bool scan_begin(Scan<W>& z, const uint32_t* tab, const uint8_t* a,
                                           const uint8_t* b, const uint4& head_b, uint32_t la,
                                           uint32_t lb, uint32_t p, int need, float thr,
                                           WorkTally* ops) {
  z.ls = min(la, lb);
  z.ll = max(la, lb);
  z.h = (z.ls + 1u) >> 1;
  z.n_iter = min(lb, la + z.h);
  if (p == kPrefixUnknown) {
    p = prefix_len(a, b, z.ls);
    need = m_need_lo(z.ls, z.ll, p, thr);
  }
  if (need > (int)min(z.n_iter, z.ls)) return false;
  z.p = p;
  z.thr = thr;
  z.allowed = (int)z.n_iter - need;
  z.i = 0;
  z.tab = tab;
  z.b = b;
  z.cur = head_b;
  if (z.n_iter > 16u) z.nxt = __ldg(reinterpret_cast<const uint4*>(b + 16));
#pragma unroll
  for (int k = 0; k < W; k++) {
    const int nb = (int)z.h + 1 - 32 * k;
    z.win[k] = nb >= 32 ? 0xffffffffu : (nb <= 0 ? 0u : ((1u << nb) - 1u));
    z.mt[k] = 0u;
  }
  ops->scans++;
  return true;
}

// One scan step of 16 symbols, the chunk in hand (the next chunk was asked
// for one step earlier); after each, the pair stops once even matching every
// remaining symbol stays below its bound.  Returns 0 (not decided yet), 1
// (the scan is complete: *m = the match count) or 2 (the pair cannot reach
// the scan's threshold).
constexpr int kScanQuadUnroll = 1;
template <int W>
__device__ __forceinline__ int scan_step(Scan<W>& z, uint32_t* m_out, WorkTally* ops) {
  constexpr int S = row_words(W);
  if (z.i) {
    // chunk i/16 arrived one chunk ago; ask for the one after it
    z.cur = z.nxt;
    if (z.i + 16u < z.n_iter) z.nxt = __ldg(reinterpret_cast<const uint4*>(z.b + z.i + 16u));
  }
  // four symbols per 32-bit word of the chunk, one word per loop turn: the
  // smaller loop body runs faster than the fully unrolled chunk (C3, 300k
  // rows: 98.5 ms of evaluation against 102.4 ms with two words per turn and
  // 113 ms with four), which stalled on instruction fetch
  uint4 c4 = z.cur;
#pragma unroll(kScanQuadUnroll)
  for (uint32_t q = 0; q < 4; q++) {
    const uint32_t wd = c4.x;
#pragma unroll
    for (int c = 0; c < 4; c++)
      bp_step<W, S>(z.tab, (wd >> (8 * c)) & 0xffu, z.win, z.mt,
                    (z.i + 4u * q + (uint32_t)c) < z.h ? 1u : 0u);
    c4 = make_uint4(c4.y, c4.z, c4.w, 0u);
  }
  z.i += 16;
  ops->steps += 4;
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < W; k++) m += __popc(z.mt[k]);
  *m_out = m;
  if (z.i >= z.n_iter) return 1;
  if ((int)(z.i - m) > z.allowed) return 2;  // even matching every remaining symbol stays below
  return 0;
}

// The similarity predicates after predicate s of a pair that passed it, in
// order, until one needs a scan (returns 2, the scan state set up and s its
// index), one fails (0) or all pass (1).  Each predicate first goes through
// the filters of the first one: length bound, common prefix, count
// signatures.  (A launch without rule groups: every rule evaluated alone.)
template <int W>
__device__ __forceinline__ int advance_rule(const EvalParams& P, uint32_t rule, uint32_t* s,
                                            uint32_t lrow, uint32_t rrow, Scan<W>& z,
                                            WorkTally* ops) {
  const Rule* R = P.rules + rule;
  const uint32_t n_sim = R->n_sim;
  for (uint32_t k = *s + 1; k < n_sim; k++) {
    *s = k;
    const uint32_t sl = R->sim_l[k], sr = R->sim_r[k];
    const float thr = R->thr[k];
    const StrMeta* am = P.L.str_meta + (size_t)sl * P.L.n_rows + lrow;
    const StrMeta* bm = P.R.str_meta + (size_t)sr * P.R.n_rows + rrow;
    const uint4 al = am->loc, bl = bm->loc;
    const uint32_t la = al.y, lb = bl.y;
    const uint8_t* a = P.L.arena + 16ull * al.x;
    const uint8_t* b = P.R.arena + 16ull * bl.x;
    if (!has_table(P, la)) {  // the reference's own loops
      if (la && lb) ops->ops += jw_eval_ops(min(la, lb), max(la, lb));
      if (!sim_pass_slow(a, la, b, lb, thr, P.ctr)) return 0;
      continue;
    }
    if (lb == 0) {
      if (!jw_exact(0, la, 0, 0, thr, &P.ctr->ambiguous)) return 0;
      continue;
    }
    const uint32_t ls = min(la, lb), ll = max(la, lb);
    ops->ops += jw_eval_ops(ls, ll);
    const uint4 bh = bm->head;
    const uint32_t p16 = prefix16(am->head, bh);
    uint32_t p = kPrefixUnknown;
    int need = 0;
    if (!(p16 == 16u && ls > 16u)) {
      p = min(p16, ls);
      need = m_need_lo(ls, ll, p, thr);
      const uint32_t n_iter = min(lb, la + ((ls + 1u) >> 1));
      if (need > (int)min(n_iter, ls)) return 0;
      if (need > 0 &&
          (int)sig_bound(am->sig[0], am->sig[1], bm->sig[0], bm->sig[1]) < need)
        return 0;
    }
    ops->rest++;
    return scan_begin<W>(z, peq_table(P, sl, lrow), a, b, bh, la, lb, p, need, thr, ops) ? 2 : 0;
  }
  return 1;
}

// The similarity predicates after the group's first column, for the live
// members of a pair's group in member order, from predicate *s of member
// *mi: until one needs a scan (returns 2, the scan state set up for (*mi,
// *s)), a member passes all of its predicates (1: the pair matches) or no
// member is left (0).  A member drops out at its first failing predicate.
// Each predicate first goes through the filters of the first column: length
// bound, common prefix, count signatures.
//
// A member that needs a scan of a column scans it at the smallest threshold
// among itself and the live members after it that test the same column, so
// that one scan serves them all: *memo then names the column (left slot <<
// 16 | right slot) and memo_m holds its match count (the scan state z still
// holds the pair's lengths and prefix) or kMemoBelow (the scan stopped below
// that smallest threshold, so every one of those members fails the column).
// Each member decides at its own threshold.  Starting a scan ends the memo.
constexpr uint32_t kNoMemo = 0xffffffffu;
constexpr uint32_t kMemoBelow = 0xffffffffu;

// Smallest threshold on column (sl, sr) of member mi (threshold thr) and of
// the live members after it that test that column; NaN (no bound) when one
// of them has a NaN threshold.
__device__ __forceinline__ float shared_thr(const Rule* R, uint32_t live, uint32_t mi, uint32_t sl,
                                            uint32_t sr, float thr) {
  float t = thr;
  for (uint32_t x = live & ~((2u << mi) - 1u); x; x &= x - 1) {
    const Member* M = R->mem + (__ffs(x) - 1);
    for (uint32_t j = 0; j < M->n_rest; j++)
      if (M->rest_l[j] == sl && M->rest_r[j] == sr) {
        const float u = M->rest_thr[j];
        t = (u != u || t != t) ? __int_as_float(0x7fc00000) : fminf(t, u);
        break;
      }
  }
  return t;
}

template <int W>
__device__ __forceinline__ int advance_group(const EvalParams& P, uint32_t rule, uint32_t* live,
                                             uint32_t* mi, uint32_t* s, uint32_t lrow,
                                             uint32_t rrow, Scan<W>& z, uint32_t* memo,
                                             uint32_t memo_m, WorkTally* ops) {
  const Rule* R = P.rules + rule;
  while (*live) {
    const Member* M = R->mem + *mi;
    const uint32_t n_rest = M->n_rest;
    uint32_t k = *s;
    for (; k < n_rest; k++) {
      const uint32_t sl = M->rest_l[k], sr = M->rest_r[k];
      const float thr = M->rest_thr[k];
      if (*memo == (sl << 16 | sr)) {
        if (memo_m == kMemoBelow || !jw_decide(memo_m, z.ls, z.ll, z.p, thr, &P.ctr->ambiguous))
          break;
        continue;
      }
      const StrMeta* am = P.L.str_meta + (size_t)sl * P.L.n_rows + lrow;
      const StrMeta* bm = P.R.str_meta + (size_t)sr * P.R.n_rows + rrow;
      const uint4 al = am->loc, bl = bm->loc;
      const uint32_t la = al.y, lb = bl.y;
      const uint8_t* a = P.L.arena + 16ull * al.x;
      const uint8_t* b = P.R.arena + 16ull * bl.x;
      if (!has_table(P, la)) {  // the reference's own loops
        if (la && lb) ops->ops += jw_eval_ops(min(la, lb), max(la, lb));
        if (!sim_pass_slow(a, la, b, lb, thr, P.ctr)) break;
        continue;
      }
      if (lb == 0) {
        if (!jw_exact(0, la, 0, 0, thr, &P.ctr->ambiguous)) break;
        continue;
      }
      const uint32_t ls = min(la, lb), ll = max(la, lb);
      ops->ops += jw_eval_ops(ls, ll);
      const uint4 bh = bm->head;
      const uint32_t p16 = prefix16(am->head, bh);
      uint32_t p = kPrefixUnknown;
      int need = 0;
      if (!(p16 == 16u && ls > 16u)) {
        p = min(p16, ls);
        need = m_need_lo(ls, ll, p, thr);
        const uint32_t n_iter = min(lb, la + ((ls + 1u) >> 1));
        if (need > (int)min(n_iter, ls)) break;
        if (need > 0 && (int)sig_bound(am->sig[0], am->sig[1], bm->sig[0], bm->sig[1]) < need)
          break;
      }
      // member *mi may pass: one scan for it and the later members testing
      // this column, at the smallest of their thresholds
      const float ts = shared_thr(R, *live, *mi, sl, sr, thr);
      if (p != kPrefixUnknown && ts != thr) need = m_need_lo(ls, ll, p, ts);
      *memo = kNoMemo;  // z is about to hold another pair's scan
      ops->rest++;
      if (scan_begin<W>(z, peq_table(P, sl, lrow), a, b, bh, la, lb, p, need, ts, ops)) {
        *s = k;
        return 2;
      }
      break;
    }
    if (k >= n_rest) return 1;
    *live &= ~(1u << *mi);  // member *mi failed predicate k
    if (!*live) return 0;
    *mi = (uint32_t)__ffs(*live) - 1u;
    *s = 0;
  }
  return 0;
}

// Warp-uniform state of the evaluation loop kept in shared memory (every
// lane reads it; every lane writes the same values, after a __syncwarp when
// the values were read in the same step): the work items the warp has
// claimed, the claim in each staging buffer, and the item being filtered.
constexpr uint32_t kMaxClaimChunk = 16;
// Kind of a claimed item: its rule has similarity predicates, and some
// member of its group has extra equality slots; bits 8-11 hold the group's
// member count.
constexpr uint32_t kItemSim = 1u, kItemExtras = 2u, kItemMore = 4u;  // more: n_sim > 1
__device__ __forceinline__ uint32_t item_members(uint32_t kind) { return (kind >> 8) & 15u; }
// A claimed work item: the sources of its bulk copies (right-row metadata
// from the block's first row, right rows from the 16-byte boundary at or
// before it, the left string's metadata), left row, rule, rows, the shift of
// the first row past the boundary, its kind and the group's smallest
// first-column threshold.
struct ItemDesc {
  const StrMeta* meta_src;
  const uint32_t* rows_src;
  const StrMeta* lm_src;
  uint32_t lrow, rule, n, shift, kind;
  float thr0;
  int32_t lcode[2];  // the left row's codes of the group's first two extra slots
};
constexpr uint32_t kOutBuf = 64;  // matches a warp holds before writing them out
struct WarpCtl {
  ItemDesc desc[kMaxClaimChunk];  // claimed items not yet staged
  uint32_t c_rule[kMaxStageBufs], c_lrow[kMaxStageBufs];  // claim per staging buffer
  uint32_t c_n[kMaxStageBufs], c_shift[kMaxStageBufs];    // (n = 0: none)
  uint32_t c_kind[kMaxStageBufs];
  float c_thr[kMaxStageBufs];
  int32_t c_lcode[kMaxStageBufs][2];
  // the item being filtered; i_lcode: its left row's codes of the group's
  // extra equality slots
  uint32_t i_rule, i_lrow, i_kind, i_fast, i_all;
  float i_thr;
  int32_t i_lcode[kMaxEq];
  // matches not yet written out (emit): fewer than 32 between calls
  uint2 out_buf[kOutBuf];
  uint32_t out_n;
};
static_assert(sizeof(WarpCtl) <= kWarpCtlWords * 4, "warp control block outgrows its words");

// Collects the warp's final matches of one step; every 32 of them go out
// together (flush_pairs), so the duplicate-set probes and the output
// reservation pay their round trips once per 32 matches instead of once per
// step with a match.
__device__ __forceinline__ void emit(const EvalParams& P, WarpCtl* C, bool pass, uint32_t lrow,
                                     uint32_t rrow, int lane) {
  const unsigned pm = __ballot_sync(kFull, pass);
  if (!pm) return;
  const uint32_t n0 = C->out_n;
  if (pass) C->out_buf[n0 + __popc(pm & ((1u << lane) - 1u))] = make_uint2(lrow, rrow);
  const uint32_t n = n0 + __popc(pm);
  __syncwarp();
  if (n < 32) {
    if (lane == 0) C->out_n = n;
    __syncwarp();
    return;
  }
  const uint2 e = C->out_buf[lane];
  const bool more = (uint32_t)lane + 32u < n;
  const uint2 t = more ? C->out_buf[32 + lane] : make_uint2(0u, 0u);
  __syncwarp();
  if (more) C->out_buf[lane] = t;
  if (lane == 0) C->out_n = n - 32u;
  __syncwarp();
  flush_pairs(P, true, e.x, e.y, lane);
}

// Writes out the matches emit still holds (at the end of the warp's loop).
__device__ __forceinline__ void emit_drain(const EvalParams& P, WarpCtl* C, int lane) {
  const uint32_t n = C->out_n;
  const bool have = (uint32_t)lane < n;
  const uint2 e = have ? C->out_buf[lane] : make_uint2(0u, 0u);
  __syncwarp();
  if (lane == 0) C->out_n = 0;
  __syncwarp();
  flush_pairs(P, have, e.x, e.y, lane);
}

// Filter one batch of 32 right rows of the item against its group's first
// similarity column: first the members whose extra equalities hold for the
// pair (live), then one staged metadata record per right row gives its
// length and first 16 symbols, hence the common prefix p (when below 16) and
// the match count the smallest live threshold needs, and its count
// signature, an upper bound on the matches; pairs that cannot reach it are
// decided here, the rest go to the ring with their first 16 symbols.  Pairs
// decided without a scan that pass go to the ring for their members' further
// predicates, or match at once when a passing member has none.  lm: the
// item's left string metadata.  Returns the entries appended.
// G: the launch has rule groups; without, every rule is its own group of one
// and its predicates take the plain path (one threshold per predicate).
template <bool G>
__device__ __forceinline__ uint32_t filter_batch(const EvalParams& P, WarpCtl* C,
                                                 const StrMeta* lm, const uint32_t* rows,
                                                 const StrMeta* meta, uint32_t n, uint32_t e0,
                                                 uint4* q, uint32_t tail, WorkTally* ops) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t e = e0 + (uint32_t)lane;
  const bool act = e < n;
  const uint32_t rrow = act ? rows[e] : 0u;
  const uint32_t la = lm->loc.y, a_off = lm->loc.x;
  const Rule* R = P.rules + C->i_rule;
  const uint32_t all = C->i_all;
  uint32_t live = act ? all : 0u;
  float thr = C->i_thr;
  uint4 loc = make_uint4(0, 0, 0, 0), head = make_uint4(0, 0, 0, 0);
  if (act) loc = meta[e].loc;
  if (G && act && (C->i_kind & kItemExtras)) {
    // the right row's codes of the extra slots: the first two staged with
    // its metadata (sorted_meta), the others from device memory
    uint32_t eqm = 0;
    const uint32_t nx = R->n_xslots;
    if ((int32_t)loc.z == C->i_lcode[0]) eqm |= 1u;
    if (nx > 1 && (int32_t)loc.w == C->i_lcode[1]) eqm |= 2u;
    if (nx <= 2u) {  // the group's table (Rule::x_live, x_thr)
      live = R->x_live[eqm];
      if (live != all) thr = R->x_thr[eqm];
    } else {
      for (uint32_t j = 2; j < nx; j++)
        if (P.R.eq_codes[(size_t)R->xslot[j] * P.R.n_rows + rrow] == C->i_lcode[j]) eqm |= 1u << j;
      for (uint32_t x = all; x; x &= x - 1) {
        const uint32_t k = (uint32_t)__ffs(x) - 1u;
        if (R->mem[k].xmask & ~eqm) live &= ~(1u << k);
      }
      if (live != all) thr = live_thr(R, live);
    }
  }
  if (live) head = meta[e].head;
  uint32_t pass1 = 0;  // members that passed the first column without a scan
  bool scan = false;
  uint32_t p = 0;
  int need = 0;
  if (live) {
    const uint32_t lb = loc.y;
    if (!C->i_fast) {  // the reference's own loops
      if (la && lb) ops->ops += jw_eval_ops(min(la, lb), max(la, lb));
      if constexpr (G) {
        uint32_t m = 0, pp = 0;
        sim_m_slow(P.L.arena + 16ull * a_off, la, P.R.arena + 16ull * loc.x, lb, P.ctr, &m, &pp);
        pass1 = first_pass(R, live, m, la, lb, pp, &P.ctr->ambiguous);
      } else {
        pass1 = sim_pass_slow(P.L.arena + 16ull * a_off, la, P.R.arena + 16ull * loc.x, lb, thr,
                              P.ctr) ? 1u : 0u;
      }
    } else if (lb == 0) {
      if constexpr (G)
        pass1 = first_pass(R, live, 0, la, 0, 0, &P.ctr->ambiguous);
      else
        pass1 = jw_exact(0, la, 0, 0, thr, &P.ctr->ambiguous) ? 1u : 0u;
    } else {
      const uint32_t ls = min(la, lb), ll = max(la, lb);
      ops->ops += jw_eval_ops(ls, ll);
      const uint32_t p16 = prefix16(lm->head, head);
      if (p16 == 16u && ls > 16u) {
        scan = true;  // prefix longer than 16: measured exactly before the scan
        p = kPrefixUnknown;
      } else {
        p = min(p16, ls);
        need = m_need_lo(ls, ll, p, thr);
        const uint32_t n_iter = min(lb, la + ((ls + 1u) >> 1));
        scan = need <= (int)min(n_iter, ls);  // else the threshold is out of reach
        // the count signatures bound the matches from above: below the need,
        // the pair cannot pass
        if (scan && need > 0 &&
            (int)sig_bound(lm->sig[0], lm->sig[1], meta[e].sig[0], meta[e].sig[1]) < need)
          scan = false;
      }
    }
  }
  bool done;
  if constexpr (G)
    done = pass1 && member_done(R, pass1);
  else
    done = pass1 && !(C->i_kind & kItemMore);
  const bool push = scan || (pass1 && !done);
  const unsigned qm = __ballot_sync(kFull, push);
  const uint32_t lrow = C->i_lrow;
  if (push) {
    const uint32_t slot = (tail + __popc(qm & lt)) & (kRing - 1);
    uint4* en = q + kRingWords / 4 * slot;
    const uint32_t tag = scan ? ring_tag((uint32_t)need, p, 0, live, 0)
                              : (ring_tag(0, 0, 0, pass1, (uint32_t)__ffs(pass1) - 1u) | kAdvance);
    en[0] = make_uint4(rrow, loc.x, loc.y, tag);
    en[1] = head;
    en[2] = scan ? make_uint4(lrow, la | (min(R->sim_l[0], 127u) << 9) | (C->i_rule << 16), a_off,
                              __float_as_uint(thr))
                 : make_uint4(lrow, la, a_off, C->i_rule);
  }
  emit(P, C, done, lrow, rrow, lane);
  return __popc(qm);
}

// Maps a position of the launch's work list to a global work item: the list
// is the concatenation of the segments [seg_begin[k], seg_end[k]).
__device__ __forceinline__ unsigned long long seg_item(const EvalParams& P, unsigned long long v) {
  for (uint32_t k = 0; k < P.n_seg; k++) {
    const unsigned long long len = P.seg_end[k] - P.seg_begin[k];
    if (v < len) return P.seg_begin[k] + v;
    v -= len;
  }
  return ~0ull;
}

// ---- bulk copies (TMA) into shared memory, completed on an mbarrier --------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

// Global -> shared bulk copy: both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase with the given parity, at most kMaxWaitSpins tries
// (each try suspends the thread for a while).  false = gave up.
constexpr uint32_t kMaxWaitSpins = 1u << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t k = 0; k < kMaxWaitSpins; k++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}


// Key of the item at position `local` of a rule's item space, searched in
// [lo, hi): item_off[lo] <= local < item_off[hi].
__device__ __forceinline__ uint32_t find_key_in(const unsigned long long* item_off, uint32_t lo,
                                                uint32_t hi, unsigned long long local) {
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(item_off + mid) <= local)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Claims up to `chunk` consecutive work positions with one atomic and
// computes their item descriptors into C->desc, one lane per item, so the
// dependent loads of every item (rule fields included) overlap.  Within one rule, the first and
// last lanes find their keys over the whole key space and the others search
// only between those two.  Returns the count (0: the work list is exhausted).
__device__ __forceinline__ uint32_t claim_chunk(const EvalParams& P, WarpCtl* C,
                                                unsigned long long n_work, uint32_t chunk) {
  const int lane = threadIdx.x & 31;
  unsigned long long v0 = 0;
  if (lane == 0) v0 = atomicAdd(&P.ctr->work_next, (unsigned long long)chunk);
  v0 = __shfl_sync(kFull, v0, 0);
  if (v0 >= n_work) return 0;
  const uint32_t n = (uint32_t)min((unsigned long long)chunk, n_work - v0);
  const uint32_t k = min((uint32_t)lane, n - 1);  // lanes past n repeat the last item
  const unsigned long long v = v0 + k;
  const unsigned long long it = P.n_seg ? seg_item(P, v) : v;
  uint32_t r = 0;
  while (r + 1 < P.n_rules && P.rule_item_base[r + 1] <= it) r++;
  const Rule& R = P.rules[r];
  const unsigned long long local = it - P.rule_item_base[r];
  const uint32_t r_first = __shfl_sync(kFull, r, 0), r_last = __shfl_sync(kFull, r, n - 1);
  uint32_t jl;  // left key (word class, join key)
  if (r_first == r_last) {
    uint32_t kb = 0;
    if (k == 0 || k == n - 1) kb = find_key(R.item_off, R.domain_l, local);
    const uint32_t k0 = __shfl_sync(kFull, kb, 0), k1 = __shfl_sync(kFull, kb, n - 1);
    jl = find_key_in(R.item_off, k0, k1 + 1, local);
  } else {
    jl = find_key(R.item_off, R.domain_l, local);
  }
  const uint32_t key = jl % R.domain;  // join key
  const unsigned long long in_key = local - R.item_off[jl];
  const uint32_t nl = R.cnt_l[jl];
  const uint32_t ri = (uint32_t)(in_key / nl);
  const uint32_t li = (uint32_t)(in_key - (unsigned long long)ri * nl);
  const uint32_t lrow = R.sorted_l[R.off_l[jl] + li];
  const uint32_t offr = R.off_r[key];
  const uint32_t rb0 = offr + ri * P.tile_right;
  const uint32_t rb1 = min(rb0 + P.tile_right, offr + R.cnt_r[key]);
  const uint32_t a0 = rb0 & ~3u;
  ItemDesc d;
  const bool sim = R.n_sim != 0;
  d.kind = (sim ? kItemSim : 0u) | (R.n_xslots ? kItemExtras : 0u) |
           (R.n_sim > 1 ? kItemMore : 0u) | (R.n_members << 8) | (R.n_xslots << 12);
  // loaded here, a claim ahead of the item's filtering
  d.lcode[0] = R.n_xslots > 0 ? P.L.eq_codes[(size_t)R.xslot[0] * P.L.n_rows + lrow] : 0;
  d.lcode[1] = R.n_xslots > 1 ? P.L.eq_codes[(size_t)R.xslot[1] * P.L.n_rows + lrow] : 0;
  d.meta_src = sim ? R.sorted_meta_r + rb0 : nullptr;
  d.rows_src = R.sorted_r + a0;
  d.lm_src = sim ? P.L.str_meta + (size_t)R.sim_l[0] * P.L.n_rows + lrow : nullptr;
  d.lrow = lrow;
  d.rule = r;
  d.n = rb1 - rb0;
  d.shift = rb0 - a0;
  d.thr0 = sim ? R.thr_min : 0.0f;
  __syncwarp();  // earlier reads of the descriptors are done
  if ((uint32_t)lane < n) C->desc[lane] = d;
  __syncwarp();
  return n;
}

// Claims the next work item whose rule has similarity predicates and starts
// the bulk copies of its right rows, their metadata and its left string's
// metadata into staging buffer b (completing on bar).  Items of rules with
// equalities only are emitted on the spot.  Items come from the warp's
// claimed descriptors C->desc[*d_pos, *d_n), refilled by claim_chunk.  Once
// the work list is exhausted or the cycle budget has run out, *stop is set
// and this and every later claim leave c_n[b] = 0.
__device__ __forceinline__ void claim_item(const EvalParams& P, WarpCtl* C, uint32_t b,
                                           uint32_t* buf, uint64_t* bar, unsigned long long n_work,
                                           uint32_t chunk, long long t_start, bool* stop,
                                           uint32_t* d_pos, uint32_t* d_n,
                                           unsigned long long* done) {
  const int lane = threadIdx.x & 31;
  while (!*stop) {
    if (*d_pos >= *d_n) {
      *d_n = claim_chunk(P, C, n_work, chunk);
      *d_pos = 0;
      if (*d_n == 0) {
        *stop = true;
        break;
      }
    }
    if (P.watchdog_cycles && (unsigned long long)(clock64() - t_start) > P.watchdog_cycles) {
      if (lane == 0) atomicAdd(&P.ctr->watchdog_trips, 1ull);
      *stop = true;
      break;
    }
    const ItemDesc d = C->desc[(*d_pos)++];
    if (!(d.kind & kItemSim)) {  // equalities only: every candidate matches
      for (uint32_t e = 0; e < d.n; e += 32) {
        const uint32_t k = e + (uint32_t)lane;
        const uint32_t rrow = k < d.n ? d.rows_src[d.shift + k] : 0u;
        emit(P, C, k < d.n, d.lrow, rrow, lane);
      }
      (*done)++;
      continue;
    }
    if (lane == 0) {
      const uint32_t mbytes = d.n * (uint32_t)sizeof(StrMeta);
      const uint32_t rbytes = ((d.n + d.shift) * 4u + 15u) & ~15u;
      // earlier reads of this buffer are done (__syncwarp before the claim);
      // order them before the asynchronous writes
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(bar, mbytes + rbytes + (uint32_t)sizeof(StrMeta));
      bulk_g2s(buf, d.meta_src, mbytes, bar);
      bulk_g2s(buf + P.buf_rows_off, d.rows_src, rbytes, bar);
      bulk_g2s(buf + P.buf_lmeta_off, d.lm_src, (uint32_t)sizeof(StrMeta), bar);
    }
    C->c_rule[b] = d.rule;
    C->c_lrow[b] = d.lrow;
    C->c_n[b] = d.n;
    C->c_shift[b] = d.shift;
    C->c_kind[b] = d.kind;
    C->c_thr[b] = d.thr0;
    C->c_lcode[b][0] = d.lcode[0];
    C->c_lcode[b][1] = d.lcode[1];
    return;
  }
  C->c_n[b] = 0;
}

// The evaluation loop of one warp, for scans over W-word masks.  Work items
// (one left row x up to tile_right right rows of one candidate block) are
// claimed one ahead, so the bulk copies of the next item run while the
// current one is filtered.  Filtered pairs queue in the warp's ring; lanes
// take the next queued pair as soon as theirs is decided, whichever item it
// came from, since every pair reads its left string's Peq table from device
// memory; the ring is refilled from the current item, then the next ones, as
// it drains.  A pair that passes its group's first column goes on with the
// further predicates of the members that passed, member by member, in the
// same lane; matches leave by warp-aggregated atomics.
template <int W, bool G>
__device__ __forceinline__ void eval_loop(const EvalParams& P, uint32_t* region,
                                          unsigned long long n_work, WorkTally* ops,
                                          unsigned long long* done) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  uint4* q = reinterpret_cast<uint4*>(region);
  WarpCtl* C = reinterpret_cast<WarpCtl*>(region + P.ctl_off);
  uint64_t* bar0 = reinterpret_cast<uint64_t*>(region + P.mbar_off);
  const long long t_start = clock64();
  if (lane == 0) C->out_n = 0;
  __syncwarp();
  // work positions per claim: every warp gets about eight claims, at most
  // kMaxClaimChunk items each
  const unsigned long long n_warps = (unsigned long long)gridDim.x * kWarpsPerCta;
  const uint32_t chunk =
      (uint32_t)max(1ull, min((unsigned long long)kMaxClaimChunk, n_work / (n_warps * 8ull)));
  bool stop = false;
  uint32_t d_pos = 0, d_n = 0;  // the warp's claimed descriptors not yet taken
  for (uint32_t b = 0; b < P.n_bufs; b++)
    claim_item(P, C, b, region + P.buf_off + b * P.buf_words, bar0 + b, n_work, chunk, t_start,
               &stop, &d_pos, &d_n, done);
  uint32_t cb = 0;      // buffer of the current item (buffer cb + k holds the k-th next)
  uint32_t phs = 0;     // bit b: mbarrier phase of buffer b
  bool active = false;  // current item waited for and being filtered
  uint32_t in_pos = 0, cur_n = C->c_n[0];
  uint32_t head = 0, tail = 0;
  // lane state: the pair, its group's live members, the member and predicate
  // in hand (first = the group's first column)
  bool busy = false, first = false;
  uint32_t rrow = 0, lrow = 0, rule = 0, s = 0, live = 0, mi = 0;
  uint32_t memo = kNoMemo, memo_m = 0;  // the last finished column scan (advance_group)
  Scan<W> z;
  z.tab = nullptr;
  z.b = nullptr;
  z.cur = z.nxt = make_uint4(0, 0, 0, 0);
  z.ls = z.ll = z.i = z.n_iter = z.h = z.p = 0;
  z.allowed = 0;
  z.thr = 0.0f;
#pragma unroll
  for (int k = 0; k < W; k++) z.win[k] = z.mt[k] = 0u;

  for (;;) {
    const unsigned idle = __ballot_sync(kFull, !busy);
    const uint32_t n_idle = __popc(idle);
    // refill the ring until it holds a pair for every idle lane
    while (tail - head < n_idle && tail - head <= kRing - 32) {
      uint32_t* buf = region + P.buf_off + cb * P.buf_words;
      if (active) {
        if (in_pos < cur_n) {
          tail += filter_batch<G>(P, C, reinterpret_cast<const StrMeta*>(buf + P.buf_lmeta_off),
                               buf + P.buf_rows_off + C->c_shift[cb],
                               reinterpret_cast<const StrMeta*>(buf), cur_n, in_pos, q, tail, ops);
          in_pos += 32;
          continue;
        }
        // the item is filtered: its buffer takes the item after the next one
        active = false;
        __syncwarp();
        claim_item(P, C, cb, buf, bar0 + cb, n_work, chunk, t_start, &stop, &d_pos, &d_n, done);
        cb = cb + 1u == P.n_bufs ? 0u : cb + 1u;
        buf = region + P.buf_off + cb * P.buf_words;
        cur_n = C->c_n[cb];
      }
      if (cur_n == 0) break;  // no work left (claims run in order)
      const bool ok = mbar_wait(bar0 + cb, (phs >> cb) & 1u);
      phs ^= 1u << cb;
      if (!__all_sync(kFull, ok)) {
        // a copy never completed: report, wait once more (bounded) for it
        // and for the other buffers' copies, stop
        if (lane == 0) atomicAdd(&P.ctr->watchdog_trips, 1ull);
        mbar_wait(bar0 + cb, ((phs >> cb) & 1u) ^ 1u);
        for (uint32_t b = 0; b < P.n_bufs; b++)
          if (b != cb && C->c_n[b]) mbar_wait(bar0 + b, (phs >> b) & 1u);
        emit_drain(P, C, lane);
        return;
      }
      active = true;
      in_pos = 0;
      (*done)++;
      const StrMeta* lm = reinterpret_cast<const StrMeta*>(buf + P.buf_lmeta_off);
      const uint32_t ir = C->c_rule[cb], il = C->c_lrow[cb], kind = C->c_kind[cb];
      const float thr = C->c_thr[cb];
      const uint32_t la = lm->loc.y;
      __syncwarp();  // the previous item's fields are read
      C->i_rule = ir;
      C->i_lrow = il;
      C->i_thr = thr;
      C->i_kind = kind;
      C->i_all = (1u << item_members(kind)) - 1u;
      C->i_fast = has_table(P, la) ? 1u : 0u;
      if (G && (kind & kItemExtras)) {  // the left row's codes of the extra equality slots
        const uint32_t nx = (kind >> 12) & 15u;
        if (lane < 2) {
          C->i_lcode[lane] = C->c_lcode[cb][lane];  // loaded with the claim
        } else if ((uint32_t)lane < nx) {
          const Rule* R = P.rules + ir;
          C->i_lcode[lane] = P.L.eq_codes[(size_t)R->xslot[lane] * P.L.n_rows + il];
        }
      }
      __syncwarp();
    }
    // idle lanes take the next queued pairs
    bool fin = false, pass = false;
    const uint32_t avail = tail - head;
    const uint32_t rank = __popc(idle & lt);
    if (!busy && rank < avail) {
      const uint4* en = q + kRingWords / 4 * ((head + rank) & (kRing - 1));
      const uint4 e0 = en[0], e2 = en[2];
      rrow = e0.x;
      lrow = e2.x;
      live = tag_live(e0.w);
      memo = kNoMemo;
      int st = 0;
      if (e0.w & kAdvance) {
        rule = e2.w;
        first = false;
        mi = tag_member(e0.w);
        s = tag_s(e0.w);
        if constexpr (G)
          st = advance_group<W>(P, rule, &live, &mi, &s, lrow, rrow, z, &memo, memo_m, ops);
        else
          st = advance_rule<W>(P, rule, &s, lrow, rrow, z, ops);
      } else {
        // the group's first column at the smallest live threshold (without
        // groups: the rule's first predicate), as the filter computed it
        rule = e2.y >> 16;
        first = true;
        s = 0;
        uint32_t sl0 = (e2.y >> 9) & 127u;  // 127: the slot did not fit, read it from the rule
        if (sl0 == 127u) sl0 = P.rules[rule].sim_l[0];
        const uint32_t p = (e0.w >> 10) & 31u;
        st = scan_begin<W>(z, peq_table(P, sl0, lrow), P.L.arena + 16ull * e2.z,
                           P.R.arena + 16ull * e0.y, en[1], e2.y & 511u, e0.z, p,
                           (int)(e0.w & 1023u), __uint_as_float(e2.w), ops)
                 ? 2
                 : 0;
      }
      if (st == 2) {
        busy = true;
      } else {
        fin = true;
        pass = st == 1;
      }
    }
    head += min(n_idle, avail);
    // every lane votes (a warp vote must be reached by all lanes of its mask)
    const bool any_busy = __any_sync(kFull, busy);
    if (lane == 0 && any_busy) ops->wsteps++;
    if (busy) {
      uint32_t m = 0;
      const int sc = scan_step<W>(z, &m, ops);
      if (sc) {
        busy = false;
        int st = 0;
        if constexpr (!G) {
          // one rule: the scanned predicate s decides, then its next ones
          if (sc == 1 && jw_decide(m, z.ls, z.ll, z.p, z.thr, &P.ctr->ambiguous))
            st = advance_rule<W>(P, rule, &s, lrow, rrow, z, ops);
        } else if (first) {
          // decided per live member; the scan stopped early only when even
          // the smallest threshold is out of reach
          const Rule* R = P.rules + rule;
          const uint32_t pass1 =
              sc == 1 ? first_pass(R, live, m, z.ls, z.ll, z.p, &P.ctr->ambiguous) : 0u;
          if (pass1 && member_done(R, pass1)) {
            st = 1;
          } else if (pass1) {
            first = false;
            live = pass1;
            mi = (uint32_t)__ffs(pass1) - 1u;
            s = 0;
            memo = kNoMemo;
            st = advance_group<W>(P, rule, &live, &mi, &s, lrow, rrow, z, &memo, memo_m, ops);
          }
        } else {
          // the scan ran at the smallest threshold of the members testing
          // this column (advance_group): remembered for them, and member mi
          // decides at its own threshold
          const Member* M = P.rules[rule].mem + mi;
          memo = M->rest_l[s] << 16 | M->rest_r[s];
          memo_m = sc == 1 ? m : kMemoBelow;
          if (sc == 1 && jw_decide(m, z.ls, z.ll, z.p, M->rest_thr[s], &P.ctr->ambiguous)) {
            s++;  // member mi passed predicate s
          } else {
            live &= ~(1u << mi);
            mi = live ? (uint32_t)__ffs(live) - 1u : 0u;
            s = 0;
          }
          if (live)
            st = advance_group<W>(P, rule, &live, &mi, &s, lrow, rrow, z, &memo, memo_m, ops);
        }
        if (st == 2) {
          busy = true;
        } else {
          fin = true;
          pass = st == 1;
        }
      }
    }
    emit(P, C, fin && pass, lrow, rrow, lane);
    if (!__any_sync(kFull, busy) && head == tail && !active && cur_n == 0) break;
  }
  emit_drain(P, C, lane);
}

// The evaluation kernel body for masks of W words, instantiated below with
// two register budgets (k_eval / k_eval_wide) and for rule groups.  One
// kernel per mask width: a kernel holding every width's scan loop is
// register-allocated for the widest and spills in the narrow ones too.
template <int W, bool G>
__device__ __forceinline__ void eval_body(const EvalParams& P) {
  extern __shared__ __align__(16) uint32_t smem[];
  pdl_wait();  // the join is complete (launched after it with launch_dependent)
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  uint32_t* region = smem + (size_t)warp * P.warp_words;
  if (lane == 0) {
    uint64_t* bar = reinterpret_cast<uint64_t*>(region + P.mbar_off);
    for (uint32_t b = 0; b < P.n_bufs; b++) mbar_init(bar + b);
  }
  __syncwarp();
  unsigned long long n_work = 0;  // length of this launch's work list
  if (P.n_seg == 0) {
    n_work = P.rule_item_base[P.n_rules];
  } else {
    for (uint32_t k = 0; k < P.n_seg; k++) n_work += P.seg_end[k] - P.seg_begin[k];
  }
  unsigned long long done = 0;
  WorkTally tally{0ull, 0u, 0u, 0u, 0u};
  eval_loop<W, G>(P, region, n_work, &tally, &done);
  if (lane == 0 && done) atomicAdd(&P.ctr->items_done, done);
  unsigned long long ops = tally.ops, scans = tally.scans, steps = tally.steps, rest = tally.rest;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ops += __shfl_down_sync(kFull, ops, o);
    scans += __shfl_down_sync(kFull, scans, o);
    steps += __shfl_down_sync(kFull, steps, o);
    rest += __shfl_down_sync(kFull, rest, o);
  }
  if (lane == 0) {
    if (ops) atomicAdd(&P.ctr->jw_word_ops, ops);
    if (scans) atomicAdd(&P.ctr->scans, scans);
    if (steps) atomicAdd(&P.ctr->scan_steps, steps);
    if (rest) atomicAdd(&P.ctr->rest_scans, rest);
    if (tally.wsteps) atomicAdd(&P.ctr->scan_warp_steps, (unsigned long long)tally.wsteps);
  }
}

// Peq tables (PeqShape): one warp per (slot, row); the table is cleared,
// then every symbol's mask per 32-symbol word is built with __match_any_sync
// (lanes holding the same symbol agree on it; the lowest of them stores it).
__global__ void k_peq_build(Side L, uint32_t n_slots, PeqShape shape, uint32_t* peq) {
  const int lane = threadIdx.x & 31;
  const unsigned long long n_tasks = (unsigned long long)n_slots * L.n_rows;
  const unsigned long long n_warps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
  for (unsigned long long t = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       t < n_tasks; t += n_warps) {
    const uint4 loc = L.str_meta[t].loc;  // slot-major: t = slot * n_rows + row
    const uint32_t la = loc.y;
    if (la == 0 || la > shape.fast_max) continue;
    uint32_t* tab = peq + t * shape.tab_words;
    uint4* t4 = reinterpret_cast<uint4*>(tab);
    for (uint32_t w = (uint32_t)lane; w < shape.tab_words / 4; w += 32)
      t4[w] = make_uint4(0, 0, 0, 0);
    __syncwarp();
    const uint8_t* a = L.arena + 16ull * loc.x;
    const uint32_t nw = (la + 31u) >> 5;
    for (uint32_t k = 0; k < nw; k++) {
      const uint32_t j = k * 32u + (uint32_t)lane;
      const uint32_t sym = j < la ? (uint32_t)a[j] : 0xffffffffu;
      const unsigned mm = __match_any_sync(kFull, sym);
      if (j < la && lane == __ffs(mm) - 1) tab[sym * shape.s + k] = mm;
    }
    __syncwarp();
  }
}

// Dense variant: 3 CTAs (24 warps) per SM, at most 85 registers per thread.
template <int W>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 3) k_eval(EvalParams P) {
  eval_body<W, false>(P);
}

// Wide variant: 2 CTAs (16 warps) per SM, up to 128 registers per thread, so
// the longer-string scan variants keep their state in registers.
template <int W>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 2) k_eval_wide(EvalParams P) {
  eval_body<W, false>(P);
}

// The same two over rule groups (Rule: "Group evaluation").
template <int W>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 3) k_eval_groups(EvalParams P) {
  eval_body<W, true>(P);
}
template <int W>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 2) k_eval_groups_wide(EvalParams P) {
  eval_body<W, true>(P);
}

namespace {
template <int W>
EvalKernel pick(int wide, bool groups) {
  return groups ? (wide ? k_eval_groups_wide<W> : k_eval_groups<W>)
                : (wide ? k_eval_wide<W> : k_eval<W>);
}
}  // namespace

EvalKernel eval_kernel(int wide, bool groups, uint32_t peq_w) {
  switch (peq_w) {
    case 1: return pick<1>(wide, groups);
    case 2: return pick<2>(wide, groups);
    case 3: return pick<3>(wide, groups);
    case 4: return pick<4>(wide, groups);
    default: return pick<8>(wide, groups);
  }
}

}  // namespace dev
}  // namespace hbx
