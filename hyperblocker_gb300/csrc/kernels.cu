// kernels.cu -- sm_103a kernels of the blocking engine (see kernels.cuh).
#include "kernels.cuh"

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
  for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < S.n_rows;
       row += gridDim.x * blockDim.x) {
    const uint32_t k = row_key(S, R, row);
    keys[row] = k;
    atomicAdd(cnt + k, 1u);
  }
}

__global__ void k_scatter(Side S, const Rule* rules, uint32_t rule, int side) {
  const Rule& R = rules[rule];
  const uint32_t* keys = side ? R.key_r : R.key_l;
  const uint32_t* off = side ? R.off_r : R.off_l;
  uint32_t* cur = side ? R.cur_r : R.cur_l;
  uint32_t* sorted = side ? R.sorted_r : R.sorted_l;
  for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < S.n_rows;
       row += gridDim.x * blockDim.x) {
    const uint32_t k = keys[row];
    sorted[off[k] + atomicAdd(cur + k, 1u)] = row;
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

__device__ __forceinline__ unsigned long long key_items(const Rule& R, uint32_t key,
                                                        uint32_t tile_right,
                                                        unsigned long long* pairs) {
  const uint32_t nl = R.cnt_l[key], nr = R.cnt_r[key];
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
    if (base + k < R.domain) {
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
    v[k] = (base + k < R.domain) ? key_items(R, (uint32_t)(base + k), tile_right, &p) : 0ull;
    sum += v[k];
  }
  unsigned long long ex =
      block_excl_scan<unsigned long long>(sum, s_warp, &s_total) + partial[blockIdx.x];
  for (int k = 0; k < 4; k++) {
    if (base + k < R.domain) R.item_off[base + k] = ex;
    ex += v[k];
    if (base + k + 1 == R.domain) R.item_off[R.domain] = ex;
  }
}

__global__ void k_rule_base(const Rule* rules, uint32_t n_rules, unsigned long long* base) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    unsigned long long acc = 0;
    for (uint32_t r = 0; r < n_rules; r++) {
      base[r] = acc;
      acc += rules[r].item_off[rules[r].domain];
    }
    base[n_rules] = acc;
  }
}

// =====================================================================
// Jaro-Winkler
// =====================================================================

// n = 0 - x over W 32-bit words (two's complement of the W*32-bit number).
template <int W>
struct Neg;
template <>
struct Neg<1> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[1], uint32_t (&n)[1]) {
    n[0] = 0u - x[0];
  }
};
template <>
struct Neg<2> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[2], uint32_t (&n)[2]) {
    asm("sub.cc.u32 %0, %2, %3;\n\tsubc.u32 %1, %2, %4;"
        : "=r"(n[0]), "=r"(n[1])
        : "r"(0u), "r"(x[0]), "r"(x[1]));
  }
};
template <>
struct Neg<3> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[3], uint32_t (&n)[3]) {
    asm("sub.cc.u32 %0, %3, %4;\n\tsubc.cc.u32 %1, %3, %5;\n\tsubc.u32 %2, %3, %6;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]));
  }
};
template <>
struct Neg<4> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[4], uint32_t (&n)[4]) {
    asm("sub.cc.u32 %0, %4, %5;\n\tsubc.cc.u32 %1, %4, %6;\n\tsubc.cc.u32 %2, %4, %7;\n\t"
        "subc.u32 %3, %4, %8;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]));
  }
};
template <>
struct Neg<5> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[5], uint32_t (&n)[5]) {
    asm("sub.cc.u32 %0, %5, %6;\n\tsubc.cc.u32 %1, %5, %7;\n\tsubc.cc.u32 %2, %5, %8;\n\t"
        "subc.cc.u32 %3, %5, %9;\n\tsubc.u32 %4, %5, %10;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3]), "=r"(n[4])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]));
  }
};
template <>
struct Neg<6> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[6], uint32_t (&n)[6]) {
    asm("sub.cc.u32 %0, %6, %7;\n\tsubc.cc.u32 %1, %6, %8;\n\tsubc.cc.u32 %2, %6, %9;\n\t"
        "subc.cc.u32 %3, %6, %10;\n\tsubc.cc.u32 %4, %6, %11;\n\tsubc.u32 %5, %6, %12;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3]), "=r"(n[4]), "=r"(n[5])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]));
  }
};
template <>
struct Neg<7> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[7], uint32_t (&n)[7]) {
    asm("sub.cc.u32 %0, %7, %8;\n\tsubc.cc.u32 %1, %7, %9;\n\tsubc.cc.u32 %2, %7, %10;\n\t"
        "subc.cc.u32 %3, %7, %11;\n\tsubc.cc.u32 %4, %7, %12;\n\tsubc.cc.u32 %5, %7, %13;\n\t"
        "subc.u32 %6, %7, %14;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3]), "=r"(n[4]), "=r"(n[5]), "=r"(n[6])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]),
          "r"(x[6]));
  }
};
template <>
struct Neg<8> {
  __device__ __forceinline__ static void run(const uint32_t (&x)[8], uint32_t (&n)[8]) {
    asm("sub.cc.u32 %0, %8, %9;\n\tsubc.cc.u32 %1, %8, %10;\n\tsubc.cc.u32 %2, %8, %11;\n\t"
        "subc.cc.u32 %3, %8, %12;\n\tsubc.cc.u32 %4, %8, %13;\n\tsubc.cc.u32 %5, %8, %14;\n\t"
        "subc.cc.u32 %6, %8, %15;\n\tsubc.u32 %7, %8, %16;"
        : "=r"(n[0]), "=r"(n[1]), "=r"(n[2]), "=r"(n[3]), "=r"(n[4]), "=r"(n[5]), "=r"(n[6]),
          "=r"(n[7])
        : "r"(0u), "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]), "r"(x[6]),
          "r"(x[7]));
  }
};

template <int S>
__device__ __forceinline__ void load_row(const uint32_t* row, uint32_t (&pe)[S]) {
  if constexpr (S == 1) {
    pe[0] = row[0];
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

// Jaro match count m of left string a (Peq table `tab`, la <= 32*W) and right
// string b: greedy over b's positions i, taking the lowest unmatched position
// of a inside [i - h, i + h]; that greedy is a maximum matching, the same
// count the reference's loops produce when min(la, lb) <= 256.
template <int W>
__device__ __forceinline__ uint32_t bitpar_m(const uint32_t* __restrict__ tab, uint32_t la,
                                             const uint8_t* __restrict__ b, uint32_t lb) {
  constexpr int S = row_words(W);
  const uint32_t h = (min(la, lb) + 1u) >> 1;
  const uint32_t n_iter = min(lb, la + h);
  uint32_t win[W], mt[W];
#pragma unroll
  for (int k = 0; k < W; k++) {
    const int nb = (int)h + 1 - 32 * k;
    win[k] = nb >= 32 ? 0xffffffffu : (nb <= 0 ? 0u : ((1u << nb) - 1u));
    mt[k] = 0u;
  }
  const uint4* bp = reinterpret_cast<const uint4*>(b);
  for (uint32_t base = 0; base < n_iter; base += 16) {
    const uint4 ch = __ldg(bp + (base >> 4));
    const uint32_t wv[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (base + 4u * q >= n_iter) break;
      const uint32_t wd = wv[q];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const uint32_t sym = (wd >> (8 * c)) & 0xffu;
        uint32_t pe[S];
        load_row<S>(tab + sym * S, pe);
        uint32_t x[W], n[W];
#pragma unroll
        for (int k = 0; k < W; k++) x[k] = pe[k] & win[k] & ~mt[k];
        Neg<W>::run(x, n);
#pragma unroll
        for (int k = 0; k < W; k++) mt[k] |= x[k] & n[k];
        const uint32_t grow = (base + 4u * q + (uint32_t)c) < h ? 1u : 0u;
#pragma unroll
        for (int k = W - 1; k > 0; k--) win[k] = __funnelshift_l(win[k - 1], win[k], 1);
        win[0] = (win[0] << 1) | grow;
      }
    }
  }
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < W; k++) m += __popc(mt[k]);
  return m;
}

__device__ __noinline__ uint32_t bitpar_dispatch(uint32_t W, const uint32_t* tab, uint32_t la,
                                                 const uint8_t* b, uint32_t lb) {
  switch (W) {
    case 1: return bitpar_m<1>(tab, la, b, lb);
    case 2: return bitpar_m<2>(tab, la, b, lb);
    case 3: return bitpar_m<3>(tab, la, b, lb);
    case 4: return bitpar_m<4>(tab, la, b, lb);
    case 5: return bitpar_m<5>(tab, la, b, lb);
    case 6: return bitpar_m<6>(tab, la, b, lb);
    case 7: return bitpar_m<7>(tab, la, b, lb);
    default: return bitpar_m<8>(tab, la, b, lb);
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

// Decision from the match count: a float estimate settles every pair whose
// JW lies farther than kDecisionMargin from the threshold (estimate error is
// below 2e-6); the rest take the exact path.
__device__ __forceinline__ bool jw_decide(uint32_t m, uint32_t la, uint32_t lb, const uint8_t* a,
                                          const uint8_t* b, float thr,
                                          unsigned long long* ambiguous) {
  const uint32_t ls = min(la, lb), ll = max(la, lb);
  const float fm = (float)m;
  const float ja = m ? (__fdividef(fm, (float)ls) + __fdividef(fm, (float)ll) + 1.0f) * (1.0f / 3.0f)
                     : 0.0f;
  if (ja >= thr + kDecisionMargin) return true;  // the prefix term is never negative
  const uint32_t p = m ? prefix_len(a, b, ls) : 0u;
  const float jwa = ja + (1.0f - ja) * (0.1f * (float)p);
  if (jwa >= thr + kDecisionMargin) return true;
  if (jwa < thr - kDecisionMargin) return false;
  return jw_exact(m, ls, ll, p, thr, ambiguous);
}

// Algorithmic work of one Jaro-Winkler evaluation in 64-bit word operations:
// 6 per character of the scanned string per 64-bit word of the window string
// (Peq lookup, window AND, ANDNOT matched, lowest-bit isolate x2, OR), the
// prefix compare in 32-bit steps, and 16 for the count and the formula.
__device__ __forceinline__ unsigned long long jw_word_ops(uint32_t la, uint32_t lb) {
  const uint32_t ls = min(la, lb), ll = max(la, lb);
  const uint32_t h = (ls + 1u) >> 1;
  const uint32_t to = min(ls + h, ll);
  return 6ull * to * ((ls + 63u) >> 6) + 2ull * ((ls + 3u) >> 2) + 16ull;
}

// Slow exact similarity check of one pair (any lengths).
__device__ __noinline__ bool sim_pass_slow(const Side& L, const Side& R, uint32_t slot_l,
                                           uint32_t slot_r, uint32_t lrow, uint32_t rrow, float thr,
                                           Counters* ctr) {
  const uint32_t la = L.str_len[(size_t)slot_l * L.n_rows + lrow];
  const uint32_t lb = R.str_len[(size_t)slot_r * R.n_rows + rrow];
  const uint8_t* a = L.arena + 16ull * L.str_off[(size_t)slot_l * L.n_rows + lrow];
  const uint8_t* b = R.arena + 16ull * R.str_off[(size_t)slot_r * R.n_rows + rrow];
  if (la == 0 || lb == 0) return jw_exact(0, la, lb, 0, thr, &ctr->ambiguous);
  const uint32_t mn = min(la, lb);
  if (mn > 256) atomicAdd(&ctr->long_pairs, 1ull);
  atomicAdd(&ctr->jw_word_ops, jw_word_ops(la, lb));
  const uint32_t m = jaro_m_ref(a, la, b, lb);
  const uint32_t p = prefix_len(a, b, mn);
  return jw_exact(m, mn, max(la, lb), p, thr, &ctr->ambiguous);
}

// Does an earlier rule (index < r) also match (lrow, rrow)?  Then that rule
// reports the pair, and this one must not report it again.
__device__ __noinline__ bool earlier_rule_matches(const EvalParams& P, uint32_t r, uint32_t lrow,
                                                  uint32_t rrow) {
  for (uint32_t j = 0; j < r; j++) {
    const Rule& Q = P.rules[j];
    bool eq = true;
    if (Q.composite) {
      eq = P.L.comp_codes[(size_t)Q.comp_index * P.L.n_rows + lrow] ==
           P.R.comp_codes[(size_t)Q.comp_index * P.R.n_rows + rrow];
    } else {
      for (uint32_t e = 0; e < Q.n_eq && eq; e++)
        eq = P.L.eq_codes[(size_t)Q.eq_slot[e] * P.L.n_rows + lrow] ==
             P.R.eq_codes[(size_t)Q.eq_slot[e] * P.R.n_rows + rrow];
    }
    if (!eq) continue;
    bool all = true;
    for (uint32_t s = 0; s < Q.n_sim && all; s++)
      all = sim_pass_slow(P.L, P.R, Q.sim_l[s], Q.sim_r[s], lrow, rrow, Q.thr[s], P.ctr);
    if (all) return true;
  }
  return false;
}

// Peq table of the warp's left string: row `sym` (stride S words) has bit j of
// word k set when a[32k + j] == sym.  Built with __match_any_sync: lanes that
// hold the same symbol agree on the mask, the lowest of them stores it.
__device__ __forceinline__ void build_peq(uint32_t* tab, uint32_t S, uint32_t n_symbols,
                                          const uint8_t* a, uint32_t la, int lane) {
  const uint32_t words = n_symbols * S;
  for (uint32_t w = (uint32_t)lane; w < words; w += 32) tab[w] = 0u;
  __syncwarp();
  const uint32_t W = (la + 31u) >> 5;
  for (uint32_t k = 0; k < W; k++) {
    const uint32_t j = k * 32u + (uint32_t)lane;
    const uint32_t sym = j < la ? (uint32_t)a[j] : 0xffffffffu;
    const unsigned mm = __match_any_sync(kFull, sym);
    if (j < la && lane == __ffs(mm) - 1) tab[sym * S + k] = mm;
  }
  __syncwarp();
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

__global__ void __launch_bounds__(kWarpsPerCta * 32) k_eval(EvalParams P) {
  extern __shared__ __align__(16) uint32_t smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  uint32_t* region = smem + (size_t)warp * P.warp_words;
  const unsigned long long end = P.range_is_device ? P.rule_item_base[P.n_rules] : P.item_end;
  const long long t_start = clock64();
  // warp-level cache of the last (rule, key) item range
  uint32_t c_rule = 0xffffffffu, c_key = 0;
  unsigned long long c_lo = 1, c_hi = 0;
  unsigned long long done = 0;
  unsigned long long ops = 0;

  for (;;) {
    unsigned long long it = 0;
    if (lane == 0) it = P.item_begin + atomicAdd(&P.ctr->work_next, 1ull);
    it = __shfl_sync(kFull, it, 0);
    if (it >= end) break;
    if (P.watchdog_cycles && (unsigned long long)(clock64() - t_start) > P.watchdog_cycles) {
      if (lane == 0) atomicAdd(&P.ctr->watchdog_trips, 1ull);
      break;
    }
    uint32_t r = 0;
    while (r + 1 < P.n_rules && P.rule_item_base[r + 1] <= it) r++;
    const Rule& R = P.rules[r];
    const unsigned long long local = it - P.rule_item_base[r];
    if (r != c_rule || local < c_lo || local >= c_hi) {
      c_rule = r;
      c_key = find_key(R.item_off, R.domain, local);
      c_lo = R.item_off[c_key];
      c_hi = R.item_off[c_key + 1];
    }
    const uint32_t key = c_key;
    const unsigned long long in_key = local - c_lo;
    const uint32_t nl = R.cnt_l[key], nr = R.cnt_r[key];
    const uint32_t ri = (uint32_t)(in_key / nl);
    const uint32_t li = (uint32_t)(in_key - (unsigned long long)ri * nl);
    const uint32_t lrow = R.sorted_l[R.off_l[key] + li];
    const uint32_t rb0 = R.off_r[key] + ri * P.tile_right;
    const uint32_t rb1 = min(rb0 + P.tile_right, R.off_r[key] + nr);

    uint32_t built = 0;
    for (uint32_t rb = rb0; rb < rb1; rb += 32) {
      const uint32_t idx = rb + (uint32_t)lane;
      const bool act = idx < rb1;
      const uint32_t rrow = act ? R.sorted_r[idx] : 0u;
      bool pass = act;
      for (uint32_t s = 0; s < R.n_sim; s++) {
        if (!__ballot_sync(kFull, pass)) break;
        const uint32_t sl = R.sim_l[s], sr = R.sim_r[s];
        const uint32_t la = P.L.str_len[(size_t)sl * P.L.n_rows + lrow];
        const uint8_t* a = P.L.arena + 16ull * P.L.str_off[(size_t)sl * P.L.n_rows + lrow];
        const uint32_t W = (la + 31u) >> 5;
        const bool fast = la > 0 && la <= 256 && R.peq_rows_words[s] >= (uint32_t)row_words((int)W);
        uint32_t* tab = region + R.peq_off[s];
        if (fast && !((built >> s) & 1u)) {
          build_peq(tab, (uint32_t)row_words((int)W), P.n_symbols, a, la, lane);
          built |= 1u << s;
        }
        if (pass) {
          if (fast) {
            const uint32_t lb = P.R.str_len[(size_t)sr * P.R.n_rows + rrow];
            const uint8_t* b = P.R.arena + 16ull * P.R.str_off[(size_t)sr * P.R.n_rows + rrow];
            if (lb == 0) {
              pass = jw_exact(0, la, 0, 0, R.thr[s], &P.ctr->ambiguous);
            } else {
              const uint32_t m = bitpar_dispatch(W, tab, la, b, lb);
              ops += jw_word_ops(la, lb);
              pass = jw_decide(m, la, lb, a, b, R.thr[s], &P.ctr->ambiguous);
            }
          } else {
            pass = sim_pass_slow(P.L, P.R, sl, sr, lrow, rrow, R.thr[s], P.ctr);
          }
        }
      }
      if (pass && r > 0) pass = !earlier_rule_matches(P, r, lrow, rrow);
      const unsigned mask = __ballot_sync(kFull, pass);
      if (mask) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&P.ctr->out_count, (unsigned long long)__popc(mask));
        base = __shfl_sync(kFull, base, 0);
        if (pass) {
          const unsigned long long pos = base + __popc(mask & ((1u << lane) - 1u));
          if (pos < P.capacity) {
            P.out_l[pos] = lrow;
            P.out_r[pos] = rrow;
          }
        }
      }
    }
    done++;
  }
  if (lane == 0 && done) atomicAdd(&P.ctr->items_done, done);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ops += __shfl_down_sync(kFull, ops, o);
  if (lane == 0 && ops) atomicAdd(&P.ctr->jw_word_ops, ops);
}

}  // namespace dev
}  // namespace hbx
