// ingest.cu -- device-side encoding of two host tables (see ingest.h).
//
// Only the columns a plan reads are copied: per column its cell bytes and
// int64 cell offsets, as the host table holds them.  Then, on the device:
//   k_buckets        partition bucket of every row: std::hash of the
//                    partition cell (and of the prefix cell's first byte)
//                    modulo n_partitions, exactly as data_mngr.h:150-202
//                    computes it; a per-side histogram of buckets;
//   k_pairs_covered  sum over partitions of |L_p| * |R_p|;
//   dictionaries     per equality slot, both tables' cells go into one
//                    open-addressing table keyed by the 64-bit hash of the
//                    cell (up to its first NUL, as equalities_kernel
//                    compares); the occupied slots, numbered by a scan, are
//                    the codes; every cell is then compared byte by byte
//                    with its slot's representative (the lowest row holding
//                    that hash), so a hash collision is always detected;
//   k_byte_hist +    the frequency-ordered symbol alphabet of the string
//   k_symbol_map     columns (ties by byte value), as the host encoder;
//   k_units + scan + the arenas: string k of slot s starts at the 16-byte
//   k_pack           unit given by the scan of the padded lengths in
//                    (slot, row) order, one warp per string translating
//                    bytes to symbols and writing the string's metadata.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "ingest.h"
#include "kernels.cuh"
#include "std_hash.h"

namespace hbx {
namespace ing {

constexpr uint32_t kSharedHist = 4096;  // partitions counted in shared memory

__global__ void k_buckets(ColDev part, uint32_t use_part, ColDev pre, uint32_t use_pre,
                          unsigned long long n_part, uint32_t n, uint32_t* bucket,
                          unsigned long long* hist) {
  extern __shared__ uint32_t s_hist[];
  const bool sh = n_part <= kSharedHist;
  if (sh)
    for (uint32_t k = threadIdx.x; k < n_part; k += blockDim.x) s_hist[k] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned long long b = 0;
    if (use_part) {
      const int64_t a = part.off[i];
      const uint64_t len = (uint64_t)(part.off[i + 1] - a);
      b = std_hash_bytes(part.bytes + a, len) % n_part;
    }
    if (use_pre) {
      const int64_t a = pre.off[i];
      const uint64_t len = (uint64_t)(pre.off[i + 1] - a);
      if (len > 2) {
        const unsigned long long two_d = (std_hash_bytes(pre.bytes + a, 1) + b) % n_part;
        b = (b + two_d) % n_part;
      }
    }
    bucket[i] = (uint32_t)b;
    if (sh)
      atomicAdd(&s_hist[b], 1u);
    else
      atomicAdd(&hist[b], 1ull);
  }
  __syncthreads();
  if (sh)
    for (uint32_t k = threadIdx.x; k < n_part; k += blockDim.x)
      if (s_hist[k]) atomicAdd(&hist[k], (unsigned long long)s_hist[k]);
}

__global__ void k_pairs_covered(const unsigned long long* hl, const unsigned long long* hr,
                                unsigned long long n_part, unsigned long long* sum) {
  unsigned long long pairs = 0, used = 0;
  for (unsigned long long p = blockIdx.x * blockDim.x + threadIdx.x; p < n_part;
       p += gridDim.x * blockDim.x) {
    pairs += hl[p] * hr[p];
    used += (hl[p] && hr[p]) ? 1ull : 0ull;
  }
  for (int o = 16; o; o >>= 1) {
    pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    used += __shfl_xor_sync(0xffffffffu, used, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (pairs) atomicAdd(&sum[kSumPairs], pairs);
    if (used) atomicAdd(&sum[kSumUsed], used);
  }
}

__global__ void k_dict_insert(ColDev c, uint32_t n, uint32_t gid_base, unsigned long long* keys,
                              uint32_t* rep, uint32_t mask, uint32_t* row_slot,
                              unsigned long long* sum, unsigned long long seed) {
  // seed bit 63 set: the test build of kDictSeed that keeps 3 bits of the hash
  const unsigned long long hmask = (seed >> 63) ? 7ull : ~0ull;
  seed &= ~(1ull << 63);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int64_t a;
    const uint32_t len = cell_len(c, i, &a);
    unsigned long long h = hash_bytes_seeded(c.bytes + a, len, seed) & hmask;
    if (h == kEmpty) h = kEmpty - 1;  // the empty marker; verification keeps this exact
    uint32_t slot = (uint32_t)(h ^ (h >> 32)) & mask;
    bool placed = false;
    for (uint32_t probe = 0; probe <= mask; probe++) {
      const unsigned long long prev = atomicCAS(&keys[slot], kEmpty, h);
      if (prev == kEmpty || prev == h) {
        atomicMin(&rep[slot], gid_base + i);
        row_slot[i] = slot;
        placed = true;
        break;
      }
      slot = (slot + 1) & mask;
    }
    if (!placed) {
      row_slot[i] = 0;
      atomicOr(&sum[kSumFlags], (unsigned long long)kFlagTableFull);
    }
  }
}

__global__ void k_occupied(const unsigned long long* keys, uint32_t cap, uint32_t* occ) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < cap; s += gridDim.x * blockDim.x)
    occ[s] = keys[s] != kEmpty ? 1u : 0u;
}

// code of each row, and the exact check against the slot's representative
// (row gid < n_left: left table row gid, else right table row gid - n_left)
__global__ void k_dict_assign(ColDev c, uint32_t n, uint32_t gid_base, const uint32_t* row_slot,
                              const uint32_t* code, const uint32_t* rep, ColDev cl, ColDev cr,
                              uint32_t n_left, int32_t* out, unsigned long long* sum) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t slot = row_slot[i];
    out[i] = (int32_t)code[slot];
    const uint32_t r = rep[slot];
    if (r == gid_base + i) continue;
    int64_t a, b;
    const uint32_t la = cell_len(c, i, &a);
    const uint32_t lb = r < n_left ? cell_len(cl, r, &b) : cell_len(cr, r - n_left, &b);
    const uint8_t* pb = r < n_left ? cl.bytes : cr.bytes;
    bool same = la == lb;
    for (uint32_t k = 0; same && k < la; k++) same = c.bytes[a + k] == pb[b + k];
    if (!same) atomicOr(&sum[kSumFlags], (unsigned long long)kFlagCollision);
  }
}

// Composite join keys.  Row i's tuple: its bucket, then its dictionary code
// of each of the rule's equality slots, as 4-byte little-endian words (a
// fixed-width cell for the dictionary kernels).
struct TupleSlots {
  uint32_t k;
  uint32_t slot[dev::kMaxEq];
};
__global__ void k_tuples(const uint32_t* bucket, const int32_t* eq, uint32_t n, TupleSlots ts,
                         uint32_t* out) {
  const uint32_t w = ts.k + 1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t* o = out + (size_t)i * w;
    o[0] = bucket[i];
    for (uint32_t j = 0; j < ts.k; j++) o[1 + j] = (uint32_t)eq[(size_t)ts.slot[j] * n + i];
  }
}

// The bucket of every tuple code (the bucket of its slot's representative
// row), and the tuples per bucket.
__global__ void k_code_bucket(const unsigned long long* keys, const uint32_t* code,
                              const uint32_t* rep, uint32_t cap, const uint32_t* bucket_l,
                              const uint32_t* bucket_r, uint32_t n_left, uint32_t* code_bucket,
                              uint32_t* per_bucket) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < cap; s += gridDim.x * blockDim.x) {
    if (keys[s] == kEmpty) continue;
    const uint32_t r = rep[s];
    const uint32_t b = r < n_left ? bucket_l[r] : bucket_r[r - n_left];
    code_bucket[code[s]] = b;
    atomicAdd(per_bucket + b, 1u);
  }
}

// Dense ids grouped by bucket: code c gets start[bucket] + its rank there
// (ranks in any order; only equality and the grouping matter).
__global__ void k_code_remap(const uint32_t* code_bucket, uint32_t n_codes, const uint32_t* start,
                             uint32_t* cursor, uint32_t* remap) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n_codes; c += gridDim.x * blockDim.x) {
    const uint32_t b = code_bucket[c];
    remap[c] = start[b] + atomicAdd(cursor + b, 1u);
  }
}

__global__ void k_apply_remap(const int32_t* codes, uint32_t n, const uint32_t* remap, int32_t* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = (int32_t)remap[(uint32_t)codes[i]];
}

// dst = scan[n - 1] + in[n - 1] (+ extra): the total of an exclusive scan
__global__ void k_scan_total(const uint32_t* scan, const uint32_t* in, uint32_t n,
                             unsigned long long extra, unsigned long long* dst) {
  if (threadIdx.x == 0 && blockIdx.x == 0)
    *dst = (n ? (unsigned long long)scan[n - 1] + in[n - 1] : 0ull) + extra;
}

// byte counts of a string column (bytes up to each cell's first NUL)
__global__ void k_byte_hist(ColDev c, uint32_t n, unsigned long long* hist) {
  __shared__ uint32_t s[8][256];
  const uint32_t warp = threadIdx.x >> 5;
  for (uint32_t k = threadIdx.x; k < 8 * 256; k += blockDim.x) (&s[0][0])[k] = 0;
  __syncthreads();
  if (!c.has_nul && ((uintptr_t)c.bytes & 15) == 0) {
    const uint64_t total = (uint64_t)c.off[n];  // cells are contiguous from byte 0
    const uint64_t chunks = (total + 15) / 16;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < chunks;
         k += (uint64_t)gridDim.x * blockDim.x) {
      const uint64_t b0 = k * 16;
      if (b0 + 16 <= total) {
        const uint4 v = *reinterpret_cast<const uint4*>(c.bytes + b0);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
          for (int j = 0; j < 4; j++) atomicAdd(&s[warp][(w[q] >> (8 * j)) & 0xffu], 1u);
      } else {
        for (uint64_t b = b0; b < total; b++) atomicAdd(&s[warp][c.bytes[b]], 1u);
      }
    }
  } else {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      int64_t a;
      const uint32_t len = cell_len(c, i, &a);
      for (uint32_t k = 0; k < len; k++) atomicAdd(&s[warp][c.bytes[a + k]], 1u);
    }
  }
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < 256; b += blockDim.x) {
    uint32_t t = 0;
    for (int w = 0; w < 8; w++) t += s[w][b];
    if (t) atomicAdd(&hist[b], (unsigned long long)t);
  }
}

// symbol of byte b = 1 + (bytes more frequent than b, or as frequent and
// smaller): the host encoder's stable sort by descending frequency
__global__ void k_symbol_map(const unsigned long long* hist, uint8_t* sym,
                             unsigned long long* sum) {
  __shared__ unsigned long long f[256];
  const uint32_t b = threadIdx.x;
  f[b] = b ? hist[b] : 0ull;
  __syncthreads();
  uint32_t rank = 0, nz = 0;
  for (uint32_t k = 1; k < 256; k++) {
    const unsigned long long fk = f[k];
    if (!fk) continue;
    nz++;
    if (fk > f[b] || (fk == f[b] && k < b)) rank++;
  }
  sym[b] = (b && f[b]) ? (uint8_t)(rank + 1) : (uint8_t)0;
  if (b == 0) sum[kSumSymbols] = nz + 1;
}

__global__ void k_units(ColDev c, uint32_t n, uint32_t* units) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int64_t a;
    units[i] = (cell_len(c, i, &a) + 15u) / 16u;
  }
}

// One warp per string: symbols into the arena at unit off16[i], metadata
// {offset / 16, length, 0, 0} + the first 16 symbols + the count signature
// (dev::StrMeta); the longest length goes to *maxlen.  256 threads per block.
__global__ void k_pack(ColDev c, uint32_t n, const uint32_t* off16, const uint8_t* sym_g,
                       uint8_t* arena, dev::StrMeta* meta, unsigned long long* maxlen) {
  __shared__ uint8_t sym[256];
  __shared__ uint32_t s_cnt[8][dev::kSigBuckets];
  for (uint32_t k = threadIdx.x; k < 256; k += blockDim.x) sym[k] = sym_g[k];
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  uint32_t* cnt = s_cnt[threadIdx.x >> 5];
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  uint32_t mx = 0;
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const int64_t a = c.off[i];
    const uint32_t full = (uint32_t)(c.off[i + 1] - a);
    uint32_t len = full;
    if (c.has_nul) {
      for (uint32_t base = 0; base < full; base += 32) {
        const uint32_t z = __ballot_sync(0xffffffffu, base + lane < full && c.bytes[a + base + lane] == 0);
        if (z) {
          len = base + (uint32_t)__ffs(z) - 1;
          break;
        }
      }
    }
    const uint64_t pos = (uint64_t)off16[i] * 16;
    cnt[lane] = 0;
    __syncwarp();
    for (uint32_t base = 0; base < len; base += 32) {
      const uint32_t j = base + lane;
      const uint32_t v = j < len ? sym[c.bytes[a + j]] : 0u;
      if (j < len) arena[pos + j] = (uint8_t)v;
      // one add per (bucket, chunk): the lowest lane of each bucket group
      const uint32_t b = v ? dev::sig_bucket(v) : 0xffffffffu;
      const unsigned grp = __match_any_sync(0xffffffffu, b);
      if (v && lane == (uint32_t)(__ffs(grp) - 1)) cnt[b] += (uint32_t)__popc(grp);
      __syncwarp();
    }
    __syncwarp();
    uint32_t sw = 0;  // signature word `lane` (lanes 0-7)
    if (lane < 8) {
      if (len > dev::kSigMaxLen) {
        sw = 0xffffffffu;
      } else {
        for (int k = 0; k < 4; k++) sw |= cnt[4 * lane + k] << (8 * k);
      }
    }
    const uint32_t s = (lane < 16 && lane < len) ? sym[c.bytes[a + lane]] : 0u;
    uint32_t v = s << (8 * (lane & 3));
    v |= __shfl_xor_sync(0xffffffffu, v, 1);
    v |= __shfl_xor_sync(0xffffffffu, v, 2);
    const uint32_t w0 = __shfl_sync(0xffffffffu, v, 0), w1 = __shfl_sync(0xffffffffu, v, 4);
    const uint32_t w2 = __shfl_sync(0xffffffffu, v, 8), w3 = __shfl_sync(0xffffffffu, v, 12);
    uint32_t g[8];
#pragma unroll
    for (int k = 0; k < 8; k++) g[k] = __shfl_sync(0xffffffffu, sw, k);
    if (lane == 0) {
      dev::StrMeta m;
      m.loc = make_uint4(off16[i], len, 0u, 0u);
      m.head = make_uint4(w0, w1, w2, w3);
      m.sig[0] = make_uint4(g[0], g[1], g[2], g[3]);
      m.sig[1] = make_uint4(g[4], g[5], g[6], g[7]);
      meta[i] = m;
      mx = max(mx, len);
    }
    __syncwarp();
  }
  if (lane == 0 && mx) atomicMax(maxlen, (unsigned long long)mx);
}

}  // namespace ing

int grid_for(uint64_t n, int n_sm, int per_sm) {
  const uint64_t g = (n + 255) / 256;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)n_sm * per_sm));
}

void check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) fail(HBX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void scan_u32(const uint32_t* in, uint32_t n, uint32_t* out, cudaStream_t st) {
  const uint32_t nb = (n + dev::kScanChunk - 1) / dev::kScanChunk;
  DBuf<uint32_t> part;
  part.alloc(nb);
  dev::k_scan_partial_u32<<<nb, 1024, 0, st>>>(in, n, part.p);
  dev::k_scan_top_u32<<<1, 1024, 0, st>>>(part.p, nb);
  dev::k_scan_final_u32<<<nb, 1024, 0, st>>>(in, n, part.p, out);
  check_launch("ingest scan");
}

namespace {

struct DevCol {
  DBuf<uint8_t> bytes;
  DBuf<int64_t> off;
  uint32_t has_nul = 0;
};

}  // namespace

std::vector<uint32_t> bucket_rows(const Table& t, int part_col, int64_t prefix_idx,
                                  uint64_t n_part, int n_sm, cudaStream_t st) {
  const uint64_t n = (uint64_t)t.n_rows;
  std::vector<uint32_t> out(n, 0);
  const int pre = prefix_idx != INT_MAX ? (int)prefix_idx : -1;
  if (!n || (part_col < 0 && pre < 0)) return out;
  constexpr uint64_t kChunk = 1ull << 22;
  DBuf<unsigned long long> hist;
  hist.alloc(n_part);
  DBuf<uint32_t> d_out;
  d_out.alloc(std::min(n, kChunk));
  const size_t hist_smem = n_part <= ing::kSharedHist ? n_part * sizeof(uint32_t) : 0;
  for (uint64_t r0 = 0; r0 < n; r0 += kChunk) {
    const uint64_t r1 = std::min(n, r0 + kChunk), m = r1 - r0;
    DBuf<uint8_t> b[2];
    DBuf<int64_t> o[2];
    ing::ColDev view[2] = {{nullptr, nullptr, 0}, {nullptr, nullptr, 0}};
    const int cols[2] = {part_col, pre};
    for (int k = 0; k < 2; k++) {
      if (cols[k] < 0) continue;
      const Column& c = t.cols[(size_t)cols[k]];
      const int64_t a = c.off[r0], z = c.off[r1];
      std::vector<int64_t> off(m + 1);
      for (uint64_t i = 0; i <= m; i++) off[i] = c.off[r0 + i] - a;
      b[k].alloc(std::max<int64_t>(z - a, 16));
      o[k].alloc(m + 1);
      if (z > a)
        HBX_CUDA(cudaMemcpyAsync(b[k].p, c.bytes.data() + a, (size_t)(z - a), cudaMemcpyHostToDevice, st));
      HBX_CUDA(cudaMemcpyAsync(o[k].p, off.data(), (m + 1) * 8, cudaMemcpyHostToDevice, st));
      HBX_CUDA(cudaStreamSynchronize(st));  // off is a local vector
      view[k] = ing::ColDev{b[k].p, o[k].p, 0};
    }
    ing::k_buckets<<<grid_for(m, n_sm, 4), 256, hist_smem, st>>>(
        view[0], part_col >= 0 ? 1u : 0u, view[1], pre >= 0 ? 1u : 0u, n_part, (uint32_t)m, d_out.p,
        hist.p);
    check_launch("bucket_rows");
    HBX_CUDA(cudaMemcpyAsync(out.data() + r0, d_out.p, m * 4, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaStreamSynchronize(st));
  }
  return out;
}

void pin_table(const hbx_table* ct) {
  hbx_table* t = const_cast<hbx_table*>(ct);
  std::lock_guard<std::mutex> lock(t->pin_mu);
  if (t->pin_tried) return;
  t->pin_tried = true;
  auto pin = [&](const void* p, size_t bytes) {
    if (!p || bytes < (1u << 16)) return;  // small buffers copy fast enough pageable
    if (cudaHostRegister(const_cast<void*>(p), bytes, cudaHostRegisterPortable) == cudaSuccess)
      t->pinned.push_back(const_cast<void*>(p));
    else
      cudaGetLastError();  // not fatal: the copy stages through the driver
  };
  for (const Column& c : t->t.cols) {
    pin(c.bytes.data(), c.bytes.size());
    pin(c.off.data(), c.off.size() * sizeof(int64_t));
  }
}

void unpin_table(hbx_table* t) {
  std::lock_guard<std::mutex> lock(t->pin_mu);
  for (void* p : t->pinned) cudaHostUnregister(p);
  t->pinned.clear();
}

bool device_encode(const hbx_table* left, const hbx_table* right, Encoded* Ep, SideBufs* LB,
                   SideBufs* RB, int n_sm, cudaStream_t st, uint64_t* h2d, std::string* why,
                   bool pin) {
  Encoded& E = *Ep;
  const Table& TL = left->t;
  const Table& TR = right->t;
  const uint32_t nL = (uint32_t)E.L.n_rows, nR = (uint32_t)E.R.n_rows;
  const uint64_t n_part = E.n_partitions;
  if ((uint64_t)nL + nR > (1ull << 30)) {
    *why = "more than 2^30 rows in the two tables";
    return false;
  }
  if (pin) {
    pin_table(left);
    pin_table(right);
  }
  *h2d = 0;

  // ---- copy the columns the plan reads
  std::map<int, DevCol> cols_l, cols_r;
  auto need = [&](const Table& t, std::map<int, DevCol>& m, int col) {
    if (col < 0 || m.count(col)) return;
    const Column& c = t.cols[(size_t)col];
    DevCol& d = m[col];
    d.bytes.alloc(std::max<size_t>(c.bytes.size(), 16));
    d.off.alloc(c.off.size());
    if (!c.bytes.empty())
      HBX_CUDA(cudaMemcpyAsync(d.bytes.p, c.bytes.data(), c.bytes.size(), cudaMemcpyHostToDevice, st));
    HBX_CUDA(cudaMemcpyAsync(d.off.p, c.off.data(), c.off.size() * sizeof(int64_t),
                             cudaMemcpyHostToDevice, st));
    d.has_nul = c.has_nul ? 1u : 0u;
    *h2d += c.bytes.size() + c.off.size() * sizeof(int64_t);
  };
  const int pre = E.prefix_idx != INT_MAX ? (int)E.prefix_idx : -1;
  for (int col : {E.part_col, pre}) {
    need(TL, cols_l, col);
    need(TR, cols_r, col);
  }
  for (auto& s : E.eq_slots) {
    need(TL, cols_l, s.first);
    need(TR, cols_r, s.second);
  }
  for (int col : E.L.str_col) need(TL, cols_l, col);
  for (int col : E.R.str_col) need(TR, cols_r, col);
  auto view = [](std::map<int, DevCol>& m, int col) {
    if (col < 0) return ing::ColDev{nullptr, nullptr, 0};
    const DevCol& d = m.at(col);
    return ing::ColDev{d.bytes.p, d.off.p, d.has_nul};
  };

  const size_t n_eq = E.eq_slots.size();
  const size_t n_sl = E.L.str_col.size(), n_sr = E.R.str_col.size();
  // summary: fixed words, eq card, maxlen L, maxlen R, arena units L, R
  const size_t i_card = ing::kSumFixed, i_mxl = i_card + n_eq, i_mxr = i_mxl + n_sl,
               i_units = i_mxr + n_sr, n_sum = i_units + 2;
  DBuf<unsigned long long> sum;
  sum.alloc(n_sum);
  HBX_CUDA(cudaMemsetAsync(sum.p, 0, n_sum * sizeof(unsigned long long), st));

  // ---- partition buckets
  DBuf<unsigned long long> hist;
  hist.alloc(2 * n_part);
  HBX_CUDA(cudaMemsetAsync(hist.p, 0, 2 * n_part * sizeof(unsigned long long), st));
  const size_t hist_smem = n_part <= ing::kSharedHist ? n_part * sizeof(uint32_t) : 0;
  auto buckets = [&](std::map<int, DevCol>& m, uint32_t n, SideBufs* B, unsigned long long* h) {
    B->bucket.alloc(n);
    if (!n) return;
    ing::k_buckets<<<grid_for(n, n_sm, 4), 256, hist_smem, st>>>(
        view(m, E.part_col), E.part_col >= 0 ? 1u : 0u, view(m, pre), pre >= 0 ? 1u : 0u, n_part,
        n, B->bucket.p, h);
  };
  buckets(cols_l, nL, LB, hist.p);
  buckets(cols_r, nR, RB, hist.p + n_part);
  ing::k_pairs_covered<<<grid_for(n_part, n_sm, 2), 256, 0, st>>>(hist.p, hist.p + n_part, n_part,
                                                                   sum.p);
  check_launch("ingest buckets");

  // ---- joint dictionaries (rebuilt with a fresh seed after a collision,
  // below)
  LB->eq.alloc(std::max<size_t>(n_eq * nL, 1));
  RB->eq.alloc(std::max<size_t>(n_eq * nR, 1));
  uint32_t cap = 1024;
  while (cap < 2ull * ((uint64_t)nL + nR)) cap <<= 1;
  DBuf<unsigned long long> keys;
  DBuf<uint32_t> rep, occ, code, slot_l, slot_r;
  keys.alloc(cap);
  rep.alloc(cap);
  occ.alloc(cap);
  code.alloc(cap);
  slot_l.alloc(std::max<uint32_t>(nL, 1));
  slot_r.alloc(std::max<uint32_t>(nR, 1));
  // One joint dictionary of columns cl (left) and cr (right): codes into
  // out_l / out_r, the number of distinct cells into *card_sum.
  auto dictionary = [&](const ing::ColDev& cl, const ing::ColDev& cr, int32_t* out_l,
                        int32_t* out_r, unsigned long long* card_sum, unsigned long long seed) {
    HBX_CUDA(cudaMemsetAsync(keys.p, 0xff, (size_t)cap * sizeof(unsigned long long), st));
    HBX_CUDA(cudaMemsetAsync(rep.p, 0xff, (size_t)cap * sizeof(uint32_t), st));
    if (nL)
      ing::k_dict_insert<<<grid_for(nL, n_sm), 256, 0, st>>>(cl, nL, 0, keys.p, rep.p, cap - 1,
                                                             slot_l.p, sum.p, seed);
    if (nR)
      ing::k_dict_insert<<<grid_for(nR, n_sm), 256, 0, st>>>(cr, nR, nL, keys.p, rep.p, cap - 1,
                                                             slot_r.p, sum.p, seed);
    ing::k_occupied<<<grid_for(cap, n_sm), 256, 0, st>>>(keys.p, cap, occ.p);
    scan_u32(occ.p, cap, code.p, st);
    if (nL)
      ing::k_dict_assign<<<grid_for(nL, n_sm), 256, 0, st>>>(cl, nL, 0, slot_l.p, code.p, rep.p,
                                                             cl, cr, nL, out_l, sum.p);
    if (nR)
      ing::k_dict_assign<<<grid_for(nR, n_sm), 256, 0, st>>>(cr, nR, nL, slot_r.p, code.p, rep.p,
                                                             cl, cr, nL, out_r, sum.p);
    ing::k_scan_total<<<1, 32, 0, st>>>(code.p, occ.p, cap, 0, card_sum);
    check_launch("ingest dictionary");
  };
  const char* collide_env = std::getenv("HBX_TEST_DICT_COLLIDE");
  const bool collide_test = collide_env && std::strcmp(collide_env, "1") == 0;
  // attempt k hashes with seed kDictSeed + k; the test build of attempt 0
  // keeps 3 bits of each hash (bit 63 of the seed word asks for that)
  auto seed_of = [&](int attempt) {
    unsigned long long sd = kDictSeed + (unsigned long long)attempt;
    if (collide_test && attempt == 0) sd |= 1ull << 63;
    return sd;
  };
  auto eq_dictionaries = [&](unsigned long long seed) {
    for (size_t k = 0; k < n_eq; k++)
      dictionary(view(cols_l, E.eq_slots[k].first), view(cols_r, E.eq_slots[k].second),
                 LB->eq.p + k * nL, RB->eq.p + k * nR, sum.p + i_card + k, seed);
  };
  eq_dictionaries(seed_of(0));

  // ---- symbol alphabet
  DBuf<unsigned long long> bhist;
  DBuf<uint8_t> sym;
  bhist.alloc(256);
  sym.alloc(256);
  HBX_CUDA(cudaMemsetAsync(bhist.p, 0, 256 * sizeof(unsigned long long), st));
  auto byte_hist = [&](std::map<int, DevCol>& m, const std::vector<int>& str_col, uint32_t n,
                       const Table& t) {
    for (int col : str_col) {
      const uint64_t bytes = t.cols[(size_t)col].bytes.size();
      const uint64_t work = t.cols[(size_t)col].has_nul ? n : (bytes + 15) / 16;
      if (n) ing::k_byte_hist<<<grid_for(work, n_sm, 4), 256, 0, st>>>(view(m, col), n, bhist.p);
    }
  };
  byte_hist(cols_l, E.L.str_col, nL, TL);
  byte_hist(cols_r, E.R.str_col, nR, TR);
  ing::k_symbol_map<<<1, 256, 0, st>>>(bhist.p, sym.p, sum.p);
  check_launch("ingest symbols");

  // ---- arenas and string metadata
  auto arenas = [&](std::map<int, DevCol>& m, const std::vector<int>& str_col, uint32_t n,
                    const Table& t, SideBufs* B, size_t i_mx, size_t i_un) {
    const size_t ns = str_col.size();
    uint64_t bound = 16;  // the zero block at the end
    for (int col : str_col) bound += t.cols[(size_t)col].bytes.size() + 15ull * n;
    bound = (bound + 15) / 16 * 16;
    if (bound / 16 > UINT32_MAX) fail(HBX_ERR_UNSUPPORTED, "string arena above 64 GiB");
    B->arena.alloc(bound);
    HBX_CUDA(cudaMemsetAsync(B->arena.p, 0, bound, st));
    B->meta.alloc(std::max<size_t>(ns * n, 1));
    if (!ns || !n) return;
    DBuf<uint32_t> units, off16;
    units.alloc(ns * n);
    off16.alloc(ns * n);
    for (size_t s = 0; s < ns; s++)
      ing::k_units<<<grid_for(n, n_sm), 256, 0, st>>>(view(m, str_col[s]), n, units.p + s * n);
    if ((uint64_t)ns * n > UINT32_MAX) fail(HBX_ERR_UNSUPPORTED, "more than 2^32 strings");
    scan_u32(units.p, (uint32_t)(ns * n), off16.p, st);
    ing::k_scan_total<<<1, 32, 0, st>>>(off16.p, units.p, (uint32_t)(ns * n), 1, sum.p + i_un);
    for (size_t s = 0; s < ns; s++)
      ing::k_pack<<<grid_for((uint64_t)n * 32, n_sm), 256, 0, st>>>(
          view(m, str_col[s]), n, off16.p + s * n, sym.p, B->arena.p, B->meta.p + s * n,
          sum.p + i_mx + s);
    check_launch("ingest arenas");
  };
  arenas(cols_l, E.L.str_col, nL, TL, LB, i_mxl, i_units);
  arenas(cols_r, E.R.str_col, nR, TR, RB, i_mxr, i_units + 1);

  // ---- summary
  constexpr int kMaxAttempts = 4;
  std::vector<unsigned long long> h(n_sum);
  auto read_summary = [&]() {
    HBX_CUDA(cudaMemcpyAsync(h.data(), sum.p, n_sum * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaStreamSynchronize(st));
  };
  HBX_CUDA(cudaMemcpyAsync(E.sym_of_byte.data(), sym.p, 256, cudaMemcpyDeviceToHost, st));
  read_summary();
  auto give_up = [&](const std::string& reason) {
    *why = reason;
    *LB = SideBufs{};
    *RB = SideBufs{};
    return false;
  };
  // two distinct cells shared a hash: every dictionary again with the next seed
  for (int attempt = 1; (h[ing::kSumFlags] & ing::kFlagCollision) && attempt < kMaxAttempts;
       attempt++) {
    const unsigned long long clear = h[ing::kSumFlags] & ~(unsigned long long)ing::kFlagCollision;
    HBX_CUDA(cudaMemcpyAsync(sum.p + ing::kSumFlags, &clear, sizeof clear, cudaMemcpyHostToDevice, st));
    eq_dictionaries(seed_of(attempt));
    read_summary();
  }
  if (h[ing::kSumFlags] & ing::kFlagCollision)
    return give_up("dictionary cells collide under four hash seeds");
  if (h[ing::kSumFlags] & ing::kFlagTableFull) return give_up("dictionary table full");
  E.pairs_covered = h[ing::kSumPairs];
  E.n_partitions_used = (uint32_t)h[ing::kSumUsed];
  E.n_symbols = (uint32_t)h[ing::kSumSymbols];
  E.eq_card.assign(n_eq, 1);
  for (size_t k = 0; k < n_eq; k++) E.eq_card[k] = (uint32_t)std::max<unsigned long long>(h[i_card + k], 1);
  E.L.str_maxlen.assign(n_sl, 0);
  E.R.str_maxlen.assign(n_sr, 0);
  for (size_t s = 0; s < n_sl; s++) E.L.str_maxlen[s] = (uint32_t)h[i_mxl + s];
  for (size_t s = 0; s < n_sr; s++) E.R.str_maxlen[s] = (uint32_t)h[i_mxr + s];

  // ---- join-key domains; composite ids for rules whose mixed-radix domain
  // is too large: each row's (bucket, codes) tuple through a dictionary of
  // its own, then the tuple ids regrouped by bucket
  std::vector<size_t> comp_rules;
  for (size_t r = 0; r < E.rules.size(); r++)
    if (!rule_mixed_domain(E, &E.rules[r])) comp_rules.push_back(r);
  const size_t n_comp = comp_rules.size();
  LB->comp.alloc(std::max<size_t>(n_comp * nL, 1));
  RB->comp.alloc(std::max<size_t>(n_comp * nR, 1));
  if (n_comp) {
    DBuf<int32_t> tcode_l, tcode_r;
    DBuf<uint32_t> tup_l, tup_r, code_bucket, per_bucket, start, cursor, remap;
    tcode_l.alloc(std::max<uint32_t>(nL, 1));
    tcode_r.alloc(std::max<uint32_t>(nR, 1));
    code_bucket.alloc(cap);
    remap.alloc(cap);
    per_bucket.alloc(n_part + 1);
    start.alloc(n_part + 1);
    cursor.alloc(n_part + 1);
    DBuf<unsigned long long> dsum;
    dsum.alloc(1);
    for (size_t ci = 0; ci < n_comp; ci++) {
      RuleEnc& re = E.rules[comp_rules[ci]];
      ing::TupleSlots ts{};
      ts.k = (uint32_t)re.eq_slot.size();
      for (uint32_t j = 0; j < ts.k; j++) ts.slot[j] = (uint32_t)re.eq_slot[j];
      const uint32_t w = ts.k + 1;
      tup_l.alloc(std::max<size_t>((size_t)nL * w, 1));
      tup_r.alloc(std::max<size_t>((size_t)nR * w, 1));
      if (nL) ing::k_tuples<<<grid_for(nL, n_sm), 256, 0, st>>>(LB->bucket.p, LB->eq.p, nL, ts, tup_l.p);
      if (nR) ing::k_tuples<<<grid_for(nR, n_sm), 256, 0, st>>>(RB->bucket.p, RB->eq.p, nR, ts, tup_r.p);
      const ing::ColDev tl{reinterpret_cast<const uint8_t*>(tup_l.p), nullptr, 0, 4 * w};
      const ing::ColDev tr{reinterpret_cast<const uint8_t*>(tup_r.p), nullptr, 0, 4 * w};
      unsigned long long n_codes = 0;
      for (int attempt = 0;; attempt++) {
        HBX_CUDA(cudaMemsetAsync(sum.p + ing::kSumFlags, 0, sizeof(unsigned long long), st));
        dictionary(tl, tr, tcode_l.p, tcode_r.p, dsum.p, seed_of(attempt));
        unsigned long long got[2] = {0, 0};
        HBX_CUDA(cudaMemcpyAsync(&got[0], sum.p + ing::kSumFlags, 8, cudaMemcpyDeviceToHost, st));
        HBX_CUDA(cudaMemcpyAsync(&got[1], dsum.p, 8, cudaMemcpyDeviceToHost, st));
        HBX_CUDA(cudaStreamSynchronize(st));
        if (got[0] & ing::kFlagTableFull) return give_up("dictionary table full");
        n_codes = got[1];
        if (!(got[0] & ing::kFlagCollision)) break;
        if (attempt + 1 == kMaxAttempts) return give_up("join-key tuples collide under four hash seeds");
      }
      HBX_CUDA(cudaMemsetAsync(per_bucket.p, 0, (n_part + 1) * 4, st));
      HBX_CUDA(cudaMemsetAsync(cursor.p, 0, (n_part + 1) * 4, st));
      ing::k_code_bucket<<<grid_for(cap, n_sm), 256, 0, st>>>(keys.p, code.p, rep.p, cap,
                                                              LB->bucket.p, RB->bucket.p, nL,
                                                              code_bucket.p, per_bucket.p);
      scan_u32(per_bucket.p, (uint32_t)(n_part + 1), start.p, st);  // start[n_part] = n_codes
      if (n_codes)
        ing::k_code_remap<<<grid_for(n_codes, n_sm), 256, 0, st>>>(code_bucket.p, (uint32_t)n_codes,
                                                                  start.p, cursor.p, remap.p);
      if (nL)
        ing::k_apply_remap<<<grid_for(nL, n_sm), 256, 0, st>>>(tcode_l.p, nL, remap.p,
                                                               LB->comp.p + ci * nL);
      if (nR)
        ing::k_apply_remap<<<grid_for(nR, n_sm), 256, 0, st>>>(tcode_r.p, nR, remap.p,
                                                               RB->comp.p + ci * nR);
      check_launch("ingest composite keys");
      std::vector<uint32_t> hs(n_part + 1);
      HBX_CUDA(cudaMemcpyAsync(hs.data(), start.p, (n_part + 1) * 4, cudaMemcpyDeviceToHost, st));
      HBX_CUDA(cudaStreamSynchronize(st));
      re.composite = true;
      re.comp_index = (int)ci;
      re.domain = std::max<uint64_t>(n_codes, 1);
      re.part_key_begin.assign(hs.begin(), hs.end());
      if (re.domain > (1ull << 31)) fail(HBX_ERR_UNSUPPORTED, "join key domain too large");
    }
  }
  return true;
}

}  // namespace hbx
