// sort.cu -- (left row, right row) pairs sorted on the device, for output in
// row order: a least-significant-digit radix sort of the 64-bit keys
// left << 32 | right, 8 bits per pass, over the bytes the row counts use.
//
// A pass histograms the digit per tile of kTile keys, scans the histograms
// digit-major (all tiles' counts of digit 0, then digit 1, ...) into the
// first position of every (digit, tile), and scatters each tile's keys in
// order: rounds of 256 keys, a warp ranks its 32 keys among equal digits with
// __match_any_sync, per-warp counts give each warp's start per digit, and a
// running count per digit carries across rounds, so the sort is stable.
#include <cuda_runtime.h>

#include <algorithm>

#include "context.h"
#include "device_buffers.h"
#include "hbx_core.h"
#include "ingest.h"

namespace hbx {
namespace srt {

constexpr uint32_t kThreads = 256;
constexpr uint32_t kRounds = 8;
constexpr uint32_t kTile = kThreads * kRounds;  // keys per tile
constexpr unsigned kFull = 0xffffffffu;

__global__ void k_pack(const uint32_t* l, const uint32_t* r, uint64_t n, unsigned long long* key) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    key[i] = ((unsigned long long)l[i] << 32) | r[i];
}

__global__ void k_unpack(const unsigned long long* key, uint64_t n, uint32_t* l, uint32_t* r) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    l[i] = (uint32_t)(key[i] >> 32);
    r[i] = (uint32_t)key[i];
  }
}

// hist[digit * n_tiles + tile]: keys of the tile with that digit.
__global__ void __launch_bounds__(kThreads) k_hist(const unsigned long long* key, uint64_t n,
                                                   uint32_t shift, uint32_t n_tiles,
                                                   uint32_t* hist) {
  __shared__ uint32_t h[256];
  const uint32_t tile = blockIdx.x;
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)tile * kTile;
  for (uint32_t k = 0; k < kRounds; k++) {
    const uint64_t i = base + k * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(uint32_t)(key[i] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * n_tiles + tile] = h[threadIdx.x];
}

// Scatters one tile's keys, in order, to off[digit * n_tiles + tile] on.
__global__ void __launch_bounds__(kThreads) k_scatter(const unsigned long long* key, uint64_t n,
                                                      uint32_t shift, uint32_t n_tiles,
                                                      const uint32_t* off,
                                                      unsigned long long* out) {
  __shared__ uint32_t wcnt[kThreads / 32][256];  // this round's keys per warp and digit
  __shared__ uint32_t wpre[kThreads / 32][256];  // where each warp starts, per digit
  __shared__ uint32_t run[256];                  // keys of earlier rounds per digit
  const uint32_t tile = blockIdx.x;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  run[threadIdx.x] = off[(uint64_t)threadIdx.x * n_tiles + tile];
  const uint64_t base = (uint64_t)tile * kTile;
  for (uint32_t k = 0; k < kRounds; k++) {
    for (uint32_t w = 0; w < kThreads / 32; w++) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const uint64_t i = base + k * kThreads + threadIdx.x;
    const bool act = i < n;
    const unsigned long long v = act ? key[i] : 0ull;
    const uint32_t d = act ? (uint32_t)(v >> shift) & 0xffu : 256u + lane;  // inactive: unique
    const unsigned peers = __match_any_sync(kFull, d);
    const uint32_t rank = (uint32_t)__popc(peers & ((1u << lane) - 1u));
    if (act && rank == 0) wcnt[warp][d] = (uint32_t)__popc(peers);
    __syncthreads();
    {  // thread t: digit t over the warps, in order
      uint32_t acc = run[threadIdx.x];
      for (uint32_t w = 0; w < kThreads / 32; w++) {
        wpre[w][threadIdx.x] = acc;
        acc += wcnt[w][threadIdx.x];
      }
      run[threadIdx.x] = acc;
    }
    __syncthreads();
    if (act) out[wpre[warp][d] + rank] = v;
    __syncthreads();
  }
}

}  // namespace srt

// Sorts n pairs by (left row, right row) in place; rows below n_left /
// n_right (the bytes of the keys beyond them are 0 and take no pass).
void sort_pairs_device(hbx_ctx* C, uint32_t* l, uint32_t* r, uint64_t n, uint32_t n_left,
                       uint32_t n_right) {
  if (n < 2) return;
  if (n >= (1ull << 32)) fail(HBX_ERR_UNSUPPORTED, "more than 2^32 pairs to sort");
  cudaStream_t st = C->stream;
  PoolScope scope(C->pool, st);
  auto bytes_of = [](uint32_t rows) {
    uint32_t b = 0;
    while (b < 4 && (uint64_t)rows > (1ull << (8 * b))) b++;
    return b;  // digit bytes that hold row indices below rows
  };
  const uint32_t br = bytes_of(n_right), bl = bytes_of(n_left);
  DBuf<unsigned long long> a, b;
  a.alloc(n);
  b.alloc(n);
  const int g = grid_for(n, C->n_sm);
  srt::k_pack<<<g, 256, 0, st>>>(l, r, n, a.p);
  const uint32_t n_tiles = (uint32_t)((n + srt::kTile - 1) / srt::kTile);
  const uint64_t nh = 256ull * n_tiles;
  if (nh >= (1ull << 32)) fail(HBX_ERR_UNSUPPORTED, "too many pairs to sort");
  DBuf<uint32_t> hist, off;
  hist.alloc(nh);
  off.alloc(nh);
  unsigned long long* src = a.p;
  unsigned long long* dst = b.p;
  for (uint32_t byte = 0; byte < 8; byte++) {
    const bool used = byte < 4 ? byte < br : byte - 4 < bl;
    if (!used) continue;
    const uint32_t shift = 8 * byte;
    srt::k_hist<<<n_tiles, srt::kThreads, 0, st>>>(src, n, shift, n_tiles, hist.p);
    scan_u32(hist.p, (uint32_t)nh, off.p, st);
    srt::k_scatter<<<n_tiles, srt::kThreads, 0, st>>>(src, n, shift, n_tiles, off.p, dst);
    check_launch("pair sort");
    std::swap(src, dst);
  }
  srt::k_unpack<<<g, 256, 0, st>>>(src, n, l, r);
  check_launch("pair sort");
  HBX_CUDA(cudaStreamSynchronize(st));
}

}  // namespace hbx
