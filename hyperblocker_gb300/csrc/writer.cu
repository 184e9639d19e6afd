// writer.cu -- "<id_l>,<id_r>\n" lines of pairs formatted on the device (the
// reference's WriteMatch, core/components/host_reducer.h:80-90: column 0 of
// each table printed as a C string, one line per pair, appended to a file).
//
// Pairs are taken in chunks whose text fits a fixed device buffer: per pair
// the line length (the two ids cut at their first NUL, a comma, a newline),
// an exclusive scan of the lengths into line offsets, then one thread per
// pair copies its line into the chunk's text, which goes back to page-locked
// host memory and is appended to the file while the next chunk is formatted.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>

#include "context.h"
#include "device_buffers.h"
#include "hbx_core.h"
#include "ingest.h"

namespace hbx {
namespace wr {

// Line length of every pair of the chunk; a row index outside its table sets
// *bad (the line then has length 0).
__global__ void k_line_len(ing::ColDev il, uint32_t n_left, ing::ColDev ir, uint32_t n_right,
                           const uint32_t* l_row, const uint32_t* r_row, uint32_t n, uint32_t* len,
                           unsigned int* bad) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t l = l_row[i], r = r_row[i];
    if (l >= n_left || r >= n_right) {
      atomicOr(bad, 1u);
      len[i] = 0;
      continue;
    }
    int64_t a, b;
    len[i] = ing::cell_len(il, l, &a) + ing::cell_len(ir, r, &b) + 2u;
  }
}

// Copies every pair's line to its offset in the chunk's text.
__global__ void k_line_write(ing::ColDev il, uint32_t n_left, ing::ColDev ir, uint32_t n_right,
                            const uint32_t* l_row, const uint32_t* r_row, uint32_t n,
                            const uint32_t* off, uint8_t* text) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t l = l_row[i], r = r_row[i];
    if (l >= n_left || r >= n_right) continue;
    int64_t a, b;
    const uint32_t na = ing::cell_len(il, l, &a), nb = ing::cell_len(ir, r, &b);
    uint8_t* o = text + off[i];
    for (uint32_t k = 0; k < na; k++) o[k] = il.bytes[a + k];
    o[na] = ',';
    for (uint32_t k = 0; k < nb; k++) o[na + 1 + k] = ir.bytes[b + k];
    o[na + 1 + nb] = '\n';
  }
}

}  // namespace wr

namespace {

// Column 0 of a table on the device.
struct IdColumn {
  DBuf<uint8_t> bytes;
  DBuf<int64_t> off;
  ing::ColDev view{};
  uint32_t max_len = 0;
  void upload(const Column& c, int64_t n_rows, cudaStream_t st) {
    bytes.alloc(std::max<size_t>(c.bytes.size(), 16));
    off.alloc((size_t)n_rows + 1);
    if (!c.bytes.empty())
      HBX_CUDA(cudaMemcpyAsync(bytes.p, c.bytes.data(), c.bytes.size(), cudaMemcpyHostToDevice, st));
    HBX_CUDA(cudaMemcpyAsync(off.p, c.off.data(), ((size_t)n_rows + 1) * 8, cudaMemcpyHostToDevice, st));
    for (int64_t i = 0; i < n_rows; i++) max_len = std::max<uint32_t>(max_len, (uint32_t)c.len(i));
    view = ing::ColDev{bytes.p, off.p, c.has_nul ? 1u : 0u};
  }
};

constexpr uint64_t kTextChunkBytes = 64ull << 20;  // device text per chunk

}  // namespace

void write_pairs_device(hbx_ctx* C, const Table& TL, const Table& TR, const uint32_t* l_row,
                        const uint32_t* r_row, uint64_t n, const char* path) {
  if (TL.n_cols() == 0 || TR.n_cols() == 0) fail(HBX_ERR_INVALID_ARG, "table without an id column");
  if (TL.n_rows > UINT32_MAX || TR.n_rows > UINT32_MAX) fail(HBX_ERR_INVALID_ARG, "table too large");
  cudaStream_t st = C->stream;
  PoolScope scope(C->pool, st);
  IdColumn il, ir;
  il.upload(TL.cols[0], TL.n_rows, st);
  ir.upload(TR.cols[0], TR.n_rows, st);
  const uint64_t max_line = (uint64_t)il.max_len + ir.max_len + 2;
  if (max_line >= (1ull << 31)) fail(HBX_ERR_INVALID_ARG, "id cells too long");
  // pairs per chunk: their text fits kTextChunkBytes (and u32 offsets)
  const uint32_t per_chunk =
      (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(kTextChunkBytes / max_line, 1u << 24));
  FILE* f = std::fopen(path, "ab");
  if (!f) fail(HBX_ERR_IO, std::string("cannot open ") + path);
  struct Closer {
    FILE* f;
    ~Closer() {
      if (f) std::fclose(f);
    }
  } closer{f};
  // two chunk slots: one is written to the file while the other is formatted
  struct Slot {
    DBuf<uint32_t> len, off;
    DBuf<uint8_t> text;
    void* host = nullptr;
    uint64_t host_n = 0, bytes = 0;
    cudaEvent_t done = nullptr;
    ~Slot() {
      if (host) cudaFreeHost(host);
      if (done) cudaEventDestroy(done);
    }
  } slots[2];
  // copies into the slots' page-locked buffers end before those are freed,
  // also when a chunk fails
  struct SyncOnExit {
    cudaStream_t st;
    ~SyncOnExit() { cudaStreamSynchronize(st); }
  } sync_on_exit{st};
  DBuf<unsigned int> bad;
  bad.alloc(1);
  DBuf<unsigned long long> total;
  total.alloc(1);
  HBX_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(unsigned int), st));
  for (Slot& s : slots) {
    s.len.alloc(per_chunk);
    s.off.alloc(per_chunk);
    s.text.alloc((uint64_t)per_chunk * max_line + 16);
    HBX_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
  }
  auto format = [&](Slot& s, uint64_t i0) {
    const uint32_t m = (uint32_t)std::min<uint64_t>(per_chunk, n - i0);
    const int grid = grid_for(m, C->n_sm);
    wr::k_line_len<<<grid, 256, 0, st>>>(il.view, (uint32_t)TL.n_rows, ir.view, (uint32_t)TR.n_rows,
                                         l_row + i0, r_row + i0, m, s.len.p, bad.p);
    scan_u32(s.len.p, m, s.off.p, st);
    ing::k_scan_total<<<1, 1, 0, st>>>(s.off.p, s.len.p, m, 0ull, total.p);
    wr::k_line_write<<<grid, 256, 0, st>>>(il.view, (uint32_t)TL.n_rows, ir.view,
                                           (uint32_t)TR.n_rows, l_row + i0, r_row + i0, m, s.off.p,
                                           s.text.p);
    check_launch("pair formatting");
    unsigned long long bytes = 0;
    unsigned int b = 0;
    HBX_CUDA(cudaMemcpyAsync(&bytes, total.p, 8, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaMemcpyAsync(&b, bad.p, 4, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaStreamSynchronize(st));
    if (b) fail(HBX_ERR_INVALID_ARG, "row index out of range");
    if (bytes > s.host_n) {
      if (s.host) cudaFreeHost(s.host);
      s.host = nullptr;
      s.host_n = 0;
      HBX_CUDA(cudaHostAlloc(&s.host, std::max<uint64_t>(bytes, 1), cudaHostAllocDefault));
      s.host_n = std::max<uint64_t>(bytes, 1);
    }
    s.bytes = bytes;
    if (bytes) HBX_CUDA(cudaMemcpyAsync(s.host, s.text.p, bytes, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaEventRecord(s.done, st));
  };
  auto drain = [&](Slot& s) {
    HBX_CUDA(cudaEventSynchronize(s.done));
    if (s.bytes && std::fwrite(s.host, 1, s.bytes, f) != s.bytes)
      fail(HBX_ERR_IO, std::string("write failed: ") + path);
    s.bytes = 0;
  };
  int k = 0;
  bool pending = false;
  for (uint64_t i0 = 0; i0 < n; i0 += per_chunk, k ^= 1) {
    format(slots[k], i0);  // the other slot's copy is in flight or written
    if (pending) drain(slots[k ^ 1]);
    pending = true;
  }
  if (pending) drain(slots[k ^ 1]);
  closer.f = nullptr;
  if (std::fclose(f) != 0) fail(HBX_ERR_IO, std::string("close failed: ") + path);
}

}  // namespace hbx

extern "C" hbx_status hbx_write_pairs_device(hbx_ctx* ctx, const hbx_table* left,
                                             const hbx_table* right, const uint32_t* l_row,
                                             const uint32_t* r_row, uint64_t n, const char* path) {
  if (!ctx || !left || !right || !path || (n && (!l_row || !r_row))) return HBX_ERR_INVALID_ARG;
  try {
    HBX_CUDA(cudaSetDevice(ctx->device));
    hbx::write_pairs_device(ctx, left->t, right->t, l_row, r_row, n, path);
    ctx->err.clear();
    return HBX_OK;
  } catch (const hbx::Error& e) {
    ctx->err = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    ctx->err = "host out of memory";
    return HBX_ERR_OOM;
  }
}

// hbx_write_pairs with a context and many pairs: the host arrays go to the
// device and the lines are formatted there (same bytes as the host loop).
extern "C" hbx_status hbx_internal_write_pairs_via_device(hbx_ctx* ctx, const hbx_table* left,
                                                          const hbx_table* right,
                                                          const uint32_t* l_row,
                                                          const uint32_t* r_row, uint64_t n,
                                                          const char* path) {
  try {
    HBX_CUDA(cudaSetDevice(ctx->device));
    hbx::PoolScope scope(ctx->pool, ctx->stream);
    hbx::DBuf<uint32_t> dl, dr;
    dl.alloc(n);
    dr.alloc(n);
    HBX_CUDA(cudaMemcpyAsync(dl.p, l_row, n * 4, cudaMemcpyHostToDevice, ctx->stream));
    HBX_CUDA(cudaMemcpyAsync(dr.p, r_row, n * 4, cudaMemcpyHostToDevice, ctx->stream));
    hbx::write_pairs_device(ctx, left->t, right->t, dl.p, dr.p, n, path);
    HBX_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->err.clear();
    return HBX_OK;
  } catch (const hbx::Error& e) {
    cudaStreamSynchronize(ctx->stream);
    ctx->err = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    ctx->err = "host out of memory";
    return HBX_ERR_OOM;
  }
}
