// csv_gpu.cu -- the CSV tokenization of csv.cpp (rapidcsv 8.x with the
// reference's parameters, core/components/data_mngr.h:48-51) on the device.
//
// A line break always ends a row (no quoted line breaks), so rows are the
// spans between '\n' bytes and tokenize independently.  A warp takes 32
// consecutive rows -- one contiguous span of the file -- and copies it into
// shared memory with 16-byte loads (a span longer than the warp's staging
// area is read from device memory instead); each lane then walks its row's
// bytes once with the host loop's state machine (a '"' toggles the quote
// state when it is the first kept byte of the cell or the cell began with
// '"'; a separator other than '"' ends a cell outside quotes; '\r' is
// dropped) and, in the same pass, keeps what unquoting needs: a cell whose
// kept bytes are "..." reads as its interior with every run of k '"' in it
// reading as ceil(k/2) of them (csv.cpp push_cell pairs "" -> " from the
// left).  The first walk (k_measure) gives every cell's unquoted length
// and whether it is enclosed; after a scan of the lengths per column the
// second (k_write) writes the cells into column-major arenas.  The table is
// then copied back into host columns, byte for byte what table_from_buffer
// builds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "context.h"
#include "device_buffers.h"
#include "hbx_core.h"
#include "ingest.h"

namespace hbx {
namespace csvd {

constexpr uint32_t kChunk = 64;  // bytes per thread when finding line breaks
constexpr uint32_t kRowThreads = 256;   // threads per block of the row kernels
constexpr uint32_t kStageBytes = 8192;  // shared memory per warp for its rows' bytes

// Byte source of the row walks: position `a` at s[0] -- the file in device
// memory (a = 0) or a warp's staged copy of its rows (a = the first staged
// position).  Bytes are read one at a time: a per-lane register window of
// 16 bytes was slower, since the lanes of a warp cross their window
// boundaries at different bytes and reload on nearly every step.
struct Src {
  const uint8_t* s;
  uint64_t a;
  __device__ __forceinline__ uint8_t operator()(uint64_t i) const { return s[i - a]; }
};

// Line breaks per 64-byte chunk of the buffer.
__global__ void k_nl_count(const uint8_t* buf, uint64_t n, uint32_t n_chunks, uint32_t* cnt) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n_chunks; c += gridDim.x * blockDim.x) {
    const uint64_t a = (uint64_t)c * kChunk, b = min(a + kChunk, n);
    uint32_t k = 0;
    for (uint64_t i = a; i < b; i++) k += buf[i] == '\n';
    cnt[c] = k;
  }
}

// Positions of the line breaks, in order.
__global__ void k_nl_write(const uint8_t* buf, uint64_t n, uint32_t n_chunks, const uint32_t* off,
                           uint64_t* pos) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n_chunks; c += gridDim.x * blockDim.x) {
    const uint64_t a = (uint64_t)c * kChunk, b = min(a + kChunk, n);
    uint32_t k = off[c];
    for (uint64_t i = a; i < b; i++)
      if (buf[i] == '\n') pos[k++] = i;
  }
}

struct Rows {
  const uint64_t* nl;  // line-break positions
  uint64_t n_nl;
  uint64_t start;      // first byte of row 0 (after a BOM)
  uint64_t end;        // end of the buffer
  uint64_t n_rows;     // n_nl, plus one when bytes other than '\r' follow the last break
};

__device__ __forceinline__ void row_span(const Rows& R, uint64_t r, uint64_t* s, uint64_t* e) {
  *s = r == 0 ? R.start : R.nl[r - 1] + 1;
  *e = r < R.n_nl ? R.nl[r] : R.end;
}

// Copies the bytes of rows [r0, r0 + 32) -- positions [*a, ...) rounded out
// to 16 bytes -- into the warp's staging area; false (nothing copied) when
// they do not fit.  The file buffer is padded to a multiple of 16 bytes.
__device__ __forceinline__ bool stage_rows(const uint8_t* buf, const Rows& R, uint64_t r0,
                                           uint32_t lane, uint8_t* stage, uint64_t* a) {
  const uint64_t r1 = min(r0 + 32, R.n_rows) - 1;
  uint64_t s0, e0, s1, e1;
  row_span(R, r0, &s0, &e0);
  row_span(R, r1, &s1, &e1);
  const uint64_t lo = s0 & ~15ull, hi = (e1 + 15) & ~15ull;
  if (hi - lo > kStageBytes) return false;
  const uint4* src = reinterpret_cast<const uint4*>(buf + lo);
  uint4* dst = reinterpret_cast<uint4*>(stage);
  for (uint32_t k = lane; k < (uint32_t)((hi - lo) >> 4); k += 32) dst[k] = src[k];
  __syncwarp();
  *a = lo;
  return true;
}

// Warps over groups of 32 rows: f(source, row) for every row, from the
// staged copy when it fits.
template <class F>
__device__ __forceinline__ void for_row_groups(const uint8_t* buf, const Rows& R, F&& f) {
  extern __shared__ uint4 s_stage[];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint8_t* stage = reinterpret_cast<uint8_t*>(s_stage) + (size_t)warp * kStageBytes;
  const uint64_t n_warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t w = (uint64_t)blockIdx.x * (blockDim.x >> 5) + warp; w * 32 < R.n_rows;
       w += n_warps) {
    const uint64_t r = w * 32 + lane;
    uint64_t a = 0;
    if (stage_rows(buf, R, w * 32, lane, stage, &a)) {
      if (r < R.n_rows) f(Src{stage, a}, r);
    } else if (r < R.n_rows) {
      f(Src{buf, 0}, r);
    }
    __syncwarp();  // the staging area is rewritten next
  }
}

// The host loop's cell rule, byte by byte: true when ch (not '\r') ends the
// current cell; otherwise ch is one of the cell's kept bytes.
struct CellRule {
  bool quoted = false, empty = true, first_quote = false;
  __device__ __forceinline__ bool ends_cell(uint8_t ch, uint8_t sep) {
    if (ch != '"' && ch == sep && !quoted) {
      empty = true;
      first_quote = false;
      return true;
    }
    if (ch == '"') {
      if (empty || first_quote) quoted = !quoted;
      if (empty) first_quote = true;
    }
    empty = false;
    return false;
  }
};

// Pass 1: unquoted length of every cell [col][row] and whether its kept
// bytes are "..." (enclosed); rows with fewer cells than n_cols report
// (row << 32 | cells) into *short_row (smallest wins).
__global__ void __launch_bounds__(kRowThreads) k_measure(const uint8_t* buf, Rows R, uint8_t sep,
                                                         uint32_t n_cols, uint32_t* len,
                                                         uint8_t* enclosed,
                                                         unsigned long long* short_row) {
  for_row_groups(buf, R, [&](const Src& B, uint64_t r) {
    uint64_t s, e;
    row_span(R, r, &s, &e);
    CellRule rule;
    uint32_t c = 0;
    // the current cell: kept bytes, first and last, the open run of '"'
    // (and whether it began at the first kept byte), '"' swallowed by
    // earlier runs
    uint32_t n = 0, run = 0, swallowed = 0;
    uint8_t first = 0, last = 0;
    bool run_at_start = false;
    auto end_cell = [&]() {
      const uint64_t at = (uint64_t)c * R.n_rows + r;
      const bool enc = n >= 2 && first == '"' && last == '"';
      uint32_t w = n;
      if (enc) {  // the open run holds the closing '"' (and the opening one)
        const int k = (int)run - 1 - (run_at_start ? 1 : 0);
        w = n - 2 - swallowed - (k > 0 ? (uint32_t)k / 2 : 0u);
      }
      len[at] = w;
      enclosed[at] = enc ? 1 : 0;
      c++;
      n = run = swallowed = 0;
      first = last = 0;
      run_at_start = false;
    };
    for (uint64_t i = s; i < e && c < n_cols; i++) {
      const uint8_t ch = B(i);
      if (ch == '\r') continue;
      if (rule.ends_cell(ch, sep)) {
        end_cell();
        continue;
      }
      if (n == 0) first = ch;
      last = ch;
      if (ch == '"') {
        if (run == 0) run_at_start = n == 0;
        run++;
      } else if (run) {
        swallowed += (run - (run_at_start ? 1u : 0u)) / 2;
        run = 0;
        run_at_start = false;
      }
      n++;
    }
    if (c < n_cols) end_cell();  // the row's last cell
    if (c < n_cols) {
      atomicMin(short_row, ((unsigned long long)r << 32) | c);
      for (; c < n_cols; c++) {
        len[(uint64_t)c * R.n_rows + r] = 0;
        enclosed[(uint64_t)c * R.n_rows + r] = 0;
      }
    }
  });
}

// Pass 2: the cells into their columns' arenas: an enclosed cell's bytes
// after the opening '"' until its length is reached, a '"' right after a
// written '"' swallowed; any other cell's kept bytes.
__global__ void __launch_bounds__(kRowThreads) k_write(const uint8_t* buf, Rows R, uint8_t sep,
                                                       uint32_t n_cols, const uint32_t* off,
                                                       const uint32_t* len,
                                                       const uint8_t* enclosed,
                                                       uint8_t* const* arena) {
  for_row_groups(buf, R, [&](const Src& B, uint64_t r) {
    uint64_t s, e;
    row_span(R, r, &s, &e);
    CellRule rule;
    uint32_t c = 0, j = 0, w = 0, want = 0;
    bool enc = false, pending = false;
    uint8_t* out = nullptr;
    auto open_cell = [&]() {
      const uint64_t at = (uint64_t)c * R.n_rows + r;
      out = arena[c] + off[at];
      want = len[at];
      enc = enclosed[at] != 0;
      j = w = 0;
      pending = false;
    };
    open_cell();
    for (uint64_t i = s; i < e; i++) {
      const uint8_t ch = B(i);
      if (ch == '\r') continue;
      if (rule.ends_cell(ch, sep)) {
        if (++c >= n_cols) break;
        open_cell();
        continue;
      }
      const uint32_t jj = j++;
      if (!enc) {
        out[w++] = ch;
      } else if (jj > 0 && w < want) {
        if (ch == '"' && pending) {
          pending = false;
        } else {
          out[w++] = ch;
          pending = ch == '"';
        }
      }
    }
  });
}

// Exclusive u32 offsets of one column (plus its total) as int64.
__global__ void k_widen(const uint32_t* off, const uint32_t* len, uint64_t n, int64_t* out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = i < n ? (int64_t)off[i] : (n ? (int64_t)off[n - 1] + len[n - 1] : 0);
}

}  // namespace csvd

bool table_from_buffer_device(hbx_ctx* C, const char* data, size_t n, char sep, Table* out) {
  // the same BOM rule and row count as the host loop; the header row's cell
  // count, on the host
  size_t skip = 0;
  if (n >= 3 && (unsigned char)data[0] == 0xEF && (unsigned char)data[1] == 0xBB &&
      (unsigned char)data[2] == 0xBF)
    skip = 3;
  const char* p = data + skip;
  const size_t m = n - skip;
  const char* first_nl = (const char*)std::memchr(p, '\n', m);
  const size_t first_end = first_nl ? (size_t)(first_nl - p) : m;
  // cells of row 0 by the host tokenizer itself
  const Table head = table_from_buffer(p, first_end, sep);
  const uint32_t n_cols = (uint32_t)head.n_cols();
  if (n_cols == 0 || m > (1ull << 40)) return false;
  HBX_CUDA(cudaSetDevice(C->device));
  cudaStream_t st = C->stream;
  PoolScope scope(C->pool, st);
  DBuf<uint8_t> buf;
  buf.alloc(((m + 15) & ~(size_t)15) + 16);  // the row kernels read whole 16-byte words
  HBX_CUDA(cudaMemcpyAsync(buf.p, p, m, cudaMemcpyHostToDevice, st));
  const uint64_t n_chunks64 = (m + csvd::kChunk - 1) / csvd::kChunk;
  if (n_chunks64 >= (1ull << 32)) return false;
  const uint32_t n_chunks = (uint32_t)std::max<uint64_t>(n_chunks64, 1);
  DBuf<uint32_t> cnt, coff;
  cnt.alloc(n_chunks);
  coff.alloc(n_chunks);
  HBX_CUDA(cudaMemsetAsync(cnt.p, 0, (size_t)n_chunks * 4, st));
  const int g = grid_for(n_chunks, C->n_sm);
  csvd::k_nl_count<<<g, 256, 0, st>>>(buf.p, m, n_chunks, cnt.p);
  scan_u32(cnt.p, n_chunks, coff.p, st);
  DBuf<unsigned long long> tot;
  tot.alloc(1);
  ing::k_scan_total<<<1, 1, 0, st>>>(coff.p, cnt.p, n_chunks, 0ull, tot.p);
  unsigned long long n_nl = 0;
  HBX_CUDA(cudaMemcpyAsync(&n_nl, tot.p, 8, cudaMemcpyDeviceToHost, st));
  HBX_CUDA(cudaStreamSynchronize(st));
  DBuf<uint64_t> nl;
  nl.alloc(std::max<uint64_t>(n_nl, 1));
  csvd::k_nl_write<<<g, 256, 0, st>>>(buf.p, m, n_chunks, coff.p, nl.p);
  // a last row without a line break when any byte other than '\r' follows
  // the last one
  const char* last_nl = (const char*)memrchr(p, '\n', m);
  const size_t tail = last_nl ? (size_t)(last_nl - p) + 1 : 0;
  bool tail_row = false;
  for (size_t i = tail; i < m && !tail_row; i++) tail_row = p[i] != '\r';
  csvd::Rows R{nl.p, n_nl, 0, m, n_nl + (tail_row ? 1u : 0u)};
  const uint64_t rows = R.n_rows;
  if (rows == 0 || rows >= (1ull << 31)) return false;
  DBuf<uint32_t> len, off;
  len.alloc((size_t)n_cols * rows);
  off.alloc((size_t)n_cols * rows);
  DBuf<uint8_t> encl;
  encl.alloc((size_t)n_cols * rows);
  DBuf<unsigned long long> short_row;
  short_row.alloc(1);
  HBX_CUDA(cudaMemsetAsync(short_row.p, 0xff, 8, st));
  const size_t stage_smem = (size_t)(csvd::kRowThreads / 32) * csvd::kStageBytes;
  for (const void* k : {(const void*)csvd::k_measure, (const void*)csvd::k_write})
    HBX_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage_smem));
  const int gr = (int)std::max<uint64_t>(
      1, std::min<uint64_t>((rows + csvd::kRowThreads - 1) / csvd::kRowThreads,
                            (uint64_t)C->n_sm * 3));
  csvd::k_measure<<<gr, csvd::kRowThreads, stage_smem, st>>>(buf.p, R, (uint8_t)sep, n_cols, len.p,
                                                            encl.p, short_row.p);
  check_launch("csv measure");
  // per column: exclusive offsets and total bytes
  std::vector<unsigned long long> totals(n_cols);
  DBuf<unsigned long long> dtot;
  dtot.alloc(n_cols);
  for (uint32_t c = 0; c < n_cols; c++) {
    scan_u32(len.p + (size_t)c * rows, (uint32_t)rows, off.p + (size_t)c * rows, st);
    ing::k_scan_total<<<1, 1, 0, st>>>(off.p + (size_t)c * rows, len.p + (size_t)c * rows,
                                        (uint32_t)rows, 0ull, dtot.p + c);
  }
  unsigned long long bad = 0;
  HBX_CUDA(cudaMemcpyAsync(totals.data(), dtot.p, 8ull * n_cols, cudaMemcpyDeviceToHost, st));
  HBX_CUDA(cudaMemcpyAsync(&bad, short_row.p, 8, cudaMemcpyDeviceToHost, st));
  HBX_CUDA(cudaStreamSynchronize(st));
  if (bad != ~0ull) {
    char msg[160];
    std::snprintf(msg, sizeof msg, "row %lld has %d cells, expected %d", (long long)(bad >> 32),
                  (int)(bad & 0xffffffffu), (int)n_cols);
    fail(HBX_ERR_PARSE, msg);
  }
  // a column over 4 GiB would overflow the u32 offsets: the host loop then
  for (unsigned long long t : totals)
    if (t >= (1ull << 32)) return false;
  std::vector<DBuf<uint8_t>> arenas(n_cols);
  std::vector<uint8_t*> arena_ptr(n_cols);
  for (uint32_t c = 0; c < n_cols; c++) {
    arenas[c].alloc(std::max<uint64_t>(totals[c], 16));
    arena_ptr[c] = arenas[c].p;
  }
  DBuf<uint8_t*> d_arena;
  d_arena.upload(arena_ptr, st);
  csvd::k_write<<<gr, csvd::kRowThreads, stage_smem, st>>>(buf.p, R, (uint8_t)sep, n_cols, off.p,
                                                          len.p, encl.p, d_arena.p);
  check_launch("csv write");
  DBuf<int64_t> off64;
  off64.alloc(rows + 1);
  Table t;
  t.n_rows = (int64_t)rows;
  t.cols.resize(n_cols);
  for (uint32_t c = 0; c < n_cols; c++) {
    Column& col = t.cols[c];
    col.bytes.resize(totals[c]);
    col.off.resize(rows + 1);
    csvd::k_widen<<<grid_for(rows + 1, C->n_sm), 256, 0, st>>>(
        off.p + (size_t)c * rows, len.p + (size_t)c * rows, rows, off64.p);
    if (totals[c])
      HBX_CUDA(cudaMemcpyAsync(col.bytes.data(), arenas[c].p, totals[c], cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaMemcpyAsync(col.off.data(), off64.p, (rows + 1) * 8, cudaMemcpyDeviceToHost, st));
    HBX_CUDA(cudaStreamSynchronize(st));  // off64 is reused by the next column
  }
  check_launch("csv columns");
  finish_table(&t);
  *out = std::move(t);
  return true;
}

}  // namespace hbx
