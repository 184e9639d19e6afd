// device_buffers.h -- owned device buffers of a session.
//
// Sessions allocate a few dozen buffers and free them when they end; a
// one-shot hbx_block call creates and destroys a session every time.  So the
// buffers come from the context's stream-ordered memory pool (its release
// threshold is unlimited, so freed memory stays with the pool and the next
// session's allocations do not reach the driver).  The pool is chosen by a
// PoolScope on the calling thread for the duration of one C-ABI call; outside
// any scope a buffer falls back to cudaMalloc.  A buffer remembers where it
// came from and returns there.
//
// Ordering: allocations are ordered on the scope's stream.  Every entry point
// synchronizes that stream before it returns, and a session frees its buffers
// only from hbx_session_destroy, when none of its work is in flight.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "hbx_core.h"
#include "kernels.cuh"

#define HBX_CUDA(expr)                                                                        \
  do {                                                                                        \
    cudaError_t e_ = (expr);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      ::hbx::fail(e_ == cudaErrorMemoryAllocation ? HBX_ERR_OOM : HBX_ERR_CUDA,               \
                  std::string(#expr) + ": " + cudaGetErrorString(e_));                        \
  } while (0)

namespace hbx {

struct DevPool {
  cudaMemPool_t pool = nullptr;
  cudaStream_t stream = nullptr;
};

// The pool of the C-ABI call running on this thread (null: cudaMalloc).
inline const DevPool*& current_pool() {
  thread_local const DevPool* p = nullptr;
  return p;
}

struct PoolScope {
  const DevPool* prev;
  DevPool mine;
  PoolScope(cudaMemPool_t pool, cudaStream_t stream) : prev(current_pool()) {
    mine.pool = pool;
    mine.stream = stream;
    current_pool() = pool ? &mine : nullptr;
  }
  ~PoolScope() { current_pool() = prev; }
  PoolScope(const PoolScope&) = delete;
  PoolScope& operator=(const PoolScope&) = delete;
};

// A bump allocator over device memory the caller owns (hbx_block_static's
// scratch array).  While an ArenaScope is active on the thread, every DBuf
// takes its memory from it: 256-byte aligned pieces; freeing the most
// recent piece gives its bytes back, the others stay taken until the arena
// is dropped.  A piece that does not fit refuses the input
// (HBX_ERR_INVALID_ARG) before anything is written to it.
struct DevArena {
  unsigned char* base = nullptr;
  size_t cap = 0, used = 0, peak = 0;
};

inline DevArena*& current_arena() {
  thread_local DevArena* a = nullptr;
  return a;
}

struct ArenaScope {
  DevArena* prev;
  explicit ArenaScope(DevArena* a) : prev(current_arena()) { current_arena() = a; }
  ~ArenaScope() { current_arena() = prev; }
  ArenaScope(const ArenaScope&) = delete;
  ArenaScope& operator=(const ArenaScope&) = delete;
};

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DevPool from{};  // pool and stream of the allocation (pool null: cudaMalloc)
  DevArena* arena = nullptr;  // the arena the piece came from (then nothing is freed)
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), from(o.from), arena(o.arena) {
    o.p = nullptr;
    o.n = 0;
    o.arena = nullptr;
  }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      reset();
      p = o.p;
      n = o.n;
      from = o.from;
      arena = o.arena;
      o.p = nullptr;
      o.n = 0;
      o.arena = nullptr;
    }
    return *this;
  }
  ~DBuf() { reset(); }
  void reset() {
    if (p && arena) {
      unsigned char* end = reinterpret_cast<unsigned char*>(p) + n * sizeof(T);
      if (end == arena->base + arena->used)
        arena->used = (size_t)(reinterpret_cast<unsigned char*>(p) - arena->base);
    } else if (p) {
      if (from.pool)
        cudaFreeAsync(p, from.stream);
      else
        cudaFree(p);
    }
    p = nullptr;
    n = 0;
    arena = nullptr;
  }
  void alloc(size_t count) {
    reset();
    if (count == 0) count = 1;
    if (DevArena* a = current_arena()) {
      const size_t start = (a->used + 255) / 256 * 256;
      if (start + count * sizeof(T) > a->cap)
        fail(HBX_ERR_INVALID_ARG,
             "input needs more device scratch for its encoding than the static scratch holds (" +
                 std::to_string(a->cap) + " bytes)");
      p = reinterpret_cast<T*>(a->base + start);
      n = count;
      arena = a;
      a->used = start + count * sizeof(T);
      a->peak = a->used > a->peak ? a->used : a->peak;
      return;
    }
    const DevPool* dp = current_pool();
    if (dp) {
      HBX_CUDA(cudaMallocFromPoolAsync((void**)&p, count * sizeof(T), dp->pool, dp->stream));
      from = *dp;
    } else {
      HBX_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
      from = DevPool{};
    }
    n = count;
    // the kernels' bulk copies and vector loads need 16-byte aligned bases
    if ((uintptr_t)p & 15) fail(HBX_ERR_CUDA, "device allocation not 16-byte aligned");
  }
  void upload(const std::vector<T>& v, cudaStream_t s) {
    alloc(v.size());
    if (!v.empty())
      HBX_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  }
};

// Raises (never lowers) an evaluation kernel's dynamic shared-memory limit
// to bytes; the limit is process-wide, shared by every session and server.
void raise_smem_limit(dev::EvalKernel kern, size_t bytes);

// Device copy of one encoded table.
struct SideBufs {
  DBuf<uint32_t> bucket;
  DBuf<int32_t> eq, comp;
  DBuf<uint8_t> arena;
  DBuf<dev::StrMeta> meta;
};

}  // namespace hbx
