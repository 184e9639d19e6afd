// ingest.h -- encoding of two host tables on the device.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "device_buffers.h"
#include "encode.h"
#include "hbx_core.h"

namespace hbx {

// ---- kernels shared by the session ingest and the serving loop ------------
namespace ing {

constexpr unsigned long long kEmpty = ~0ull;  // free slot of a dictionary table
constexpr uint32_t kFlagCollision = 1, kFlagTableFull = 2;
// words of an ingest summary (u64): pairs covered, used partitions, flags,
// alphabet size, then call-specific words
enum : uint32_t { kSumPairs = 0, kSumUsed = 1, kSumFlags = 2, kSumSymbols = 3, kSumFixed = 4 };

// One device column: cell bytes and int64 offsets (n + 1), as a host Column;
// or, with width > 0, cells of `width` bytes back to back (no offsets).
struct ColDev {
  const uint8_t* bytes;
  const int64_t* off;
  uint32_t has_nul;
  uint32_t width;
};

// Length of cell i, cut at its first NUL when the column has NUL bytes
// (the reference compares cells as C strings); *start = its first byte.
__device__ __forceinline__ uint32_t cell_len(const ColDev& c, uint32_t i, int64_t* start) {
  if (c.width) {
    *start = (int64_t)i * c.width;
    return c.width;
  }
  const int64_t a = c.off[i];
  const uint32_t n = (uint32_t)(c.off[i + 1] - a);
  *start = a;
  if (c.has_nul)
    for (uint32_t k = 0; k < n; k++)
      if (c.bytes[a + k] == 0) return k;
  return n;
}

__global__ void k_dict_insert(ColDev c, uint32_t n, uint32_t gid_base, unsigned long long* keys,
                              uint32_t* rep, uint32_t mask, uint32_t* row_slot,
                              unsigned long long* sum, unsigned long long seed);
__global__ void k_occupied(const unsigned long long* keys, uint32_t cap, uint32_t* occ);
__global__ void k_dict_assign(ColDev c, uint32_t n, uint32_t gid_base, const uint32_t* row_slot,
                              const uint32_t* code, const uint32_t* rep, ColDev cl, ColDev cr,
                              uint32_t n_left, int32_t* out, unsigned long long* sum);
__global__ void k_scan_total(const uint32_t* scan, const uint32_t* in, uint32_t n,
                             unsigned long long extra, unsigned long long* dst);
__global__ void k_byte_hist(ColDev c, uint32_t n, unsigned long long* hist);
__global__ void k_symbol_map(const unsigned long long* hist, uint8_t* sym, unsigned long long* sum);
__global__ void k_units(ColDev c, uint32_t n, uint32_t* units);
__global__ void k_pack(ColDev c, uint32_t n, const uint32_t* off16, const uint8_t* sym_g,
                       uint8_t* arena, dev::StrMeta* meta, unsigned long long* maxlen);

}  // namespace ing

// Blocks for n items of 256 threads, at most per_sm per SM.
int grid_for(uint64_t n, int n_sm, int per_sm = 8);
// Fails with HBX_ERR_CUDA if the last launch failed.
void check_launch(const char* what);
// Exclusive scan of n >= 1 u32 values into out (the join's scan kernels);
// its scratch comes from the current pool (or arena).
void scan_u32(const uint32_t* in, uint32_t n, uint32_t* out, cudaStream_t st);

// Seed of the dictionaries' first hash; a rebuild after a collision uses
// kDictSeed + attempt.  With the environment variable
// HBX_TEST_DICT_COLLIDE=1 the first build keeps only 3 bits of each hash, so
// that tests can check that collisions are resolved on the device.
constexpr unsigned long long kDictSeed = 0xc70f6907ull;

// Encodes both tables for one plan on the device, writing the side buffers
// directly: partition buckets with the reference's std::hash
// (data_mngr.h:150-202), one joint dictionary per equality slot, the
// frequency-ordered symbol alphabet, 16-byte-aligned symbol arenas and the
// per-string metadata -- the same layout the host encoder (encode.cpp)
// uploads, with identical buckets, alphabet, arenas and code equalities
// (dictionary code values may be numbered differently; only their equality
// matters).  Only the columns the plan reads are copied to the device.
//
// E must come from encode_schema.  On success E gets the dictionary sizes,
// the alphabet size, the longest string per slot, pairs_covered and the rule
// domains (a rule whose mixed-radix key domain exceeds kMaxKeyDomain gets
// dense composite ids built on the device: its (bucket, codes) tuples go
// through the same dictionary, and the ids are regrouped by bucket), and
// *h2d the bytes copied.  Two distinct cells with the same 64-bit hash are
// detected by comparing every cell with its slot's representative; the
// dictionaries are then rebuilt with another seed.  Returns false, with the
// reason in *why, only when the input is beyond the device path (2^30 rows
// or more, or collisions under four seeds); the side buffers are then left
// empty.  pin = false leaves the host tables pageable (no cudaHostRegister:
// the entry point without device allocation copies from pageable memory).
bool device_encode(const hbx_table* left, const hbx_table* right, Encoded* E, SideBufs* L,
                   SideBufs* R, int n_sm, cudaStream_t st, uint64_t* h2d, std::string* why,
                   bool pin = true);

// Partition bucket of every row of a table (data_mngr.h:150-202) computed on
// the device from the partition and prefix columns only, in chunks of rows.
std::vector<uint32_t> bucket_rows(const Table& t, int part_col, int64_t prefix_idx,
                                  uint64_t n_partitions, int n_sm, cudaStream_t st);

// Page-locks the column buffers of a table (once; later calls return at
// once) so that copies from them run at full link speed.  Failure to lock is
// not an error: copies then go through the driver's staging buffers.
void pin_table(const hbx_table* t);

}  // namespace hbx
