// ingest.h -- encoding of two host tables on the device.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "device_buffers.h"
#include "encode.h"
#include "hbx_core.h"

namespace hbx {

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
// domains, and *h2d the bytes copied.  Returns false, with the reason in
// *why, when only the host encoder is exact for the input: a rule whose join
// keys need composite ids, or two distinct cells of a dictionary column with
// the same 64-bit hash (detected by comparing every cell with its slot's
// representative).  The side buffers are then left empty.
bool device_encode(const hbx_table* left, const hbx_table* right, Encoded* E, SideBufs* L,
                   SideBufs* R, int n_sm, cudaStream_t st, uint64_t* h2d, std::string* why);

// Page-locks the column buffers of a table (once; later calls return at
// once) so that copies from them run at full link speed.  Failure to lock is
// not an error: copies then go through the driver's staging buffers.
void pin_table(const hbx_table* t);

}  // namespace hbx
