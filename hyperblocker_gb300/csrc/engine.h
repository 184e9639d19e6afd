// engine.h -- engine entry points used by other translation units.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/hbx.h"

namespace hbx {

// Runs a session (batched or plain) on its context's stream and copies its
// pairs, exactly sized, into host vectors.
void run_to_host(hbx_session* s, hbx_mode mode, std::vector<uint32_t>* l, std::vector<uint32_t>* r);
// Grows a session's own output (and duplicate set) to at least `pairs`
// slots before a run, so that a run expected to produce that many pairs
// does not overflow and repeat.
void reserve_output(hbx_session* s, uint64_t pairs);
struct Table;
// sort.cu: sorts n device pairs by (left row, right row) in place.
void sort_pairs_device(hbx_ctx* ctx, uint32_t* l, uint32_t* r, uint64_t n, uint32_t n_left,
                       uint32_t n_right);
// writer.cu: appends the id lines of n device pairs to path.
void write_pairs_device(hbx_ctx* ctx, const Table& left, const Table& right, const uint32_t* l_row,
                        const uint32_t* r_row, uint64_t n, const char* path);

}  // namespace hbx
