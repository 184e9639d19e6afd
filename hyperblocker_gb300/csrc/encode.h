// encode.h -- host-side encoding of two tables for one plan.
#pragma once

#include <array>
#include <cstdint>
#include <vector>

#include "hbx_core.h"

namespace hbx {

constexpr uint32_t kMaxKeyDomain = 1u << 24;  // device counting-sort domain per rule

struct SideEnc {
  int64_t n_rows = 0;
  std::vector<uint32_t> bucket;                // reference partition of each row
  std::vector<std::vector<int32_t>> eq_codes;  // per equality slot
  std::vector<std::vector<int32_t>> comp_codes;// per composite-key rule (see RuleEnc)
  std::vector<uint8_t> arena;                  // symbol strings, 16-byte aligned, zero padded
  std::vector<std::vector<uint32_t>> str_off;  // per string slot: offset / 16
  std::vector<std::vector<uint32_t>> str_len;  // per string slot: byte length (strlen)
  std::vector<uint32_t> str_maxlen;            // per string slot
  std::vector<int> str_col;                    // per string slot: table column
};

struct RuleEnc {
  std::vector<int> eq_slot;    // equality slots (joint dictionaries)
  std::vector<int> sim_slot_l; // string slot of the left column, evaluation order
  std::vector<int> sim_slot_r;
  std::vector<float> thr;
  // join key: key = bucket * radix_total + mixed(eq codes), or the dense
  // composite code when that domain would exceed kMaxKeyDomain.
  bool composite = false;
  int comp_index = -1;               // index into SideEnc::comp_codes
  std::vector<uint32_t> radix;       // cardinality of each eq slot
  uint64_t domain = 0;               // key domain size D
  std::vector<uint64_t> part_key_begin;  // n_partitions + 1: first key of each partition
};

struct Encoded {
  uint64_t n_partitions = 1;
  SideEnc L, R;
  std::vector<std::pair<int, int>> eq_slots;  // (left col, right col)
  std::vector<uint32_t> eq_card;
  std::array<uint8_t, 256> sym_of_byte{};     // 0 = byte never occurs in a string column
  uint32_t n_symbols = 1;                     // including the padding symbol 0
  std::vector<RuleEnc> rules;
  uint64_t pairs_covered = 0;
  uint32_t n_partitions_used = 0;
};

// Builds the encoding; throws hbx::Error on inputs the reference cannot run.
Encoded encode(const Plan& plan, const Table& left, const Table& right, uint64_t n_partitions,
               int64_t prefix_idx);

}  // namespace hbx
