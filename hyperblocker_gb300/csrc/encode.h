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
  int part_col = -1;             // column hashed for the partition bucket, -1 = none
  int64_t prefix_idx = 2147483647;  // column of the first-character hash (INT_MAX = none)
  SideEnc L, R;
  std::vector<std::pair<int, int>> eq_slots;  // (left col, right col)
  std::vector<uint32_t> eq_card;
  std::array<uint8_t, 256> sym_of_byte{};     // 0 = byte never occurs in a string column
  uint32_t n_symbols = 1;                     // including the padding symbol 0
  std::vector<RuleEnc> rules;
  uint64_t pairs_covered = 0;
  uint32_t n_partitions_used = 0;
};

// Slots and rules of a plan over two tables, without per-row data: checks the
// columns, gives each (left column, right column) equality pair a joint
// dictionary slot and each similarity column a string slot.  Throws
// hbx::Error on inputs the reference cannot run.
Encoded encode_schema(const Plan& plan, const Table& left, const Table& right,
                      uint64_t n_partitions, int64_t prefix_idx);
// Host encoding of every row: buckets, dictionary codes, symbols, arenas.
void encode_rows(const Table& left, const Table& right, Encoded* E);
// Join-key domains from the dictionary sizes.  A rule whose mixed-radix
// domain exceeds kMaxKeyDomain gets dense composite ids, which are built from
// the host codes of encode_rows; with allow_composite false such a rule makes
// this return false instead.
bool finish_rules(Encoded* E, bool allow_composite);
// One rule's mixed-radix join-key domain (bucket x eq codes) from the
// dictionary sizes, when it is at most kMaxKeyDomain: sets radix, domain and
// part_key_begin and returns true; else returns false (composite ids needed).
bool rule_mixed_domain(const Encoded& E, RuleEnc* re);
// The whole host encoding (schema, rows, domains).
Encoded encode(const Plan& plan, const Table& left, const Table& right, uint64_t n_partitions,
               int64_t prefix_idx);

}  // namespace hbx
