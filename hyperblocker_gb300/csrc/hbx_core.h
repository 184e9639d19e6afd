// hbx_core.h -- internal types of the blocking engine (host side).
#pragma once

#include <cstdint>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/hbx.h"

namespace hbx {

// Error carried from deep inside the host code to the C ABI, where it becomes
// an hbx_status plus hbx_last_error() text.
struct Error : std::runtime_error {
  hbx_status status;
  Error(hbx_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] inline void fail(hbx_status s, const std::string& m) { throw Error(s, m); }

constexpr int kCheckPoint = 2147483647;  // core/common/types.h:13
constexpr int kMaxEqPerRule = 8;
constexpr int kMaxSimPerRule = 8;
constexpr int kMaxRules = 64;
constexpr int kFastMaxLen = 256;  // bit-parallel JW for left strings up to this length

// One column of host strings: cell i = bytes[off[i] .. off[i+1]).
struct Column {
  std::vector<char> bytes;
  std::vector<int64_t> off;  // n_rows + 1
  bool has_nul = false;      // some cell holds a NUL byte (cells compare up to it)
  const char* ptr(int64_t i) const { return bytes.data() + off[(size_t)i]; }
  int64_t len(int64_t i) const { return off[(size_t)i + 1] - off[(size_t)i]; }
};

struct Table {
  int64_t n_rows = 0;
  std::vector<Column> cols;
  int32_t n_cols() const { return (int32_t)cols.size(); }
};

// A decoded rule (core/data_structures/rule.h:12-28, yaml_config.h:37-75).
struct RuleDef {
  std::vector<int> relation_l, relation_r, eq, sim;
  std::vector<std::pair<int, float>> threshold;  // insertion order, first key wins
  std::vector<int> con_eq;
  std::string source;
  const float* find_threshold(int col) const {
    for (auto& kv : threshold)
      if (kv.first == col) return &kv.second;
    return nullptr;
  }
};

struct Pred {
  char type;   // 'e' or 's'
  int col_l;   // column of the left table
  int col_r;   // column of the right table
  float thr;   // threshold of the left slot (similarity only)
};

struct CompiledRule {
  std::vector<Pred> eqs;
  std::vector<Pred> sims;  // evaluation order (cost-ordered)
};

struct Plan {
  std::vector<RuleDef> rules;  // reference order (after std::sort)
  std::vector<int32_t> pred_index;
  std::vector<char> pred_type;
  std::vector<float> pred_threshold;
  std::vector<CompiledRule> compiled;  // same order as rules
};

// rules.cpp
Plan plan_from_docs(const std::vector<std::pair<std::string, std::string>>& named_docs);
Plan plan_from_dir(const std::string& dir);

// csv.cpp
// The reference's tokenization of a CSV buffer (csv.cpp).
Table table_from_buffer(const char* data, size_t n, char sep);
// With a context and at least kDeviceCsvMin bytes the file is tokenized on
// the context's device (csv_gpu.cu), into the same table.
Table table_from_csv(const std::string& path, char sep, hbx_ctx* ctx = nullptr);
constexpr size_t kDeviceCsvMin = 1u << 20;
// table_from_buffer on the device; false when the input needs the host loop
// (a first line without cells, a column of 4 GiB or more, 2^31 rows or more).
bool table_from_buffer_device(hbx_ctx* ctx, const char* data, size_t n, char sep, Table* out);
Table table_from_columns(const hbx_columns* cols);

// Measured-selectivity ordering of similarity predicates (planner.cpp).
void order_predicates(Plan* plan, const Table& left, const Table& right);

}  // namespace hbx

struct hbx_plan {
  hbx::Plan p;
  // Evaluation order measured for a (left table, right table) pair, by table
  // uid.  Tables never change after creation, so an entry stays valid.
  std::mutex order_mu;
  std::map<std::pair<uint64_t, uint64_t>, std::vector<hbx::CompiledRule>> order_cache;
};
struct hbx_table {
  hbx::Table t;
  uint64_t uid = 0;  // unique per table created in this process
  // page-locked column buffers (pin_table), released by hbx_table_destroy
  std::mutex pin_mu;
  bool pin_tried = false;
  std::vector<void*> pinned;
};

namespace hbx {
// Sets has_nul of every column (after a table is built).
void finish_table(Table* t);
// Unlocks what pin_table locked (engine side; no CUDA call when nothing is).
void unpin_table(hbx_table* t);
// Next table uid.
uint64_t next_table_uid();
}  // namespace hbx
