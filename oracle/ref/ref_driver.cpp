// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own blocking_kernel (core/gpu/global_func.cuh:104-185,
// with equalities_kernel, lev_jaro_ratio and lev_jaro_winkler_ratio from
// core/gpu/device_func.cuh) on CPU threads.  The reference headers are
// compiled unchanged from the reference checkout by oracle/ref/build_ref.sh;
// this file only supplies what the reference's host side would: the
// fixed-width row-major table layout of core/data_structures/table.h:75-128
// (restated below, zero-filled) and the launch loop of
// core/components/host_producer.h:115-203 (grid 64 x block 64).
#include "ref_cuda_shim.h"

#include <thread>

#include "core/data_structures/rule.h"
#include "yaml_decl.h"
#include "core/gpu/global_func.cuh"

thread_local hbref_dim3 blockIdx;
thread_local hbref_dim3 threadIdx;
hbref_dim3 blockDim{64, 1, 1};
hbref_dim3 gridDim{64, 1, 1};
int hbref_candidate_capacity = 65536;

namespace {

struct FixedTable {
  size_t n_rows = 0, n_cols = 0, tuple = 0;
  std::vector<size_t> col_size, col_offset;
  std::vector<char> data;
};

// table.h:87-126: col_size = max length + 1, col_offset = prefix sum,
// tuple = (((sum + 1) >> 6) << 6) + 64, cells memcpy'd without terminator
// into zero-filled rows.
FixedTable serialize(size_t n_rows, size_t n_cols, const char* const* ptr, const int64_t* len,
                     const int64_t* rows) {
  FixedTable t;
  t.n_rows = n_rows;
  t.n_cols = n_cols;
  t.col_size.assign(n_cols, 0);
  t.col_offset.assign(n_cols, 0);
  for (size_t c = 0; c < n_cols; c++) {
    size_t mx = 0;
    for (size_t i = 0; i < n_rows; i++) mx = std::max(mx, (size_t)len[rows[i] * n_cols + c]);
    t.col_size[c] = mx + 1;
  }
  size_t sum = 0;
  for (size_t c = 0; c < n_cols; c++) {
    sum += t.col_size[c];
    if (c > 0) t.col_offset[c] = t.col_offset[c - 1] + t.col_size[c - 1];
  }
  t.tuple = (((sum + 1) >> 6) << 6) + 64;
  t.data.assign(n_rows * t.tuple, 0);
  for (size_t c = 0; c < n_cols; c++)
    for (size_t i = 0; i < n_rows; i++) {
      const int64_t k = rows[i] * (int64_t)n_cols + (int64_t)c;
      std::memcpy(t.data.data() + t.tuple * i + t.col_offset[c], ptr[k], (size_t)len[k]);
    }
  return t;
}

}  // namespace

extern "C" {

// Evaluates one partition (left rows rows_l[0..n_l), right rows rows_r[0..n_r))
// with the reference kernel.  Tables are row-major cells (ptr, len) with n_cols
// columns.  Candidates are written as the kernel writes them: 128-byte slots,
// left id in bytes 0..63, right id in 64..127.  Returns the candidate count, or
// -(count) when capacity was too small (retry with a bigger buffer).
int64_t hbref_block_partition(int32_t n_cols_l, const char* const* ptr_l, const int64_t* len_l,
                              const int64_t* rows_l, int64_t n_l, int32_t n_cols_r,
                              const char* const* ptr_r, const int64_t* len_r,
                              const int64_t* rows_r, int64_t n_r, const int* pred_index,
                              const char* pred_type, const float* pred_threshold, int plan_len,
                              int n_threads, char* cand_out, int64_t capacity) {
  using sics::hyperblocker::core::components::SerializedExecutionPlan;
  if (n_l <= 0 || n_r <= 0) return 0;
  FixedTable L = serialize((size_t)n_l, (size_t)n_cols_l, ptr_l, len_l, rows_l);
  FixedTable R = serialize((size_t)n_r, (size_t)n_cols_r, ptr_r, len_r, rows_r);
  std::vector<int> pi(pred_index, pred_index + plan_len);
  std::vector<char> pt(pred_type, pred_type + plan_len);
  std::vector<float> pth(pred_threshold, pred_threshold + plan_len);
  // The kernel may read one slot past a rule's last predicate; pad with a
  // checkpoint so that read stays inside the arrays.
  pi.push_back(CHECK_POINT);
  pt.push_back(CHECK_POINT_CHAR);
  pth.push_back(1.0f);
  SerializedExecutionPlan sep;
  sep.n_rules = 0;
  sep.length = plan_len;
  sep.pred_index = pi.data();
  sep.pred_type = pt.data();
  sep.pred_threshold = pth.data();

  hbref_candidate_capacity = (int)std::min<int64_t>(capacity, INT_MAX / 256);
  int result_offset = 0;
  if (n_threads < 1) n_threads = 1;
  const unsigned total = gridDim.x * blockDim.x;
  auto worker = [&](int tid) {
    for (unsigned e = (unsigned)tid; e < total; e += (unsigned)n_threads) {
      blockIdx = {e / blockDim.x, 0, 0};
      threadIdx = {e % blockDim.x, 0, 0};
      sics::hyperblocker::core::gpu::blocking_kernel(
          L.n_rows, R.n_rows, L.tuple, R.tuple, L.data.data(), R.data.data(),
          L.col_size.data(), R.col_size.data(), L.col_offset.data(), R.col_offset.data(), sep,
          &result_offset, cand_out);
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < n_threads; t++) th.emplace_back(worker, t);
  worker(0);
  for (auto& t : th) t.join();
  if ((int64_t)result_offset > (int64_t)hbref_candidate_capacity) return -(int64_t)result_offset;
  return result_offset;
}

}  // extern "C"
