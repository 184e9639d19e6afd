// capi.cpp -- host-only part of the C ABI: plans, tables, the output writer
// and the run_hyperblocker_exec command line.
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "hbx_core.h"

namespace {

// Error text for calls made without a context (plans and tables may be made
// before a context exists); hbx_last_error(nullptr) returns it.
thread_local std::string g_err;

hbx_status guard_host(hbx_ctx* ctx, const std::function<void()>& f);

}  // namespace

extern "C" const char* hbx_last_error(const hbx_ctx* ctx);

// hbx_ctx is defined in engine.cu; only its error string is touched here via
// this accessor, which engine.cu does not need.
struct hbx_ctx;
extern "C" void hbx_internal_set_error(hbx_ctx* ctx, const char* msg);
// writer.cu: the same lines formatted on the device
extern "C" hbx_status hbx_internal_write_pairs_via_device(hbx_ctx* ctx, const hbx_table* left,
                                                          const hbx_table* right,
                                                          const uint32_t* l_row,
                                                          const uint32_t* r_row, uint64_t n,
                                                          const char* path);

namespace {

hbx_status guard_host(hbx_ctx* ctx, const std::function<void()>& f) {
  try {
    f();
    return HBX_OK;
  } catch (const hbx::Error& e) {
    g_err = e.what();
    if (ctx) hbx_internal_set_error(ctx, e.what());
    return e.status;
  } catch (const std::bad_alloc&) {
    g_err = "host out of memory";
    if (ctx) hbx_internal_set_error(ctx, g_err.c_str());
    return HBX_ERR_OOM;
  } catch (const std::exception& e) {
    g_err = e.what();
    if (ctx) hbx_internal_set_error(ctx, e.what());
    return HBX_ERR_INVALID_ARG;
  }
}

}  // namespace

extern "C" {

const char* hbx_status_string(hbx_status s) {
  switch (s) {
    case HBX_OK: return "ok";
    case HBX_ERR_INVALID_ARG: return "invalid argument";
    case HBX_ERR_CUDA: return "CUDA error";
    case HBX_ERR_OOM: return "out of memory";
    case HBX_ERR_CAPACITY: return "output capacity too small";
    case HBX_ERR_WATCHDOG: return "watchdog budget exceeded";
    case HBX_ERR_PARSE: return "parse error";
    case HBX_ERR_IO: return "I/O error";
    case HBX_ERR_UNSUPPORTED: return "unsupported input";
    case HBX_ERR_TIMEOUT: return "timed out";
  }
  return "unknown status";
}

const char* hbx_host_last_error(void) { return g_err.c_str(); }

hbx_status hbx_plan_from_rule_dir(hbx_ctx* ctx, const char* rule_dir, hbx_plan** out) {
  if (!rule_dir || !out) return HBX_ERR_INVALID_ARG;
  *out = nullptr;
  auto p = std::make_unique<hbx_plan>();
  hbx_status s = guard_host(ctx, [&] { p->p = hbx::plan_from_dir(rule_dir); });
  if (s == HBX_OK) *out = p.release();
  return s;
}

hbx_status hbx_plan_from_yaml(hbx_ctx* ctx, const char* const* docs, int32_t n_docs,
                              hbx_plan** out) {
  if (!docs || n_docs < 0 || !out) return HBX_ERR_INVALID_ARG;
  *out = nullptr;
  auto p = std::make_unique<hbx_plan>();
  hbx_status s = guard_host(ctx, [&] {
    std::vector<std::pair<std::string, std::string>> v;
    for (int32_t i = 0; i < n_docs; i++) {
      if (!docs[i]) hbx::fail(HBX_ERR_INVALID_ARG, "null YAML document");
      v.emplace_back("doc" + std::to_string(i), docs[i]);
    }
    p->p = hbx::plan_from_docs(v);
  });
  if (s == HBX_OK) *out = p.release();
  return s;
}

hbx_status hbx_plan_serialized(const hbx_plan* plan, int32_t* length, const int32_t** pred_index,
                               const char** pred_type, const float** pred_threshold) {
  if (!plan || !length) return HBX_ERR_INVALID_ARG;
  *length = (int32_t)plan->p.pred_index.size();
  if (pred_index) *pred_index = plan->p.pred_index.data();
  if (pred_type) *pred_type = plan->p.pred_type.data();
  if (pred_threshold) *pred_threshold = plan->p.pred_threshold.data();
  return HBX_OK;
}

int32_t hbx_plan_n_rules(const hbx_plan* plan) { return plan ? (int32_t)plan->p.rules.size() : -1; }

hbx_status hbx_plan_destroy(hbx_plan* plan) {
  if (!plan) return HBX_ERR_INVALID_ARG;
  delete plan;
  return HBX_OK;
}

hbx_status hbx_table_from_csv(hbx_ctx* ctx, const char* path, char sep, hbx_table** out) {
  if (!path || !out) return HBX_ERR_INVALID_ARG;
  *out = nullptr;
  auto t = std::make_unique<hbx_table>();
  t->uid = hbx::next_table_uid();
  hbx_status s = guard_host(ctx, [&] { t->t = hbx::table_from_csv(path, sep ? sep : ',', ctx); });
  if (s == HBX_OK) *out = t.release();
  return s;
}

hbx_status hbx_table_ingest(hbx_ctx* ctx, const hbx_columns* cols, hbx_table** out) {
  if (!cols || !out) return HBX_ERR_INVALID_ARG;
  *out = nullptr;
  auto t = std::make_unique<hbx_table>();
  t->uid = hbx::next_table_uid();
  hbx_status s = guard_host(ctx, [&] { t->t = hbx::table_from_columns(cols); });
  if (s == HBX_OK) *out = t.release();
  return s;
}

int64_t hbx_table_n_rows(const hbx_table* t) { return t ? t->t.n_rows : -1; }
int32_t hbx_table_n_cols(const hbx_table* t) { return t ? t->t.n_cols() : -1; }

hbx_status hbx_table_column(const hbx_table* t, int32_t c, const char** bytes,
                            const int64_t** offsets) {
  if (!t || !bytes || !offsets || c < 0 || c >= t->t.n_cols()) return HBX_ERR_INVALID_ARG;
  const hbx::Column& col = t->t.cols[(size_t)c];
  *bytes = col.bytes.data();
  *offsets = col.off.data();
  return HBX_OK;
}

hbx_status hbx_table_destroy(hbx_table* t) {
  if (!t) return HBX_ERR_INVALID_ARG;
  hbx::unpin_table(t);
  delete t;
  return HBX_OK;
}

hbx_status hbx_write_pairs(hbx_ctx* ctx, const hbx_table* left, const hbx_table* right,
                           const uint32_t* l_row, const uint32_t* r_row, uint64_t n,
                           const char* path) {
  if (!left || !right || !path || (n && (!l_row || !r_row))) return HBX_ERR_INVALID_ARG;
  // with a context, many pairs are formatted on its device
  constexpr uint64_t kDeviceMin = 1 << 16;
  if (ctx && n >= kDeviceMin)
    return hbx_internal_write_pairs_via_device(ctx, left, right, l_row, r_row, n, path);
  return guard_host(ctx, [&] {
    if (left->t.n_cols() == 0 || right->t.n_cols() == 0)
      hbx::fail(HBX_ERR_INVALID_ARG, "table without an id column");
    const hbx::Column& il = left->t.cols[0];
    const hbx::Column& ir = right->t.cols[0];
    std::string buf;
    buf.reserve((size_t)std::min<uint64_t>(n, 1u << 20) * 24);
    FILE* f = std::fopen(path, "ab");
    if (!f) hbx::fail(HBX_ERR_IO, std::string("cannot open ") + path);
    auto flush = [&] {
      if (!buf.empty() && std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) {
        std::fclose(f);
        hbx::fail(HBX_ERR_IO, std::string("write failed: ") + path);
      }
      buf.clear();
    };
    for (uint64_t i = 0; i < n; i++) {
      if ((int64_t)l_row[i] >= left->t.n_rows || (int64_t)r_row[i] >= right->t.n_rows) {
        std::fclose(f);
        hbx::fail(HBX_ERR_INVALID_ARG, "row index out of range");
      }
      // the reference prints each id as a C string (host_reducer.h:85-86)
      const char* a = il.ptr(l_row[i]);
      const char* b = ir.ptr(r_row[i]);
      buf.append(a, strnlen(a, (size_t)il.len(l_row[i])));
      buf.push_back(',');
      buf.append(b, strnlen(b, (size_t)ir.len(r_row[i])));
      buf.push_back('\n');
      if (buf.size() > (1u << 22)) flush();
    }
    flush();
    if (std::fclose(f) != 0) hbx::fail(HBX_ERR_IO, std::string("close failed: ") + path);
  });
}

}  // extern "C"
