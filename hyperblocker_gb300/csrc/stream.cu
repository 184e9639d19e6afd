// stream.cu -- blocking in partition windows under a device-memory budget
// (hbx_block_streamed).
//
// Pairs are only ever compared inside one reference partition
// (data_mngr.h:150-216), so the partitions can be processed in any grouping:
// every row's partition is computed first (on the device, from the partition
// column alone), rows are grouped by partition on the host, and consecutive
// partitions are packed into windows whose encoded size stays under the
// budget.  A partition larger than a window is split by its left rows (every
// left chunk meets all of the partition's right rows: the chunks' products
// tile the partition's product).  Two workers, each with its own context and
// stream, take windows in turn: while one window's rows are copied to the
// device and encoded, the other's are evaluated, so copies overlap compute.
// Each window is an ordinary session over the window's rows, so the pairs are
// exactly the ones hbx_block returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "context.h"
#include "device_buffers.h"
#include "encode.h"
#include "engine.h"
#include "hbx_core.h"
#include "ingest.h"

namespace hbx {
namespace {

struct Window {
  uint64_t p0 = 0, p1 = 0;           // partitions [p0, p1)
  uint64_t l0 = 0, l1 = UINT64_MAX;  // left rows of the (single) partition p0, when split
};

// A sub-table holding rows idx of t: the columns the plan reads are copied,
// the others are left empty (their cells are never read).
void sub_table(const Table& t, const std::vector<int>& used, const uint32_t* idx, size_t n,
               Table* out) {
  out->n_rows = (int64_t)n;
  out->cols.assign(t.cols.size(), Column{});
  for (size_t c = 0; c < t.cols.size(); c++) {
    Column& d = out->cols[c];
    d.off.assign(n + 1, 0);
    if (!std::binary_search(used.begin(), used.end(), (int)c)) continue;
    const Column& s = t.cols[c];
    size_t bytes = 0;
    for (size_t i = 0; i < n; i++) bytes += (size_t)s.len(idx[i]);
    d.bytes.resize(bytes);
    size_t pos = 0;
    for (size_t i = 0; i < n; i++) {
      const int64_t len = s.len(idx[i]);
      if (len) std::memcpy(d.bytes.data() + pos, s.ptr(idx[i]), (size_t)len);
      pos += (size_t)len;
      d.off[i + 1] = (int64_t)pos;
    }
    d.has_nul = s.has_nul;
  }
}

}  // namespace
}  // namespace hbx

using namespace hbx;

extern "C" hbx_status hbx_block_streamed(hbx_ctx* ctx, const hbx_plan* plan, const hbx_table* left,
                                         const hbx_table* right, uint64_t n_partitions,
                                         int64_t prefix_idx, hbx_mode mode, uint64_t window_bytes,
                                         hbx_pairs* out, hbx_stats* stats) {
  if (!ctx || !plan || !left || !right || !out || window_bytes == 0) return HBX_ERR_INVALID_ARG;
  if (mode != HBX_MODE_PLAIN && mode != HBX_MODE_BATCHED) return HBX_ERR_INVALID_ARG;
  const auto t0 = std::chrono::steady_clock::now();
  hbx_stats agg{};
  try {
    if (prefix_idx != INT_MAX && (prefix_idx < 0 || prefix_idx > INT_MAX))
      fail(HBX_ERR_INVALID_ARG, "prefix_idx out of range");
    HBX_CUDA(cudaSetDevice(ctx->device));
    const Table& TL = left->t;
    const Table& TR = right->t;
    // the evaluation order is measured once on the whole tables
    hbx_plan ordered;
    ordered.p = plan->p;
    if (ctx->opts.pred_order == 0) order_predicates(&ordered.p, TL, TR);
    const Encoded schema = encode_schema(ordered.p, TL, TR, n_partitions, prefix_idx);
    std::vector<int> used_l, used_r;
    auto use = [](std::vector<int>& v, int c) {
      if (c >= 0) v.push_back(c);
    };
    use(used_l, 0);
    use(used_r, 0);
    use(used_l, schema.part_col);
    use(used_r, schema.part_col);
    if (prefix_idx != INT_MAX) {
      use(used_l, (int)prefix_idx);
      use(used_r, (int)prefix_idx);
    }
    for (auto& e : schema.eq_slots) {
      use(used_l, e.first);
      use(used_r, e.second);
    }
    for (int c : schema.L.str_col) use(used_l, c);
    for (int c : schema.R.str_col) use(used_r, c);
    for (auto* v : {&used_l, &used_r}) {
      std::sort(v->begin(), v->end());
      v->erase(std::unique(v->begin(), v->end()), v->end());
    }

    // ---- every row's partition, rows grouped by partition
    std::vector<uint32_t> bl, br;
    {
      PoolScope scope(ctx->pool, ctx->stream);
      bl = bucket_rows(TL, schema.part_col, prefix_idx, n_partitions, ctx->n_sm, ctx->stream);
      br = bucket_rows(TR, schema.part_col, prefix_idx, n_partitions, ctx->n_sm, ctx->stream);
    }
    auto group = [&](const std::vector<uint32_t>& b, std::vector<uint64_t>* start,
                     std::vector<uint32_t>* rows) {
      start->assign(n_partitions + 1, 0);
      for (uint32_t x : b) (*start)[x + 1]++;
      for (uint64_t p = 0; p < n_partitions; p++) (*start)[p + 1] += (*start)[p];
      rows->resize(b.size());
      std::vector<uint64_t> cur(start->begin(), start->end() - 1);
      for (size_t i = 0; i < b.size(); i++) (*rows)[cur[b[i]]++] = (uint32_t)i;
    };
    std::vector<uint64_t> sl, sr;
    std::vector<uint32_t> rl, rr;
    group(bl, &sl, &rl);
    group(br, &sr, &rr);

    // ---- device bytes of a row in a window (encoded strings, metadata, codes,
    // join state), an upper bound
    auto row_cost = [&](const Table& t, const std::vector<int>& used, const std::vector<int>& str,
                        size_t n_eq, uint32_t row) {
      uint64_t c = 64 + 4 * n_eq + 16 * schema.rules.size();
      for (int col : used) c += (uint64_t)t.cols[(size_t)col].len(row) + 8;
      for (int col : str) c += (uint64_t)t.cols[(size_t)col].len(row) + 16 + sizeof(dev::StrMeta);
      return c;
    };
    std::vector<uint64_t> cost_l(n_partitions, 0), cost_r(n_partitions, 0);
    std::vector<uint64_t> row_cost_l(TL.n_rows);
    for (uint32_t i = 0; i < (uint32_t)TL.n_rows; i++) {
      row_cost_l[i] = row_cost(TL, used_l, schema.L.str_col, schema.eq_slots.size(), i);
      cost_l[bl[i]] += row_cost_l[i];
    }
    for (uint32_t i = 0; i < (uint32_t)TR.n_rows; i++)
      cost_r[br[i]] += row_cost(TR, used_r, schema.R.str_col, schema.eq_slots.size(), i);

    // ---- windows: consecutive partitions under the budget; a partition above
    // it alone is split by its left rows
    std::vector<Window> windows;
    {
      Window w;
      uint64_t acc = 0;
      for (uint64_t p = 0; p < n_partitions; p++) {
        if (sl[p + 1] == sl[p] || sr[p + 1] == sr[p]) continue;  // no pairs
        const uint64_t c = cost_l[p] + cost_r[p];
        if (c > window_bytes) {
          if (w.p1 > w.p0) windows.push_back(w);
          uint64_t a = sl[p], room = window_bytes > cost_r[p] ? window_bytes - cost_r[p] : 0;
          while (a < sl[p + 1]) {
            uint64_t b = a, sum = 0;
            while (b < sl[p + 1] && (b == a || sum + row_cost_l[rl[b]] <= room)) sum += row_cost_l[rl[b++]];
            Window x;
            x.p0 = p;
            x.p1 = p + 1;
            x.l0 = a;
            x.l1 = b;
            windows.push_back(x);
            a = b;
          }
          w = Window{};
          acc = 0;
          continue;
        }
        if (w.p1 > w.p0 && acc + c > window_bytes) {
          windows.push_back(w);
          w = Window{};
          acc = 0;
        }
        if (w.p1 == w.p0) w.p0 = w.p1 = p;
        w.p1 = p + 1;
        acc += c;
      }
      if (w.p1 > w.p0) windows.push_back(w);
    }

    // ---- two workers, each with its own context and stream.  A window's
    // copies and encoding run while the other worker's window is joined and
    // evaluated; the runs themselves take turns (run_mu): two persistent
    // evaluations side by side split the SMs unevenly (the one launched
    // second starts on the slots the first leaves), and the whole call then
    // waits for the starved one.
    std::atomic<size_t> next{0};
    std::vector<std::vector<uint32_t>> win_l(windows.size()), win_r(windows.size());
    std::mutex mu, run_mu;
    // matches per pair covered in the windows done so far: sizes the next
    // windows' output so that their runs do not overflow and repeat
    double density = -1.0;
    hbx_status err = HBX_OK;
    std::string err_text;
    auto worker = [&](int id) {
      hbx_ctx* wc = nullptr;
      hbx_opts o = ctx->opts;
      o.pred_order = 1;  // the plan is already in measured order
      // windows differ in size: one fixed tile shape and kernel instead of an
      // autotuning search per window.  96 right rows per item (one staging
      // buffer, 85 KB of shared memory per block) measured best: on the C5
      // shape (500k x 500k, 64-256 character strings) 1.36 s of evaluation
      // against 2.37 s with 64 rows (two buffers) and 2.44 s with 128 rows
      // (one buffer), both of which take 103 KB per block and so leave less
      // of each SM's L1 to the Peq rows the scans read; on C3 96 and 128
      // rows are within 1 %
      if (o.tile_right <= 0) o.tile_right = 96;
      if (o.eval_variant <= 0) o.eval_variant = 2;
      if (hbx_ctx_create(ctx->device, &o, &wc) != HBX_OK) {
        std::lock_guard<std::mutex> lock(mu);
        if (err == HBX_OK) {
          err = HBX_ERR_CUDA;
          err_text = "stream worker context";
        }
        return;
      }
      (void)id;
      std::vector<uint32_t> il, ir, l, r;
      for (;;) {
        {
          std::lock_guard<std::mutex> lock(mu);
          if (err != HBX_OK) break;
        }
        const size_t k = next.fetch_add(1);
        if (k >= windows.size()) break;
        const Window& w = windows[k];
        il.clear();
        ir.clear();
        for (uint64_t p = w.p0; p < w.p1; p++) {
          const uint64_t a = std::max(sl[p], w.l0 == 0 && w.l1 == UINT64_MAX ? sl[p] : w.l0);
          const uint64_t b = std::min(sl[p + 1], w.l1);
          il.insert(il.end(), rl.begin() + (long)a, rl.begin() + (long)b);
          ir.insert(ir.end(), rr.begin() + (long)sr[p], rr.begin() + (long)sr[p + 1]);
        }
        hbx_table subl, subr;
        subl.uid = next_table_uid();
        subr.uid = next_table_uid();
        subl.pin_tried = subr.pin_tried = true;  // short-lived: copied, not page-locked
        sub_table(TL, used_l, il.data(), il.size(), &subl.t);
        sub_table(TR, used_r, ir.data(), ir.size(), &subr.t);
        hbx_session* s = nullptr;
        hbx_status st = hbx_session_create(wc, &ordered, &subl, &subr, n_partitions, prefix_idx, &s);
        hbx_stats ws{};
        if (st == HBX_OK) {
          try {
            double d;
            {
              std::lock_guard<std::mutex> lock(mu);
              d = density;
            }
            // output slots before the run, so that it does not overflow and
            // evaluate the window again: from the match density of the
            // windows done so far, or, for the first windows, as many as the
            // window's pairs can give, up to window_bytes / 8 slots
            hbx_stats pre{};
            hbx_session_stats(s, &pre);
            const uint64_t cap = std::max<uint64_t>(window_bytes / 8, 1 << 16);
            const double want =
                d >= 0 ? 1.5 * d * (double)pre.pairs_covered + 4096.0 : (double)pre.pairs_covered + 1.0;
            reserve_output(s, (uint64_t)std::min<double>(want, (double)cap));
            {
              std::lock_guard<std::mutex> turn(run_mu);
              run_to_host(s, mode, &l, &r);
            }
            hbx_session_stats(s, &ws);
          } catch (const Error& e) {
            st = e.status;
            wc->err = e.what();
          }
        }
        if (s) hbx_session_destroy(s);
        if (st == HBX_OK) {
          // the window's rows back to table rows, outside the lock: each
          // window has its own result vectors, joined once at the end
          std::vector<uint32_t>& wl = win_l[k];
          std::vector<uint32_t>& wr = win_r[k];
          wl.resize(l.size());
          wr.resize(r.size());
          for (size_t i = 0; i < l.size(); i++) {
            wl[i] = il[l[i]];
            wr[i] = ir[r[i]];
          }
        }
        std::lock_guard<std::mutex> lock(mu);
        if (st != HBX_OK) {
          if (err == HBX_OK) {
            err = st;
            err_text = hbx_last_error(wc);
          }
          break;
        }
        if (ws.pairs_covered)
          density = std::max(density, (double)l.size() / (double)ws.pairs_covered);
        agg.pair_comparisons += ws.pair_comparisons;
        agg.fma_ambiguous += ws.fma_ambiguous;
        agg.long_string_pairs += ws.long_string_pairs;
        agg.n_tiles += ws.n_tiles;
        agg.n_launches += ws.n_launches;
        agg.ms_join += ws.ms_join;
        agg.ms_eval += ws.ms_eval;
        agg.jw_word_ops += ws.jw_word_ops;
        agg.h2d_bytes += ws.h2d_bytes;
        agg.ms_create += ws.ms_create;
        agg.ingest_on_device = ws.ingest_on_device;
        agg.tile_right = ws.tile_right;
        agg.eval_variant = ws.eval_variant;
        agg.pairs_scanned += ws.pairs_scanned;
        agg.scan_steps += ws.scan_steps;
        agg.scan_word_ops += ws.scan_word_ops;
        agg.scan_warp_steps += ws.scan_warp_steps;
        agg.rest_scans += ws.rest_scans;
        agg.scan_words = std::max(agg.scan_words, ws.scan_words);
      }
      hbx_ctx_destroy(wc);
    };
    const int n_workers = windows.size() > 1 ? 2 : 1;
    std::vector<std::thread> th;
    for (int i = 0; i < n_workers; i++) th.emplace_back(worker, i);
    for (auto& t : th) t.join();
    if (err != HBX_OK) fail(err, err_text);
    for (uint64_t p = 0; p < n_partitions; p++) {
      const uint64_t a = sl[p + 1] - sl[p], b = sr[p + 1] - sr[p];
      agg.pairs_covered += a * b;
      if (a && b) agg.n_partitions_used++;
    }
    agg.n_windows = (uint32_t)windows.size();
    size_t total = 0;
    for (auto& v : win_l) total += v.size();
    agg.n_matches = total;
    out->n_required = total;
    out->n_written = 0;
    if (total > out->capacity) fail(HBX_ERR_CAPACITY, "output capacity below the match count");
    if (total && (!out->l_row || !out->r_row)) fail(HBX_ERR_INVALID_ARG, "null output pointer");
    size_t pos = 0;
    for (size_t k = 0; k < windows.size(); k++) {
      if (win_l[k].empty()) continue;
      std::memcpy(out->l_row + pos, win_l[k].data(), win_l[k].size() * 4);
      std::memcpy(out->r_row + pos, win_r[k].data(), win_r[k].size() * 4);
      pos += win_l[k].size();
    }
    out->n_written = total;
  } catch (const Error& e) {
    ctx->err = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    ctx->err = "host out of memory";
    return HBX_ERR_OOM;
  }
  agg.ms_last_run =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = agg;
  ctx->err.clear();
  return HBX_OK;
}
