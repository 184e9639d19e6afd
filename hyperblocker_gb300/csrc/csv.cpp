// csv.cpp -- CSV ingest with the reference's tokenization.
//
// The reference reads tables with rapidcsv::Document(path, LabelParams(-1,-1),
// SeparatorParams(sep)) (core/components/data_mngr.h:48-51): the header line
// is a data row and every cell is a std::string.  rapidcsv is not vendored in
// the reference; this file implements the tokenization of rapidcsv 8.x with
// the default parameters the reference uses (no trimming, CR dropped, no
// quoted line breaks, automatic unquoting, UTF-8 BOM skipped) directly into
// column-major byte arenas instead of a vector<vector<string>>.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <fstream>

#include "hbx_core.h"

namespace hbx {

namespace {

struct RowBuilder {
  std::vector<std::vector<char>> cells_bytes;  // per column
  std::vector<std::vector<int64_t>> cells_off;
  std::vector<std::pair<int64_t, int64_t>> row;  // (start, len) into scratch
  std::vector<char> scratch;
  int64_t n_rows = 0;
  int32_t n_cols = -1;

  void push_cell(const char* p, size_t n) {
    // unquote: "..." -> ..., "" -> "
    size_t start = scratch.size();
    if (n >= 2 && p[0] == '"' && p[n - 1] == '"') {
      for (size_t i = 1; i + 1 < n; i++) {
        scratch.push_back(p[i]);
        if (p[i] == '"' && i + 2 < n && p[i + 1] == '"') i++;
      }
    } else {
      scratch.insert(scratch.end(), p, p + n);
    }
    row.emplace_back((int64_t)start, (int64_t)(scratch.size() - start));
  }

  void end_row() {
    if (n_cols < 0) {
      n_cols = (int32_t)row.size();
      cells_bytes.assign((size_t)n_cols, {});
      cells_off.assign((size_t)n_cols, std::vector<int64_t>{0});
    }
    if ((int32_t)row.size() < n_cols) {
      char msg[160];
      std::snprintf(msg, sizeof msg, "row %lld has %d cells, expected %d",
                    (long long)n_rows, (int)row.size(), n_cols);
      fail(HBX_ERR_PARSE, msg);
    }
    for (int32_t c = 0; c < n_cols; c++) {
      auto& b = cells_bytes[(size_t)c];
      b.insert(b.end(), scratch.begin() + row[(size_t)c].first,
               scratch.begin() + row[(size_t)c].first + row[(size_t)c].second);
      cells_off[(size_t)c].push_back((int64_t)b.size());
    }
    row.clear();
    scratch.clear();
    n_rows++;
  }
};

}  // namespace

Table table_from_buffer(const char* data, size_t n, char sep) {
  if (n >= 3 && (unsigned char)data[0] == 0xEF && (unsigned char)data[1] == 0xBB &&
      (unsigned char)data[2] == 0xBF) {
    data += 3;
    n -= 3;
  }
  RowBuilder rb;
  std::vector<char> cell;
  bool quoted = false;
  for (size_t i = 0; i < n; i++) {
    const char ch = data[i];
    if (ch == '"') {
      if (cell.empty() || cell[0] == '"') quoted = !quoted;
      cell.push_back(ch);
    } else if (ch == sep) {
      if (!quoted) {
        rb.push_cell(cell.data(), cell.size());
        cell.clear();
      } else {
        cell.push_back(ch);
      }
    } else if (ch == '\r') {
      // dropped
    } else if (ch == '\n') {
      rb.push_cell(cell.data(), cell.size());
      rb.end_row();
      cell.clear();
      quoted = false;
    } else {
      cell.push_back(ch);
    }
  }
  if (!cell.empty() || !rb.row.empty()) {
    rb.push_cell(cell.data(), cell.size());
    rb.end_row();
  }
  Table t;
  t.n_rows = rb.n_rows;
  for (int32_t c = 0; c < rb.n_cols; c++) {
    Column col;
    col.bytes = std::move(rb.cells_bytes[(size_t)c]);
    col.off = std::move(rb.cells_off[(size_t)c]);
    t.cols.push_back(std::move(col));
  }
  finish_table(&t);
  return t;
}

Table table_from_csv(const std::string& path, char sep, hbx_ctx* ctx) {
  std::vector<char> buf;
  {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) fail(HBX_ERR_IO, "cannot open " + path);
    // one read of the whole file (grown if the file grows meanwhile)
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(size > 0 ? (size_t)size : 0);
    size_t got = buf.empty() ? 0 : std::fread(buf.data(), 1, buf.size(), f);
    for (char tmp[65536];;) {
      const size_t k = std::fread(tmp, 1, sizeof tmp, f);
      if (k == 0) break;
      buf.insert(buf.begin() + (long)got, tmp, tmp + k);
      got += k;
    }
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) fail(HBX_ERR_IO, "cannot read " + path);
    buf.resize(got);
  }
  try {
    if (ctx && buf.size() >= kDeviceCsvMin) {
      Table t;
      if (table_from_buffer_device(ctx, buf.data(), buf.size(), sep, &t)) return t;
    }
    return table_from_buffer(buf.data(), buf.size(), sep);
  } catch (const Error& e) {
    fail(e.status, path + ": " + e.what());
  }
}

Table table_from_columns(const hbx_columns* cols) {
  if (!cols || cols->n_rows < 0 || cols->n_cols < 0) fail(HBX_ERR_INVALID_ARG, "bad hbx_columns");
  Table t;
  t.n_rows = cols->n_rows;
  for (int32_t c = 0; c < cols->n_cols; c++) {
    if (!cols->data || !cols->offsets || !cols->offsets[c])
      fail(HBX_ERR_INVALID_ARG, "hbx_columns has a null column");
    const int64_t* off = cols->offsets[c];
    Column col;
    const int64_t base = off[0];
    const int64_t total = off[cols->n_rows] - base;
    if (total < 0) fail(HBX_ERR_INVALID_ARG, "hbx_columns offsets decrease");
    if (total > 0 && !cols->data[c]) fail(HBX_ERR_INVALID_ARG, "hbx_columns has a null column");
    col.bytes.assign(cols->data[c] + base, cols->data[c] + base + total);
    col.off.resize((size_t)cols->n_rows + 1);
    for (int64_t i = 0; i <= cols->n_rows; i++) {
      col.off[(size_t)i] = off[i] - base;
      if (i > 0 && col.off[(size_t)i] < col.off[(size_t)i - 1])
        fail(HBX_ERR_INVALID_ARG, "hbx_columns offsets decrease");
    }
    t.cols.push_back(std::move(col));
  }
  finish_table(&t);
  return t;
}

void finish_table(Table* t) {
  for (Column& c : t->cols)
    c.has_nul = !c.bytes.empty() && std::memchr(c.bytes.data(), 0, c.bytes.size()) != nullptr;
}

uint64_t next_table_uid() {
  static std::atomic<uint64_t> next{1};
  return next.fetch_add(1);
}

}  // namespace hbx
