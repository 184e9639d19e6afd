// cli.cpp -- the run_hyperblocker_exec command line (examples/run_hyperblocker.cu:22-59).
//
// Flags keep the reference's names and defaults (gflags syntax: -flag=value,
// --flag=value, -flag value; booleans also -flag / -noflag):
//   -data_l -data_r -rule_dir -o      (strings, default "")
//   -sep ","  -scheduler "CHBL"        (the scheduler picks among GPUs; one
//                                       GPU here, so it is accepted and unused)
//   -read_header false                 (parsed and unused, as in the reference)
//   -n_partitions 1  -prefix_hash_pred_idx INT_MAX
// Engine flags: -hbx_mode=batched|plain, -hbx_device=N.
// Unknown flags are an error, as gflags makes them.  Output lines are
// appended to -o like host_reducer.h:74, sorted by (left row, right row).
#include <algorithm>
#include <cerrno>
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/hbx.h"

// engine.cu: hbx_block, the sort and hbx_write_pairs with the pairs on the device
extern "C" hbx_status hbx_internal_block_to_file(hbx_ctx* ctx, const hbx_plan* plan,
                                                 const hbx_table* left, const hbx_table* right,
                                                 uint64_t n_partitions, int64_t prefix_idx,
                                                 hbx_mode mode, const char* path, hbx_stats* stats);

namespace {

struct Flags {
  std::string data_l, data_r, rule_dir, o, sep = ",", scheduler = "CHBL", hbx_mode = "batched";
  bool read_header = false;
  unsigned long long n_partitions = 1;
  unsigned long long prefix_hash_pred_idx = INT_MAX;
  int hbx_device = 0;
};

bool parse_bool(const std::string& v, bool* out) {
  if (v == "true" || v == "1" || v == "t" || v == "yes" || v == "y") return *out = true, true;
  if (v == "false" || v == "0" || v == "f" || v == "no" || v == "n") return *out = false, true;
  return false;
}

bool parse_u64(const std::string& v, unsigned long long* out) {
  if (v.empty()) return false;
  char* e = nullptr;
  errno = 0;
  unsigned long long x = std::strtoull(v.c_str(), &e, 0);
  if (*e || errno) return false;
  *out = x;
  return true;
}

int parse_flags(int argc, const char* const* argv, Flags* F) {
  std::map<std::string, std::string*> strs = {
      {"data_l", &F->data_l},       {"data_r", &F->data_r}, {"rule_dir", &F->rule_dir},
      {"o", &F->o},                 {"sep", &F->sep},       {"scheduler", &F->scheduler},
      {"hbx_mode", &F->hbx_mode}};
  std::map<std::string, unsigned long long*> nums = {
      {"n_partitions", &F->n_partitions}, {"prefix_hash_pred_idx", &F->prefix_hash_pred_idx}};
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    if (a.size() < 2 || a[0] != '-') {
      std::fprintf(stderr, "ERROR: unexpected argument '%s'\n", a.c_str());
      return 1;
    }
    a = a.substr(a[1] == '-' ? 2 : 1);
    std::string name = a, val;
    bool has_val = false;
    size_t eq = a.find('=');
    if (eq != std::string::npos) {
      name = a.substr(0, eq);
      val = a.substr(eq + 1);
      has_val = true;
    }
    auto next_val = [&]() -> bool {
      if (has_val) return true;
      if (i + 1 >= argc) return false;
      val = argv[++i];
      return true;
    };
    if (strs.count(name)) {
      if (!next_val()) return std::fprintf(stderr, "ERROR: flag '-%s' is missing its argument\n", name.c_str()), 1;
      *strs[name] = val;
    } else if (nums.count(name)) {
      if (!next_val() || !parse_u64(val, nums[name]))
        return std::fprintf(stderr, "ERROR: illegal value for flag '-%s'\n", name.c_str()), 1;
    } else if (name == "hbx_device") {
      unsigned long long d = 0;
      if (!next_val() || !parse_u64(val, &d)) return std::fprintf(stderr, "ERROR: illegal -hbx_device\n"), 1;
      F->hbx_device = (int)d;
    } else if (name == "read_header" || name == "noread_header") {
      bool b = name == "read_header";
      if (has_val && !parse_bool(val, &b))
        return std::fprintf(stderr, "ERROR: illegal value for flag '-read_header'\n"), 1;
      F->read_header = name == "noread_header" ? false : b;
    } else {
      std::fprintf(stderr, "ERROR: unknown command line flag '%s'\n", name.c_str());
      return 1;
    }
  }
  return 0;
}

double secs(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

}  // namespace

extern "C" int hbx_run_cli(int argc, const char* const* argv) {
  Flags F;
  if (parse_flags(argc, argv, &F)) return 1;
  hbx_mode mode;
  if (F.hbx_mode == "batched") {
    mode = HBX_MODE_BATCHED;
  } else if (F.hbx_mode == "plain") {
    mode = HBX_MODE_PLAIN;
  } else {
    std::fprintf(stderr, "ERROR: -hbx_mode must be batched or plain\n");
    return 1;
  }
  if (F.prefix_hash_pred_idx > (unsigned long long)INT_MAX) {
    std::fprintf(stderr, "ERROR: -prefix_hash_pred_idx out of range\n");
    return 1;
  }
  const auto t0 = std::chrono::steady_clock::now();
  hbx_ctx* ctx = nullptr;
  hbx_plan* plan = nullptr;
  hbx_table *L = nullptr, *R = nullptr;
  int rc = 0;
  auto die = [&](const char* what, hbx_status s) {
    std::fprintf(stderr, "ERROR: %s: %s (%s)\n", what, hbx_status_string(s), hbx_last_error(ctx));
    rc = 2;
  };
  hbx_status s = hbx_ctx_create(F.hbx_device, nullptr, &ctx);
  if (s != HBX_OK) {
    die("CUDA context", s);
    return rc;
  }
  std::vector<uint32_t> ol, orr;
  hbx_stats st{};
  do {
    if ((s = hbx_plan_from_rule_dir(ctx, F.rule_dir.c_str(), &plan)) != HBX_OK) {
      die("rules", s);
      break;
    }
    const char sep = F.sep.empty() ? ',' : F.sep[0];
    if ((s = hbx_table_from_csv(ctx, F.data_l.c_str(), sep, &L)) != HBX_OK) {
      die("data_l", s);
      break;
    }
    if ((s = hbx_table_from_csv(ctx, F.data_r.c_str(), sep, &R)) != HBX_OK) {
      die("data_r", s);
      break;
    }
    const auto t1 = std::chrono::steady_clock::now();
    std::printf("HyperBlocker.Initialize() elapsed: %f\n", secs(t0, t1));
    if (!F.o.empty()) {
      // the pairs stay on the device: run, sort by (left row, right row),
      // format the id lines and append them to -o
      s = hbx_internal_block_to_file(ctx, plan, L, R, F.n_partitions,
                                     (int64_t)F.prefix_hash_pred_idx, mode, F.o.c_str(), &st);
      if (s != HBX_OK) {
        die("blocking", s);
        break;
      }
    } else {
      hbx_pairs out{};
      ol.resize(1 << 16);
      orr.resize(1 << 16);
      for (;;) {
        out.l_row = ol.data();
        out.r_row = orr.data();
        out.capacity = ol.size();
        s = hbx_block(ctx, plan, L, R, F.n_partitions, (int64_t)F.prefix_hash_pred_idx, mode, &out,
                      &st, nullptr);
        if (s == HBX_ERR_CAPACITY) {
          ol.resize(out.n_required);
          orr.resize(out.n_required);
          continue;
        }
        break;
      }
      if (s != HBX_OK) {
        die("blocking", s);
        break;
      }
      std::fprintf(stderr, "WARNING: no -o given, pairs not written\n");
    }
    std::printf("Actual number of partitions: %u\n", st.n_partitions_used);
    std::printf("pairs covered: %llu, pair comparisons: %llu, matches: %llu, device ms: %.3f\n",
                (unsigned long long)st.pairs_covered, (unsigned long long)st.pair_comparisons,
                (unsigned long long)st.n_matches, st.ms_last_run);
    std::printf("HyperBlocker.Run() elapsed: %f\n", secs(t1, std::chrono::steady_clock::now()));
  } while (false);
  if (L) hbx_table_destroy(L);
  if (R) hbx_table_destroy(R);
  if (plan) hbx_plan_destroy(plan);
  hbx_ctx_destroy(ctx);
  return rc;
}
