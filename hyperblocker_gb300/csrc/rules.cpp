// rules.cpp -- YAML rule files -> the reference's serialized plan + the
// engine's compiled rules.
//
// Decoding follows YAML::convert<Rule>::decode (core/common/yaml_config.h:37-75):
//   * the document must have at least two top-level keys;
//   * Relations[0] and Relations[1] are read first;
//   * only when Preconditions has exactly four keys are Equalities[0], Sim[0],
//     Threshold[0] and Conseq.Equality decoded (std::stoi / std::stof);
//   * threshold list position 2+k is keyed by sim[2+2k], the LEFT column of
//     similarity predicate k; the first insertion of a key wins.
// Ordering and serialization follow execution_plan_generator.h:64-155:
// directory order, std::sort by equality-vector size (descending, the same
// comparator, so the same permutation), then per rule the equality slots,
// the similarity slots and one checkpoint slot.
//
// yaml-cpp is not vendored by the reference; this file parses the subset of
// YAML the rule format uses: block mappings, block sequences whose items are
// flow sequences or scalars, flow sequences, plain and quoted scalars and
// comments.
#include <algorithm>
#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>

#include "hbx_core.h"

namespace hbx {

namespace {

struct YNode {
  enum Kind { kNull, kScalar, kSeq, kMap } kind = kNull;
  std::string scalar;
  std::vector<std::shared_ptr<YNode>> seq;
  std::vector<std::pair<std::string, std::shared_ptr<YNode>>> map;  // document order

  const YNode* get(const std::string& k) const {
    if (kind != kMap) return nullptr;
    for (auto& kv : map)
      if (kv.first == k) return kv.second.get();
    return nullptr;
  }
  size_t size() const {
    if (kind == kMap) return map.size();
    if (kind == kSeq) return seq.size();
    return 0;
  }
};

using YPtr = std::shared_ptr<YNode>;

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t");
  return s.substr(a, b - a + 1);
}

std::string strip_comment(const std::string& line) {
  char q = 0;
  for (size_t i = 0; i < line.size(); i++) {
    char ch = line[i];
    if (q) {
      if (ch == q) q = 0;
    } else if (ch == '"' || ch == '\'') {
      q = ch;
    } else if (ch == '#' && (i == 0 || line[i - 1] == ' ' || line[i - 1] == '\t')) {
      return line.substr(0, i);
    }
  }
  return line;
}

std::string unquote_scalar(std::string s) {
  s = trim(s);
  if (s.size() >= 2 && s.front() == s.back() && (s.front() == '"' || s.front() == '\''))
    return s.substr(1, s.size() - 2);
  return s;
}

YPtr scalar_node(const std::string& s) {
  auto n = std::make_shared<YNode>();
  n->kind = YNode::kScalar;
  n->scalar = unquote_scalar(s);
  return n;
}

YPtr flow_or_scalar(const std::string& text) {
  std::string t = trim(text);
  if (!t.empty() && t.front() == '[') {
    if (t.back() != ']') fail(HBX_ERR_PARSE, "unterminated flow sequence: " + t);
    auto n = std::make_shared<YNode>();
    n->kind = YNode::kSeq;
    std::string inner = trim(t.substr(1, t.size() - 2));
    if (!inner.empty()) {
      std::stringstream ss(inner);
      std::string item;
      while (std::getline(ss, item, ',')) n->seq.push_back(scalar_node(item));
    }
    return n;
  }
  return scalar_node(t);
}

bool is_key_line(const std::string& t, std::string* key, std::string* rest) {
  // key: [value]   -- the key has no ':' '[' ']' '{' '}'
  size_t c = std::string::npos;
  for (size_t i = 0; i < t.size(); i++) {
    char ch = t[i];
    if (ch == '[' || ch == ']' || ch == '{' || ch == '}') return false;
    if (ch == ':' && (i + 1 == t.size() || t[i + 1] == ' ' || t[i + 1] == '\t')) {
      c = i;
      break;
    }
  }
  if (c == std::string::npos || c == 0) return false;
  *key = unquote_scalar(t.substr(0, c));
  *rest = trim(t.substr(c + 1));
  return true;
}

struct Line {
  int indent;
  std::string text;
};

struct Parser {
  std::vector<Line> lines;
  size_t pos = 0;

  static bool is_seq_item(const std::string& t) { return t == "-" || t.rfind("- ", 0) == 0; }

  YPtr block(int indent) {
    const std::string& text = lines[pos].text;
    std::string key, rest;
    if (!is_seq_item(text) && !is_key_line(text, &key, &rest)) {
      pos++;
      return flow_or_scalar(text);
    }
    if (is_seq_item(text)) {
      auto n = std::make_shared<YNode>();
      n->kind = YNode::kSeq;
      while (pos < lines.size() && lines[pos].indent == indent && is_seq_item(lines[pos].text)) {
        std::string item = trim(lines[pos].text.substr(1));
        pos++;
        if (!item.empty()) {
          n->seq.push_back(flow_or_scalar(item));
        } else if (pos < lines.size() && lines[pos].indent > indent) {
          n->seq.push_back(block(lines[pos].indent));
        } else {
          n->seq.push_back(std::make_shared<YNode>());
        }
      }
      return n;
    }
    auto n = std::make_shared<YNode>();
    n->kind = YNode::kMap;
    while (pos < lines.size() && lines[pos].indent == indent) {
      if (!is_key_line(lines[pos].text, &key, &rest))
        fail(HBX_ERR_PARSE, "cannot parse YAML line: " + lines[pos].text);
      pos++;
      YPtr v;
      if (!rest.empty()) {
        v = flow_or_scalar(rest);
      } else if (pos < lines.size() && lines[pos].indent > indent) {
        v = block(lines[pos].indent);
      } else if (pos < lines.size() && lines[pos].indent == indent &&
                 is_seq_item(lines[pos].text)) {
        v = block(indent);
      } else {
        v = std::make_shared<YNode>();
      }
      bool dup = false;
      for (auto& kv : n->map)
        if (kv.first == key) dup = true;
      if (dup) fail(HBX_ERR_PARSE, "duplicate YAML key: " + key);
      n->map.emplace_back(key, v);
    }
    return n;
  }
};

YPtr parse_yaml(const std::string& src) {
  Parser p;
  std::stringstream ss(src);
  std::string raw;
  while (std::getline(ss, raw)) {
    if (!raw.empty() && raw.back() == '\r') raw.pop_back();
    for (auto& ch : raw)
      if (ch == '\t') ch = ' ';
    std::string s = strip_comment(raw);
    std::string t = trim(s);
    if (t.empty() || t == "---" || t == "...") continue;
    int ind = (int)(s.find_first_not_of(' '));
    p.lines.push_back({ind, t});
  }
  if (p.lines.empty()) return std::make_shared<YNode>();
  YPtr root = p.block(p.lines[0].indent);
  if (p.pos != p.lines.size()) fail(HBX_ERR_PARSE, "unparsed YAML at: " + p.lines[p.pos].text);
  return root;
}

// std::stoi: leading whitespace, optional sign, digits; trailing text ignored.
int yaml_stoi(const std::string& s) {
  const char* b = s.c_str();
  char* e = nullptr;
  errno = 0;
  long v = std::strtol(b, &e, 10);
  if (e == b) fail(HBX_ERR_PARSE, "stoi: invalid argument '" + s + "'");
  if (errno == ERANGE || v > 2147483647L || v < -2147483647L - 1)
    fail(HBX_ERR_PARSE, "stoi: out of range '" + s + "'");
  return (int)v;
}

float yaml_stof(const std::string& s) {
  const char* b = s.c_str();
  char* e = nullptr;
  errno = 0;
  float v = std::strtof(b, &e);
  if (e == b) fail(HBX_ERR_PARSE, "stof: invalid argument '" + s + "'");
  if (errno == ERANGE) fail(HBX_ERR_PARSE, "stof: out of range '" + s + "'");
  return v;
}

std::vector<std::string> as_strings(const YNode* n, const char* what) {
  if (!n) fail(HBX_ERR_PARSE, std::string("missing ") + what);
  std::vector<std::string> out;
  if (n->kind == YNode::kScalar) {
    out.push_back(n->scalar);
    return out;
  }
  if (n->kind != YNode::kSeq) fail(HBX_ERR_PARSE, std::string(what) + " is not a sequence");
  for (auto& x : n->seq) {
    if (x->kind != YNode::kScalar) fail(HBX_ERR_PARSE, std::string(what) + " holds a non-scalar");
    out.push_back(x->scalar);
  }
  return out;
}

const YNode* seq_at(const YNode* n, size_t i, const char* what) {
  if (!n || n->kind != YNode::kSeq || i >= n->seq.size())
    fail(HBX_ERR_PARSE, std::string("missing ") + what);
  return n->seq[i].get();
}

RuleDef decode_rule(const YNode& root, const std::string& source) {
  if (root.size() < 2) fail(HBX_ERR_PARSE, source + ": Invalid rule's metadata format");
  const YNode* pre = root.get("Preconditions");
  if (!pre || pre->kind != YNode::kMap) fail(HBX_ERR_PARSE, source + ": missing Preconditions");
  const YNode* rel = pre->get("Relations");
  auto relation_l = as_strings(seq_at(rel, 0, "Relations[0]"), "Relations[0]");
  auto relation_r = as_strings(seq_at(rel, 1, "Relations[1]"), "Relations[1]");
  RuleDef r;
  r.source = source;
  if (pre->size() == 4) {
    for (auto& x : relation_l) r.relation_l.push_back(yaml_stoi(x));
    for (auto& x : relation_r) r.relation_r.push_back(yaml_stoi(x));
    for (auto& x : as_strings(seq_at(pre->get("Equalities"), 0, "Equalities[0]"), "Equalities"))
      r.eq.push_back(yaml_stoi(x));
    for (auto& x : as_strings(seq_at(pre->get("Sim"), 0, "Sim[0]"), "Sim"))
      r.sim.push_back(yaml_stoi(x));
    auto thr = as_strings(seq_at(pre->get("Threshold"), 0, "Threshold[0]"), "Threshold");
    for (size_t i = 2; i < thr.size(); i++) {
      size_t k = 2 + (i - 2) * 2;
      if (k >= r.sim.size()) fail(HBX_ERR_PARSE, source + ": threshold without a Sim predicate");
      if (!r.find_threshold(r.sim[k])) r.threshold.emplace_back(r.sim[k], yaml_stof(thr[i]));
    }
    const YNode* con = root.get("Conseq");
    if (con && con->get("Equality"))
      for (auto& x : as_strings(con->get("Equality"), "Conseq.Equality"))
        r.con_eq.push_back(yaml_stoi(x));
  }
  return r;
}

// Rules on which the reference has undefined behaviour are refused:
// undecoded rules (eq.begin()+2 past end), odd column lists, rules without a
// predicate (the plan [CP] makes blocking_kernel read past the plan), and
// similarity predicates without a threshold (find()->second on end()).
void validate_rule(const RuleDef& r) {
  if (r.eq.size() < 2 || r.sim.size() < 2)
    fail(HBX_ERR_UNSUPPORTED, r.source + ": rule not decoded (Preconditions must have 4 keys)");
  if ((r.eq.size() - 2) % 2 || (r.sim.size() - 2) % 2)
    fail(HBX_ERR_UNSUPPORTED, r.source + ": predicate lists must hold column pairs");
  if (r.eq.size() == 2 && r.sim.size() == 2)
    fail(HBX_ERR_UNSUPPORTED, r.source + ": rule has no predicate");
  if ((r.eq.size() - 2) / 2 > (size_t)kMaxEqPerRule || (r.sim.size() - 2) / 2 > (size_t)kMaxSimPerRule)
    fail(HBX_ERR_UNSUPPORTED, r.source + ": too many predicates in one rule");
  for (size_t k = 2; k < r.eq.size(); k++)
    if (r.eq[k] < 0) fail(HBX_ERR_UNSUPPORTED, r.source + ": negative column index");
  for (size_t k = 2; k < r.sim.size(); k++) {
    if (r.sim[k] < 0) fail(HBX_ERR_UNSUPPORTED, r.source + ": negative column index");
    if (k % 2 == 0 && !r.find_threshold(r.sim[k]))
      fail(HBX_ERR_UNSUPPORTED, r.source + ": similarity predicate without a threshold");
  }
}

Plan build_plan(std::vector<RuleDef> rules) {
  if (rules.empty()) fail(HBX_ERR_PARSE, "no rule files");
  if (rules.size() > (size_t)kMaxRules) fail(HBX_ERR_UNSUPPORTED, "too many rules");
  for (auto& r : rules) validate_rule(r);
  // execution_plan_generator.h:75-79 -- the same std::sort and comparator.
  std::sort(rules.begin(), rules.end(), [](const RuleDef& a, const RuleDef& b) {
    return a.eq.size() > b.eq.size();
  });
  Plan p;
  for (auto& r : rules) {
    CompiledRule cr;
    for (size_t k = 2; k < r.eq.size(); k++) {
      p.pred_index.push_back(r.eq[k]);
      p.pred_type.push_back('e');
      p.pred_threshold.push_back(1.0f);
    }
    for (size_t k = 2; k + 1 < r.eq.size(); k += 2) cr.eqs.push_back({'e', r.eq[k], r.eq[k + 1], 1.0f});
    for (size_t k = 2; k < r.sim.size(); k++) {
      p.pred_index.push_back(r.sim[k]);
      p.pred_type.push_back('s');
      const float* t = r.find_threshold(r.sim[k]);
      p.pred_threshold.push_back(t ? *t : 1.0f);  // right slots: never read
    }
    for (size_t k = 2; k + 1 < r.sim.size(); k += 2)
      cr.sims.push_back({'s', r.sim[k], r.sim[k + 1], *r.find_threshold(r.sim[k])});
    p.pred_index.push_back(kCheckPoint);
    p.pred_type.push_back(' ');
    p.pred_threshold.push_back(1.0f);
    p.compiled.push_back(std::move(cr));
  }
  p.rules = std::move(rules);
  return p;
}

}  // namespace

Plan plan_from_docs(const std::vector<std::pair<std::string, std::string>>& named_docs) {
  std::vector<RuleDef> rules;
  for (auto& nd : named_docs) {
    YPtr root = parse_yaml(nd.second);
    rules.push_back(decode_rule(*root, nd.first));
  }
  return build_plan(std::move(rules));
}

Plan plan_from_dir(const std::string& dir) {
  namespace fs = std::filesystem;
  std::error_code ec;
  fs::directory_iterator it(dir, ec);
  if (ec) fail(HBX_ERR_IO, "cannot read rule directory " + dir + ": " + ec.message());
  std::vector<std::pair<std::string, std::string>> docs;
  for (; it != fs::directory_iterator(); it.increment(ec)) {
    if (ec) fail(HBX_ERR_IO, "cannot read rule directory " + dir + ": " + ec.message());
    const std::string path = it->path().string();
    std::ifstream f(path, std::ios::binary);
    if (!f) fail(HBX_ERR_IO, "cannot read rule file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    docs.emplace_back(path, ss.str());
  }
  return plan_from_docs(docs);
}

}  // namespace hbx
