// lc2_yaml.hpp -- the YAML subset of LC2Registration's parameter files.
//
// The reference parses its configs with yaml-cpp (config/*.yaml read in
// src/Interpolator/interpolator.cu:234-391, 1538-1623 and
// src/Optimizers/optimizers.cu:22-110, 484-582) and writes *_result.yaml
// (optimizers.cu:450-480, 1040-1106). yaml-cpp is not available, so this is a
// small reader/writer of the constructs those files use: block maps and
// sequences by indentation, flow maps {a: 1, b: 2} and flow sequences [1, 2],
// "-" items with nested blocks, # comments, quoted strings and numeric keys.
// Key order is preserved so a file can be rewritten in its original layout.
#pragma once

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace lc2yaml {

struct Node {
  enum Kind { Null, Scalar, Map, Seq } kind = Null;
  std::string value;                                // Scalar
  std::vector<std::pair<std::string, Node>> items;  // Map (ordered)
  std::vector<Node> seq;                            // Seq

  static Node scalar(const std::string& v) {
    Node n;
    n.kind = Scalar;
    n.value = v;
    return n;
  }
  bool has(const std::string& k) const {
    if (kind != Map) return false;
    for (auto& kv : items)
      if (kv.first == k) return true;
    return false;
  }
  const Node& operator[](const std::string& k) const {
    static const Node null_node;
    if (kind == Map)
      for (auto& kv : items)
        if (kv.first == k) return kv.second;
    return null_node;
  }
  Node& at(const std::string& k) {  // insert when missing
    if (kind != Map) {
      kind = Map;
      items.clear();
    }
    for (auto& kv : items)
      if (kv.first == k) return kv.second;
    items.emplace_back(k, Node());
    return items.back().second;
  }
  const Node& operator[](size_t i) const { return seq.at(i); }
  size_t size() const { return kind == Map ? items.size() : kind == Seq ? seq.size() : 0; }
  explicit operator bool() const { return kind != Null; }

  std::string str() const {
    if (kind != Scalar) throw std::runtime_error("yaml: expected a scalar");
    return value;
  }
  double num() const {
    const std::string s = str();
    char* end = nullptr;
    double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str()) throw std::runtime_error("yaml: '" + s + "' is not a number");
    return v;
  }
  int integer() const { return (int)num(); }
  bool boolean() const {
    std::string s = str();
    for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
    if (s == "true" || s == "yes" || s == "on" || s == "1") return true;
    if (s == "false" || s == "no" || s == "off" || s == "0") return false;
    throw std::runtime_error("yaml: '" + value + "' is not a boolean");
  }
};

namespace detail {

inline std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

inline std::string strip_comment(const std::string& s) {
  char q = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (q) {
      if (c == q) q = 0;
    } else if (c == '"' || c == '\'') {
      q = c;
    } else if (c == '#' && (i == 0 || std::isspace((unsigned char)s[i - 1]))) {
      return s.substr(0, i);
    }
  }
  return s;
}

inline std::string unquote(const std::string& s) {
  if (s.size() >= 2 && (s.front() == '"' || s.front() == '\'') && s.back() == s.front()) {
    std::string out;
    for (size_t i = 1; i + 1 < s.size(); ++i) {
      if (s.front() == '"' && s[i] == '\\' && i + 2 < s.size()) {
        const char n = s[++i];
        out += (n == 'n') ? '\n' : (n == 't') ? '\t' : n;
      } else {
        out += s[i];
      }
    }
    return out;
  }
  return s;
}

// position of the "key: value" separator outside quotes and brackets
inline size_t key_colon(const std::string& s) {
  char q = 0;
  int depth = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (q) {
      if (c == q) q = 0;
      continue;
    }
    if (c == '"' || c == '\'') q = c;
    else if (c == '{' || c == '[') ++depth;
    else if (c == '}' || c == ']') --depth;
    else if (c == ':' && depth == 0 && (i + 1 == s.size() || s[i + 1] == ' ')) return i;
  }
  return std::string::npos;
}

inline Node parse_flow(const std::string& s, size_t& i);

inline void skip_ws(const std::string& s, size_t& i) {
  while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
}

inline std::string flow_token(const std::string& s, size_t& i) {
  skip_ws(s, i);
  if (i < s.size() && (s[i] == '"' || s[i] == '\'')) {
    const char q = s[i];
    size_t j = i + 1;
    while (j < s.size() && s[j] != q) ++j;
    std::string t = s.substr(i, j - i + 1);
    i = j + 1;
    return unquote(t);
  }
  size_t j = i;
  while (j < s.size() && s[j] != ',' && s[j] != '}' && s[j] != ']' &&
         !(s[j] == ':' && (j + 1 == s.size() || s[j + 1] == ' ')))
    ++j;
  std::string t = trim(s.substr(i, j - i));
  i = j;
  return t;
}

inline Node parse_flow(const std::string& s, size_t& i) {
  skip_ws(s, i);
  if (i < s.size() && s[i] == '{') {
    Node m;
    m.kind = Node::Map;
    ++i;
    for (;;) {
      skip_ws(s, i);
      if (i < s.size() && s[i] == '}') { ++i; break; }
      std::string k = flow_token(s, i);
      skip_ws(s, i);
      if (i >= s.size() || s[i] != ':') throw std::runtime_error("yaml: bad flow map");
      ++i;
      m.items.emplace_back(k, parse_flow(s, i));
      skip_ws(s, i);
      if (i < s.size() && s[i] == ',') ++i;
    }
    return m;
  }
  if (i < s.size() && s[i] == '[') {
    Node q;
    q.kind = Node::Seq;
    ++i;
    for (;;) {
      skip_ws(s, i);
      if (i < s.size() && s[i] == ']') { ++i; break; }
      q.seq.push_back(parse_flow(s, i));
      skip_ws(s, i);
      if (i < s.size() && s[i] == ',') ++i;
    }
    return q;
  }
  const std::string t = flow_token(s, i);
  return t.empty() ? Node() : Node::scalar(t);
}

inline Node parse_value(const std::string& v) {
  const std::string t = trim(v);
  if (t.empty() || t == "~" || t == "null") return Node();
  if (t[0] == '{' || t[0] == '[') {
    size_t i = 0;
    return parse_flow(t, i);
  }
  return Node::scalar(unquote(t));
}

struct Line {
  int indent;
  std::string text;
};

inline Node parse_block(const std::vector<Line>& L, size_t& i, int indent);

inline Node parse_seq(const std::vector<Line>& L, size_t& i, int indent) {
  Node q;
  q.kind = Node::Seq;
  while (i < L.size() && L[i].indent == indent && L[i].text[0] == '-') {
    const std::string rest = trim(L[i].text.substr(1));
    ++i;
    if (rest.empty()) {
      q.seq.push_back(i < L.size() && L[i].indent > indent ? parse_block(L, i, L[i].indent)
                                                           : Node());
    } else if (key_colon(rest) != std::string::npos && rest[0] != '{' && rest[0] != '[') {
      // "- key: value" starts an inline map
      std::vector<Line> sub{{indent + 2, rest}};
      while (i < L.size() && L[i].indent > indent) sub.push_back(L[i++]);
      size_t j = 0;
      q.seq.push_back(parse_block(sub, j, indent + 2));
    } else {
      q.seq.push_back(parse_value(rest));
    }
  }
  return q;
}

inline Node parse_block(const std::vector<Line>& L, size_t& i, int indent) {
  if (i < L.size() && L[i].text[0] == '-') return parse_seq(L, i, indent);
  Node m;
  m.kind = Node::Map;
  while (i < L.size() && L[i].indent == indent) {
    const std::string& t = L[i].text;
    const size_t c = key_colon(t);
    if (c == std::string::npos) throw std::runtime_error("yaml: expected 'key: value': " + t);
    const std::string key = unquote(trim(t.substr(0, c)));
    const std::string val = trim(t.substr(c + 1));
    ++i;
    if (!val.empty()) {
      m.items.emplace_back(key, parse_value(val));
    } else if (i < L.size() && (L[i].indent > indent ||
                                (L[i].indent == indent && L[i].text[0] == '-'))) {
      m.items.emplace_back(key, parse_block(L, i, L[i].indent));
    } else {
      m.items.emplace_back(key, Node());
    }
  }
  return m;
}

}  // namespace detail

inline Node parse(const std::string& text) {
  std::vector<detail::Line> L;
  std::istringstream in(text);
  std::string raw;
  while (std::getline(in, raw)) {
    if (!raw.empty() && raw.back() == '\r') raw.pop_back();
    std::string s = detail::strip_comment(raw);
    if (detail::trim(s).empty() || detail::trim(s) == "---") continue;
    int ind = 0;
    while (ind < (int)s.size() && s[ind] == ' ') ++ind;
    L.push_back({ind, detail::trim(s)});
  }
  size_t i = 0;
  if (L.empty()) return Node();
  return detail::parse_block(L, i, L[0].indent);
}

inline Node load_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("yaml: cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return parse(ss.str());
}

// ---------------------------------------------------------------- writing
namespace detail {
inline bool needs_quotes(const std::string& s) {
  if (s.empty()) return true;
  for (char c : s)
    if (c == ':' || c == '#' || c == '\n' || c == '{' || c == '}' || c == '[' || c == ']' ||
        c == ',' || c == '"')
      return true;
  return std::isspace((unsigned char)s.front()) || std::isspace((unsigned char)s.back());
}
inline std::string quoted(const std::string& s) {
  if (!needs_quotes(s)) return s;
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    if (c == '\n') { o += "\\n"; continue; }
    o += c;
  }
  return o + "\"";
}
inline bool flat_map(const Node& n) {
  if (n.kind != Node::Map || n.items.empty()) return false;
  for (auto& kv : n.items)
    if (kv.second.kind != Node::Scalar) return false;
  return true;
}
inline void emit(const Node& n, int indent, std::ostream& o) {
  const std::string pad(indent, ' ');
  if (n.kind == Node::Map) {
    for (auto& kv : n.items) {
      o << pad << quoted(kv.first) << ":";
      const Node& v = kv.second;
      if (v.kind == Node::Scalar) {
        o << " " << quoted(v.value) << "\n";
      } else if (v.kind == Node::Null) {
        o << "\n";
      } else if (flat_map(v)) {
        o << " {";
        for (size_t i = 0; i < v.items.size(); ++i)
          o << (i ? ", " : "") << quoted(v.items[i].first) << ": " << quoted(v.items[i].second.value);
        o << "}\n";
      } else {
        o << "\n";
        emit(v, indent + 2, o);
      }
    }
  } else if (n.kind == Node::Seq) {
    for (auto& e : n.seq) {
      if (e.kind == Node::Scalar) {
        o << pad << "- " << quoted(e.value) << "\n";
      } else {
        o << pad << "-\n";
        emit(e, indent + 2, o);
      }
    }
  }
}
}  // namespace detail

inline std::string dump(const Node& n) {
  std::ostringstream o;
  detail::emit(n, 0, o);
  return o.str();
}

inline void save_file(const Node& n, const std::string& path) {
  std::ofstream f(path);
  if (!f) throw std::runtime_error("yaml: cannot write " + path);
  f << dump(n);
}

}  // namespace lc2yaml
