// JSON values written the way the reference's serde_json output is written:
// numbers in the shortest form that reads back to the same f64/f32, decimal
// notation inside the exponent ranges serde_json uses (f64: 1e-5 <= |v| < 1e16
// and integral values below 1e16 with a ".0"; f32: 1e-6 <= |v| < 1e13), and
// "1.5e20"-style exponents outside them; non-finite numbers become null;
// pretty printing with two-space indentation, "key": value, and [] / {} for
// empty containers (serde_json::to_string_pretty).
#pragma once
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace psrjson {

namespace detail {
// Shortest round-trip digits and decimal exponent: v = 0.d1d2...dn * 10^kk.
template <typename T>
inline std::string pretty(T v, int max_kk, int min_kk_exclusive) {
  if (!std::isfinite(v)) return "null";
  std::string sign = std::signbit(v) ? "-" : "";
  if (v == 0) return sign + "0.0";
  char buf[64];
  auto r = std::to_chars(buf, buf + sizeof buf, std::fabs(v), std::chars_format::scientific);
  std::string s(buf, r.ptr);
  const size_t e = s.find('e');
  std::string mant = s.substr(0, e);
  const int exp10 = std::atoi(s.c_str() + e + 1);
  std::string digits;
  for (char c : mant)
    if (c != '.') digits += c;
  const int length = (int)digits.size();
  const int kk = exp10 + 1;  // 10^(kk-1) <= v < 10^kk
  const int k = kk - length;
  std::string out;
  if (k >= 0 && kk <= max_kk) {
    out = digits + std::string((size_t)k, '0') + ".0";
  } else if (kk > 0 && kk <= max_kk) {
    out = digits.substr(0, (size_t)kk) + "." + digits.substr((size_t)kk);
  } else if (kk > min_kk_exclusive && kk <= 0) {
    out = "0." + std::string((size_t)(-kk), '0') + digits;
  } else if (length == 1) {
    out = digits + "e" + std::to_string(kk - 1);
  } else {
    out = digits.substr(0, 1) + "." + digits.substr(1) + "e" + std::to_string(kk - 1);
  }
  return sign + out;
}
}  // namespace detail

inline std::string f64(double v) { return detail::pretty<double>(v, 16, -5); }
inline std::string f32(float v) { return detail::pretty<float>(v, 13, -6); }

inline std::string quote(const std::string &s) {
  std::string o = "\"";
  for (unsigned char c : s) {
    switch (c) {
      case '"': o += "\\\""; break;
      case '\\': o += "\\\\"; break;
      case '\n': o += "\\n"; break;
      case '\r': o += "\\r"; break;
      case '\t': o += "\\t"; break;
      default:
        if (c < 0x20) {
          char b[8];
          std::snprintf(b, sizeof b, "\\u%04x", c);
          o += b;
        } else {
          o += (char)c;
        }
    }
  }
  return o + "\"";
}

// A JSON value: scalars keep their serialised text.
struct Value {
  enum Kind { SCALAR, ARRAY, OBJECT } kind = SCALAR;
  std::string text = "null";
  std::vector<Value> items;
  std::vector<std::pair<std::string, Value>> fields;

  static Value null() { return Value(); }
  static Value raw(std::string t) {
    Value v;
    v.text = std::move(t);
    return v;
  }
  static Value num(double x) { return raw(f64(x)); }
  static Value num32(float x) { return raw(f32(x)); }
  static Value u64(uint64_t x) { return raw(std::to_string(x)); }
  static Value i64(int64_t x) { return raw(std::to_string(x)); }
  static Value boolean(bool b) { return raw(b ? "true" : "false"); }
  static Value str(const std::string &s) { return raw(quote(s)); }
  static Value array() {
    Value v;
    v.kind = ARRAY;
    return v;
  }
  static Value object() {
    Value v;
    v.kind = OBJECT;
    return v;
  }
  Value &push(Value v) {
    items.push_back(std::move(v));
    return *this;
  }
  Value &set(const std::string &k, Value v) {
    fields.emplace_back(k, std::move(v));
    return *this;
  }
};

inline void dump_to(const Value &v, std::string &o, bool pretty, int depth) {
  const std::string ind = pretty ? std::string((size_t)(2 * (depth + 1)), ' ') : "";
  const std::string ind0 = pretty ? std::string((size_t)(2 * depth), ' ') : "";
  const char *nl = pretty ? "\n" : "";
  switch (v.kind) {
    case Value::SCALAR:
      o += v.text;
      break;
    case Value::ARRAY:
      if (v.items.empty()) {
        o += "[]";
        break;
      }
      o += "[";
      o += nl;
      for (size_t i = 0; i < v.items.size(); ++i) {
        o += ind;
        dump_to(v.items[i], o, pretty, depth + 1);
        if (i + 1 < v.items.size()) o += ",";
        o += nl;
      }
      o += ind0;
      o += "]";
      break;
    case Value::OBJECT:
      if (v.fields.empty()) {
        o += "{}";
        break;
      }
      o += "{";
      o += nl;
      for (size_t i = 0; i < v.fields.size(); ++i) {
        o += ind;
        o += quote(v.fields[i].first);
        o += pretty ? ": " : ":";
        dump_to(v.fields[i].second, o, pretty, depth + 1);
        if (i + 1 < v.fields.size()) o += ",";
        o += nl;
      }
      o += ind0;
      o += "}";
      break;
  }
}

inline std::string dump(const Value &v, bool pretty) {
  std::string o;
  dump_to(v, o, pretty, 0);
  return o;
}

// Reads JSON text written by dump(): scalars keep their text, so a document
// read and dumped again is unchanged.  Returns false on malformed input.
struct Reader {
  const std::string &s;
  size_t i = 0;
  explicit Reader(const std::string &text) : s(text) {}
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) ++i;
  }
  bool str(std::string &out) {
    if (i >= s.size() || s[i] != '"') return false;
    const size_t a = i++;
    while (i < s.size() && s[i] != '"') i += s[i] == '\\' ? 2 : 1;
    if (i >= s.size()) return false;
    out = s.substr(a, ++i - a);
    return true;
  }
  bool value(Value &v) {
    ws();
    if (i >= s.size()) return false;
    const char c = s[i];
    if (c == '{') {
      v = Value::object();
      ++i;
      ws();
      if (i < s.size() && s[i] == '}') return ++i, true;
      for (;;) {
        ws();
        std::string k;
        if (!str(k)) return false;
        ws();
        if (i >= s.size() || s[i++] != ':') return false;
        Value x;
        if (!value(x)) return false;
        v.set(k.substr(1, k.size() - 2), std::move(x));
        ws();
        if (i < s.size() && s[i] == ',') {
          ++i;
          continue;
        }
        if (i < s.size() && s[i] == '}') return ++i, true;
        return false;
      }
    }
    if (c == '[') {
      v = Value::array();
      ++i;
      ws();
      if (i < s.size() && s[i] == ']') return ++i, true;
      for (;;) {
        Value x;
        if (!value(x)) return false;
        v.push(std::move(x));
        ws();
        if (i < s.size() && s[i] == ',') {
          ++i;
          continue;
        }
        if (i < s.size() && s[i] == ']') return ++i, true;
        return false;
      }
    }
    if (c == '"') {
      std::string t;
      if (!str(t)) return false;
      v = Value::raw(t);
      return true;
    }
    const size_t a = i;
    while (i < s.size() && s[i] != ',' && s[i] != ']' && s[i] != '}' && s[i] != ' ' &&
           s[i] != '\n')
      ++i;
    if (i == a) return false;
    v = Value::raw(s.substr(a, i - a));
    return true;
  }
};

inline bool parse(const std::string &text, Value &out) {
  Reader r(text);
  if (!r.value(out)) return false;
  r.ws();
  return r.i == text.size();
}

// Field lookup in an object value (nullptr when absent).
inline const Value *field(const Value &v, const std::string &k) {
  for (const auto &f : v.fields)
    if (f.first == k) return &f.second;
  return nullptr;
}

}  // namespace psrjson
