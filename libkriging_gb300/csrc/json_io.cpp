// json_io.cpp -- JSON parser / writer and the base64 matrix payloads of libKriging's model files (json_io.hpp).
#include "json_io.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

namespace lkg {
namespace json {

const Value& Value::at(const std::string& key) const {
  if (kind != Kind::Object) throw std::runtime_error("JSON: '" + key + "' looked up in a value that is not an object");
  auto it = o.find(key);
  if (it == o.end()) throw std::runtime_error("JSON: missing key '" + key + "'");
  return it->second;
}

double Value::as_double() const {
  if (kind == Kind::Double) return d;
  if (kind == Kind::Int) return (double)i;
  if (kind == Kind::Null) return std::nan("");  // nlohmann writes non-finite doubles as null
  throw std::runtime_error("JSON: number expected");
}

long long Value::as_int() const {
  if (kind == Kind::Int) return i;
  if (kind == Kind::Double && d == std::floor(d) && std::fabs(d) < 9.0e18) return (long long)d;
  throw std::runtime_error("JSON: integer expected");
}

bool Value::as_bool() const {
  if (kind != Kind::Bool) throw std::runtime_error("JSON: boolean expected");
  return b;
}

const std::string& Value::as_string() const {
  if (kind != Kind::String) throw std::runtime_error("JSON: string expected");
  return s;
}

// ---------------------------------------------------------------------------------------------------------------
namespace {

struct Parser {
  const std::string& t;
  size_t p = 0;
  explicit Parser(const std::string& text) : t(text) {}

  [[noreturn]] void fail(const char* what) const {
    throw std::runtime_error(std::string("JSON parse error at offset ") + std::to_string(p) + ": " + what);
  }
  void ws() {
    while (p < t.size() && (t[p] == ' ' || t[p] == '\n' || t[p] == '\r' || t[p] == '\t')) ++p;
  }
  bool eat(char c) {
    ws();
    if (p < t.size() && t[p] == c) {
      ++p;
      return true;
    }
    return false;
  }
  void expect(char c) {
    if (!eat(c)) fail((std::string("expected '") + c + "'").c_str());
  }
  bool literal(const char* w) {
    const size_t n = std::strlen(w);
    if (t.compare(p, n, w) == 0) {
      p += n;
      return true;
    }
    return false;
  }
  static void put_utf8(std::string& out, unsigned cp) {
    if (cp < 0x80) {
      out += (char)cp;
    } else if (cp < 0x800) {
      out += (char)(0xC0 | (cp >> 6));
      out += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
      out += (char)(0xE0 | (cp >> 12));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    } else {
      out += (char)(0xF0 | (cp >> 18));
      out += (char)(0x80 | ((cp >> 12) & 0x3F));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    }
  }
  unsigned hex4() {
    if (p + 4 > t.size()) fail("truncated \\u escape");
    unsigned v = 0;
    for (int k = 0; k < 4; ++k) {
      const char c = t[p++];
      v <<= 4;
      if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
      else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
      else fail("bad hex digit in \\u escape");
    }
    return v;
  }
  std::string str() {
    ws();
    if (p >= t.size() || t[p] != '"') fail("string expected");
    ++p;
    std::string out;
    for (;;) {
      if (p >= t.size()) fail("unterminated string");
      const char c = t[p++];
      if (c == '"') break;
      if (c != '\\') {
        out += c;
        continue;
      }
      if (p >= t.size()) fail("unterminated escape");
      const char e = t[p++];
      switch (e) {
        case '"': out += '"'; break;
        case '\\': out += '\\'; break;
        case '/': out += '/'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'n': out += '\n'; break;
        case 'r': out += '\r'; break;
        case 't': out += '\t'; break;
        case 'u': {
          unsigned cp = hex4();
          if (cp >= 0xD800 && cp < 0xDC00 && p + 6 <= t.size() && t[p] == '\\' && t[p + 1] == 'u') {
            p += 2;
            const unsigned lo = hex4();
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          }
          put_utf8(out, cp);
          break;
        }
        default: fail("bad escape");
      }
    }
    return out;
  }
  Value num() {
    const size_t s0 = p;
    if (p < t.size() && (t[p] == '-' || t[p] == '+')) ++p;
    bool is_float = false;
    while (p < t.size()) {
      const char c = t[p];
      if (c >= '0' && c <= '9') {
        ++p;
      } else if (c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-') {
        is_float = true;
        ++p;
      } else {
        break;
      }
    }
    const std::string tok = t.substr(s0, p - s0);
    if (tok.empty() || tok == "-") fail("number expected");
    char* end = nullptr;
    if (!is_float) {
      errno = 0;
      const long long v = std::strtoll(tok.c_str(), &end, 10);
      if (errno == 0 && end && *end == '\0') return Value::integer(v);
    }
    const double v = std::strtod(tok.c_str(), &end);
    if (!end || *end != '\0') fail("malformed number");
    return Value::number(v);
  }
  Value value() {
    ws();
    if (p >= t.size()) fail("unexpected end of input");
    const char c = t[p];
    if (c == '{') {
      ++p;
      Value v = Value::object();
      if (eat('}')) return v;
      do {
        std::string k = str();
        expect(':');
        v.o[k] = value();
      } while (eat(','));
      expect('}');
      return v;
    }
    if (c == '[') {
      ++p;
      Value v;
      v.kind = Value::Kind::Array;
      if (eat(']')) return v;
      do {
        v.a.push_back(value());
      } while (eat(','));
      expect(']');
      return v;
    }
    if (c == '"') return Value::string(str());
    if (literal("true")) return Value::boolean(true);
    if (literal("false")) return Value::boolean(false);
    if (literal("null")) return Value::null();
    return num();
  }
};

void put_string(std::string& out, const std::string& s) {
  out += '"';
  for (unsigned char c : s) {
    switch (c) {
      case '"': out += "\\\""; break;
      case '\\': out += "\\\\"; break;
      case '\b': out += "\\b"; break;
      case '\f': out += "\\f"; break;
      case '\n': out += "\\n"; break;
      case '\r': out += "\\r"; break;
      case '\t': out += "\\t"; break;
      default:
        if (c < 0x20) {
          char buf[8];
          std::snprintf(buf, sizeof buf, "\\u%04x", c);
          out += buf;
        } else {
          out += (char)c;
        }
    }
  }
  out += '"';
}

// shortest of %.15g / %.16g / %.17g that reads back to the same double; integral values keep a ".0"
void put_double(std::string& out, double v) {
  if (!std::isfinite(v)) {
    out += "null";
    return;
  }
  char buf[40];
  for (int prec = 15; prec <= 17; ++prec) {
    std::snprintf(buf, sizeof buf, "%.*g", prec, v);
    if (std::strtod(buf, nullptr) == v) break;
  }
  std::string s(buf);
  if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
  out += s;
}

void write(std::string& out, const Value& v, int indent, int level) {
  const std::string pad((size_t)indent * (level + 1), ' '), pad0((size_t)indent * level, ' ');
  switch (v.kind) {
    case Value::Kind::Null: out += "null"; break;
    case Value::Kind::Bool: out += v.b ? "true" : "false"; break;
    case Value::Kind::Int: out += std::to_string(v.i); break;
    case Value::Kind::Double: put_double(out, v.d); break;
    case Value::Kind::String: put_string(out, v.s); break;
    case Value::Kind::Array: {
      if (v.a.empty()) {
        out += "[]";
        break;
      }
      out += "[\n";
      for (size_t k = 0; k < v.a.size(); ++k) {
        out += pad;
        write(out, v.a[k], indent, level + 1);
        out += (k + 1 < v.a.size()) ? ",\n" : "\n";
      }
      out += pad0 + "]";
      break;
    }
    case Value::Kind::Object: {
      if (v.o.empty()) {
        out += "{}";
        break;
      }
      out += "{\n";
      size_t k = 0;
      for (const auto& kv : v.o) {
        out += pad;
        put_string(out, kv.first);
        out += ": ";
        write(out, kv.second, indent, level + 1);
        out += (++k < v.o.size()) ? ",\n" : "\n";
      }
      out += pad0 + "}";
      break;
    }
  }
}

const char kB64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

int b64_index(unsigned char c) {
  if (c >= 'A' && c <= 'Z') return c - 'A';
  if (c >= 'a' && c <= 'z') return c - 'a' + 26;
  if (c >= '0' && c <= '9') return c - '0' + 52;
  if (c == '+' || c == '-') return 62;  // the URL-safe alphabet is read too
  if (c == '/' || c == '_') return 63;
  return -1;
}

// doubles as little-endian bytes, independent of the host's byte order
void put_le(std::vector<unsigned char>& out, double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  for (int k = 0; k < 8; ++k) out.push_back((unsigned char)(u >> (8 * k)));
}

double get_le(const unsigned char* p) {
  uint64_t u = 0;
  for (int k = 0; k < 8; ++k) u |= (uint64_t)p[k] << (8 * k);
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}

std::string payload(const double* p, size_t n) {
  std::vector<unsigned char> bytes;
  bytes.reserve(n * 8);
  for (size_t k = 0; k < n; ++k) put_le(bytes, p[k]);
  return base64_encode(bytes.data(), bytes.size());
}

std::vector<double> unpayload(const Value& v, size_t expect) {
  const std::vector<unsigned char> bytes = base64_decode(v.at("base64_data").as_string());
  if (bytes.size() % 8 != 0) throw std::runtime_error("JSON matrix payload is not a whole number of doubles");
  const size_t n = bytes.size() / 8;
  if (n != expect)
    throw std::runtime_error("JSON matrix payload holds " + std::to_string(n) + " values, its header says " +
                             std::to_string(expect));
  std::vector<double> out(n);
  for (size_t k = 0; k < n; ++k) out[k] = get_le(bytes.data() + 8 * k);
  return out;
}

}  // namespace

Value parse(const std::string& text) {
  Parser ps(text);
  Value v = ps.value();
  ps.ws();
  if (ps.p != text.size()) ps.fail("trailing characters");
  return v;
}

std::string dump(const Value& v, int indent) {
  std::string out;
  write(out, v, indent, 0);
  return out;
}

std::string base64_encode(const unsigned char* data, size_t len) {
  std::string out;
  out.reserve((len + 2) / 3 * 4);
  size_t k = 0;
  for (; k + 3 <= len; k += 3) {
    const unsigned w = ((unsigned)data[k] << 16) | ((unsigned)data[k + 1] << 8) | data[k + 2];
    out += kB64[(w >> 18) & 63];
    out += kB64[(w >> 12) & 63];
    out += kB64[(w >> 6) & 63];
    out += kB64[w & 63];
  }
  if (len - k == 1) {
    const unsigned w = (unsigned)data[k] << 16;
    out += kB64[(w >> 18) & 63];
    out += kB64[(w >> 12) & 63];
    out += "==";
  } else if (len - k == 2) {
    const unsigned w = ((unsigned)data[k] << 16) | ((unsigned)data[k + 1] << 8);
    out += kB64[(w >> 18) & 63];
    out += kB64[(w >> 12) & 63];
    out += kB64[(w >> 6) & 63];
    out += '=';
  }
  return out;
}

std::vector<unsigned char> base64_decode(const std::string& text) {
  std::vector<unsigned char> out;
  out.reserve(text.size() / 4 * 3);
  unsigned acc = 0;
  int bits = 0;
  for (unsigned char c : text) {
    if (c == '=') break;
    if (c == '\n' || c == '\r') continue;
    const int v = b64_index(c);
    if (v < 0) throw std::runtime_error("Input is not valid base64-encoded data.");
    acc = (acc << 6) | (unsigned)v;
    bits += 6;
    if (bits >= 8) {
      bits -= 8;
      out.push_back((unsigned char)((acc >> bits) & 0xFF));
    }
  }
  return out;
}

Value mat_to_json(const double* p, int64_t rows, int64_t cols) {
  Value v = Value::object();
  v["type"] = Value::string("mat");
  v["n_rows"] = Value::integer(rows);
  v["n_cols"] = Value::integer(cols);
  v["base64_data"] = Value::string(payload(p, (size_t)(rows * cols)));
  return v;
}

namespace {
Value vec_to_json(const std::vector<double>& x, const char* type) {
  Value v = Value::object();
  v["type"] = Value::string(type);
  v["size"] = Value::integer((long long)x.size());
  v["base64_data"] = Value::string(payload(x.data(), x.size()));
  return v;
}
}  // namespace

Value colvec_to_json(const std::vector<double>& v) { return vec_to_json(v, "colvec"); }
Value rowvec_to_json(const std::vector<double>& v) { return vec_to_json(v, "rowvec"); }

std::vector<double> mat_from_json(const Value& v, int64_t* rows, int64_t* cols) {
  if (v.at("type").as_string() != "mat") throw std::runtime_error("JSON: matrix object expected");
  const long long r = v.at("n_rows").as_int(), c = v.at("n_cols").as_int();
  if (r < 0 || c < 0) throw std::runtime_error("JSON: negative matrix size");
  *rows = r;
  *cols = c;
  return unpayload(v, (size_t)(r * c));
}

std::vector<double> vec_from_json(const Value& v, const char* type) {
  const std::string& t = v.at("type").as_string();
  if (t != type) throw std::runtime_error(std::string("JSON: ") + type + " expected, found " + t);
  const long long n = v.at("size").as_int();
  if (n < 0) throw std::runtime_error("JSON: negative vector size");
  return unpayload(v, (size_t)n);
}

}  // namespace json
}  // namespace lkg
