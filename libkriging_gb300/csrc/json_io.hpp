// json_io.hpp -- the JSON document model of libKriging's model files (version 2), written from scratch.
//
// The reference serialises models with nlohmann::json (src/lib/Kriging.cpp:2691-2749,
// src/lib/KrigingImpl.cpp:644-711) and stores every Armadillo vector / matrix as an object
//   {"type": "mat" | "colvec" | "rowvec", "n_rows": r, "n_cols": c | "size": s, "base64_data": "..."}
// whose payload is the column-major sequence of little-endian IEEE-754 doubles, base64-encoded with the standard
// alphabet and '=' padding (src/lib/utils/jsonutils.cpp:66-110).  This file holds a small JSON value type, a parser,
// a writer (objects with sorted keys and four-space indentation, as nlohmann::json's std::map objects print) and
// the matrix <-> JSON conversions of that format.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace lkg {
namespace json {

struct Value {
  enum class Kind { Null, Bool, Int, Double, String, Array, Object };
  Kind kind = Kind::Null;
  bool b = false;
  long long i = 0;
  double d = 0.0;
  std::string s;
  std::vector<Value> a;
  std::map<std::string, Value> o;

  static Value null() { return Value{}; }
  static Value boolean(bool v) {
    Value x;
    x.kind = Kind::Bool;
    x.b = v;
    return x;
  }
  static Value integer(long long v) {
    Value x;
    x.kind = Kind::Int;
    x.i = v;
    return x;
  }
  static Value number(double v) {
    Value x;
    x.kind = Kind::Double;
    x.d = v;
    return x;
  }
  static Value string(const std::string& v) {
    Value x;
    x.kind = Kind::String;
    x.s = v;
    return x;
  }
  static Value object() {
    Value x;
    x.kind = Kind::Object;
    return x;
  }

  bool contains(const std::string& key) const { return kind == Kind::Object && o.count(key) != 0; }
  // member access; throws std::runtime_error naming the key when it is missing
  const Value& at(const std::string& key) const;
  Value& operator[](const std::string& key) {
    kind = Kind::Object;
    return o[key];
  }
  double as_double() const;       // Int or Double
  long long as_int() const;       // Int, or a Double holding an integer
  bool as_bool() const;
  const std::string& as_string() const;
};

Value parse(const std::string& text);                     // throws std::runtime_error on malformed input
std::string dump(const Value& v, int indent = 4);         // pretty-printed, keys sorted

std::string base64_encode(const unsigned char* data, size_t len);
std::vector<unsigned char> base64_decode(const std::string& text);  // throws on characters outside the alphabet

// Armadillo objects of the model files.  Matrices are column-major with explicit sizes.
Value mat_to_json(const double* p, int64_t rows, int64_t cols);
Value colvec_to_json(const std::vector<double>& v);
Value rowvec_to_json(const std::vector<double>& v);
std::vector<double> mat_from_json(const Value& v, int64_t* rows, int64_t* cols);
std::vector<double> vec_from_json(const Value& v, const char* type);  // "colvec" or "rowvec"

}  // namespace json
}  // namespace lkg
