// A small JSON value for the output ledger: strict parsing (RFC 8259 grammar, UTF-8,
// \u escapes with surrogate pairs, duplicate keys and nesting deeper than 64 rejected, as
// the reference's readJson does, src/cli_output_integrity.cpp:281-292) and a compact
// serialisation with object keys in byte order and nlohmann::json's number and string
// formats, so that the digest of a serialised contract or manifest is the one the
// reference's ledger computes for the same document.
#pragma once

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace dic_cli
{

struct JsonError : std::runtime_error
{
  using std::runtime_error::runtime_error;
};

class Json
{
 public:
  enum class Kind { Null, Bool, Int, Uint, Float, String, Array, Object };

  Json() = default;
  Json(std::nullptr_t) {}
  Json(bool b) : kind_(Kind::Bool), b_(b) {}
  Json(int v) : Json((long long)v) {}
  Json(long v) : Json((long long)v) {}
  Json(long long v) : kind_(v < 0 ? Kind::Int : Kind::Uint), i_(v), u_((unsigned long long)v) {}
  Json(unsigned v) : Json((unsigned long long)v) {}
  Json(unsigned long v) : Json((unsigned long long)v) {}
  Json(unsigned long long v) : kind_(Kind::Uint), u_(v) {}
  Json(double v) : kind_(Kind::Float), d_(v) {}
  Json(const char* s) : kind_(Kind::String), s_(s) {}
  Json(std::string s) : kind_(Kind::String), s_(std::move(s)) {}
  static Json array() { Json j; j.kind_ = Kind::Array; return j; }
  static Json object() { Json j; j.kind_ = Kind::Object; return j; }

  Kind kind() const { return kind_; }
  bool is_null() const { return kind_ == Kind::Null; }
  bool is_bool() const { return kind_ == Kind::Bool; }
  bool is_number() const { return kind_ == Kind::Int || kind_ == Kind::Uint || kind_ == Kind::Float; }
  bool is_unsigned() const { return kind_ == Kind::Uint; }
  bool is_string() const { return kind_ == Kind::String; }
  bool is_array() const { return kind_ == Kind::Array; }
  bool is_object() const { return kind_ == Kind::Object; }

  bool as_bool() const;
  unsigned long long as_u64() const;
  double as_double() const;
  const std::string& as_string() const;

  size_t size() const;
  const std::vector<Json>& items() const { return a_; }
  const std::map<std::string, Json>& members() const { return o_; }
  bool has(const std::string& key) const { return kind_ == Kind::Object && o_.count(key) != 0; }
  const Json& at(const std::string& key) const;
  const Json& at(size_t i) const;
  Json& operator[](const std::string& key);   // turns null into an object
  void push(Json v);                          // turns null into an array
  void erase(const std::string& key) { o_.erase(key); }
  // member `key` when it is a string, else `fallback`
  std::string str_or(const std::string& key, const std::string& fallback) const;
  // member `key` when it is an unsigned integer, else `fallback`
  unsigned long long u64_or(const std::string& key, unsigned long long fallback) const;

  bool operator==(const Json& o) const;
  bool operator!=(const Json& o) const { return !(*this == o); }

  std::string dump() const;
  // nlohmann's dump(indent): one member or element per line, ": " after keys, empty
  // containers as {} and []
  std::string dump_indented(int indent = 2) const;
  static Json parse(const std::string& text, const std::string& label);

 private:
  Kind kind_ = Kind::Null;
  bool b_ = false;
  long long i_ = 0;
  unsigned long long u_ = 0;
  double d_ = 0.0;
  std::string s_;
  std::vector<Json> a_;
  std::map<std::string, Json> o_;
  void dump_to(std::string& out) const;
  void dump_indented_to(std::string& out, int indent, int level) const;
  friend class JsonParser;
};

// the string as one JSON string literal (nlohmann's escapes); throws on invalid UTF-8
std::string json_quote(const std::string& s);
// nlohmann's rendering of a double (shortest round trip, ".0" on integral values, exponent
// form outside 1e-5 .. 1e15)
std::string json_double(double v);
bool valid_utf8(const std::string& s);

}  // namespace dic_cli
