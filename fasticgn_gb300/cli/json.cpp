#include "json.h"

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <set>

namespace dic_cli
{

bool Json::as_bool() const
{
  if (kind_ != Kind::Bool) throw JsonError("JSON value is not a boolean");
  return b_;
}
unsigned long long Json::as_u64() const
{
  if (kind_ != Kind::Uint) throw JsonError("JSON value is not an unsigned integer");
  return u_;
}
double Json::as_double() const
{
  switch (kind_)
  {
    case Kind::Int: return (double)i_;
    case Kind::Uint: return (double)u_;
    case Kind::Float: return d_;
    default: throw JsonError("JSON value is not a number");
  }
}
const std::string& Json::as_string() const
{
  if (kind_ != Kind::String) throw JsonError("JSON value is not a string");
  return s_;
}
size_t Json::size() const
{
  if (kind_ == Kind::Array) return a_.size();
  if (kind_ == Kind::Object) return o_.size();
  return kind_ == Kind::Null ? 0 : 1;
}
const Json& Json::at(const std::string& key) const
{
  if (kind_ != Kind::Object) throw JsonError("JSON value is not an object (looking up '" + key + "')");
  const auto it = o_.find(key);
  if (it == o_.end()) throw JsonError("JSON object has no member '" + key + "'");
  return it->second;
}
const Json& Json::at(size_t i) const
{
  if (kind_ != Kind::Array || i >= a_.size()) throw JsonError("JSON array index out of range");
  return a_[i];
}
Json& Json::operator[](const std::string& key)
{
  if (kind_ == Kind::Null) kind_ = Kind::Object;
  if (kind_ != Kind::Object) throw JsonError("JSON value is not an object (setting '" + key + "')");
  return o_[key];
}
void Json::push(Json v)
{
  if (kind_ == Kind::Null) kind_ = Kind::Array;
  if (kind_ != Kind::Array) throw JsonError("JSON value is not an array");
  a_.push_back(std::move(v));
}
std::string Json::str_or(const std::string& key, const std::string& fallback) const
{
  return has(key) && o_.at(key).is_string() ? o_.at(key).s_ : fallback;
}
unsigned long long Json::u64_or(const std::string& key, unsigned long long fallback) const
{
  return has(key) && o_.at(key).is_unsigned() ? o_.at(key).u_ : fallback;
}

bool Json::operator==(const Json& o) const
{
  if (is_number() && o.is_number())
  {
    // numbers compare by value across the integer kinds (nlohmann's rule)
    if (kind_ == Kind::Float || o.kind_ == Kind::Float) return as_double() == o.as_double();
    if (kind_ == Kind::Int || o.kind_ == Kind::Int)
      return kind_ == o.kind_ ? i_ == o.i_ : false;   // a negative never equals an unsigned
    return u_ == o.u_;
  }
  if (kind_ != o.kind_) return false;
  switch (kind_)
  {
    case Kind::Null: return true;
    case Kind::Bool: return b_ == o.b_;
    case Kind::String: return s_ == o.s_;
    case Kind::Array: return a_ == o.a_;
    case Kind::Object: return o_ == o.o_;
    default: return false;
  }
}

// ------------------------------------------------------------------ serialisation
bool valid_utf8(const std::string& s)
{
  size_t i = 0;
  const size_t n = s.size();
  while (i < n)
  {
    const unsigned char c = (unsigned char)s[i];
    int extra;
    unsigned cp;
    if (c < 0x80) { ++i; continue; }
    if (c >= 0xC2 && c <= 0xDF) { extra = 1; cp = c & 0x1F; }
    else if (c >= 0xE0 && c <= 0xEF) { extra = 2; cp = c & 0x0F; }
    else if (c >= 0xF0 && c <= 0xF4) { extra = 3; cp = c & 0x07; }
    else return false;
    for (int k = 1; k <= extra; ++k)
    {
      if (i + k >= n) return false;
      const unsigned char t = (unsigned char)s[i + k];
      if ((t & 0xC0) != 0x80) return false;
      cp = (cp << 6) | (t & 0x3F);
    }
    // overlong forms, surrogates and code points past U+10FFFF
    if ((extra == 2 && cp < 0x800) || (extra == 3 && (cp < 0x10000 || cp > 0x10FFFF)) ||
        (cp >= 0xD800 && cp <= 0xDFFF))
      return false;
    i += (size_t)extra + 1;
  }
  return true;
}

std::string json_quote(const std::string& s)
{
  if (!valid_utf8(s)) throw JsonError("string is not valid UTF-8");
  std::string o;
  o.reserve(s.size() + 2);
  o += '"';
  for (unsigned char c : s)
  {
    switch (c)
    {
      case '"': o += "\\\""; break;
      case '\\': o += "\\\\"; break;
      case '\b': o += "\\b"; break;
      case '\f': o += "\\f"; break;
      case '\n': o += "\\n"; break;
      case '\r': o += "\\r"; break;
      case '\t': o += "\\t"; break;
      default:
        if (c < 0x20)
        {
          char b[8];
          std::snprintf(b, sizeof b, "\\u%04x", c);
          o += b;
        }
        else
          o += (char)c;
    }
  }
  o += '"';
  return o;
}

std::string json_double(double v)
{
  if (!std::isfinite(v)) return "null";
  if (v == 0.0) return std::signbit(v) ? "-0.0" : "0.0";
  // shortest round-trip digits and their decimal exponent
  char b[64];
  const auto r = std::to_chars(b, b + sizeof b, v, std::chars_format::scientific);
  std::string sci(b, r.ptr);
  std::string out;
  if (sci[0] == '-')
  {
    out = "-";
    sci.erase(0, 1);
  }
  const size_t epos = sci.find('e');
  std::string digits = sci.substr(0, epos);
  digits.erase(std::remove(digits.begin(), digits.end(), '.'), digits.end());
  const int exp10 = std::atoi(sci.c_str() + epos + 1);
  const int k = (int)digits.size();
  const int n = exp10 + 1;   // value = 0.d1d2..dk x 10^n
  if (k <= n && n <= 15)
    out += digits + std::string((size_t)(n - k), '0') + ".0";
  else if (0 < n && n <= 15)
    out += digits.substr(0, (size_t)n) + "." + digits.substr((size_t)n);
  else if (-4 < n && n <= 0)
    out += "0." + std::string((size_t)(-n), '0') + digits;
  else
  {
    out += digits.substr(0, 1);
    if (k > 1) out += "." + digits.substr(1);
    const int e = n - 1;
    char eb[16];
    std::snprintf(eb, sizeof eb, "e%c%02d", e < 0 ? '-' : '+', e < 0 ? -e : e);
    out += eb;
  }
  return out;
}

void Json::dump_to(std::string& out) const
{
  switch (kind_)
  {
    case Kind::Null: out += "null"; break;
    case Kind::Bool: out += b_ ? "true" : "false"; break;
    case Kind::Int: out += std::to_string(i_); break;
    case Kind::Uint: out += std::to_string(u_); break;
    case Kind::Float: out += json_double(d_); break;
    case Kind::String: out += json_quote(s_); break;
    case Kind::Array:
      out += '[';
      for (size_t i = 0; i < a_.size(); ++i)
      {
        if (i) out += ',';
        a_[i].dump_to(out);
      }
      out += ']';
      break;
    case Kind::Object:
    {
      out += '{';
      bool first = true;
      for (const auto& m : o_)
      {
        if (!first) out += ',';
        first = false;
        out += json_quote(m.first);
        out += ':';
        m.second.dump_to(out);
      }
      out += '}';
      break;
    }
  }
}

std::string Json::dump() const
{
  std::string out;
  dump_to(out);
  return out;
}

void Json::dump_indented_to(std::string& out, int indent, int level) const
{
  const std::string pad((size_t)(indent * (level + 1)), ' '), close((size_t)(indent * level), ' ');
  if (kind_ == Kind::Array && !a_.empty())
  {
    out += "[\n";
    for (size_t i = 0; i < a_.size(); ++i)
    {
      out += pad;
      a_[i].dump_indented_to(out, indent, level + 1);
      out += i + 1 < a_.size() ? ",\n" : "\n";
    }
    out += close + "]";
  }
  else if (kind_ == Kind::Object && !o_.empty())
  {
    out += "{\n";
    size_t i = 0;
    for (const auto& m : o_)
    {
      out += pad + json_quote(m.first) + ": ";
      m.second.dump_indented_to(out, indent, level + 1);
      out += ++i < o_.size() ? ",\n" : "\n";
    }
    out += close + "}";
  }
  else
    dump_to(out);
}

std::string Json::dump_indented(int indent) const
{
  std::string out;
  dump_indented_to(out, indent, 0);
  return out;
}

// ------------------------------------------------------------------ parsing
class JsonParser
{
 public:
  JsonParser(const std::string& t, const std::string& label) : t_(t), label_(label) {}
  Json run()
  {
    ws();
    Json v = value(0);
    ws();
    if (p_ != t_.size()) fail("unexpected text after the JSON value");
    return v;
  }

 private:
  const std::string& t_;
  const std::string& label_;
  size_t p_ = 0;

  [[noreturn]] void fail(const std::string& what) const
  {
    throw JsonError("invalid JSON in " + label_ + " at byte " + std::to_string(p_) + ": " + what);
  }
  void ws()
  {
    while (p_ < t_.size() && (t_[p_] == ' ' || t_[p_] == '\t' || t_[p_] == '\n' || t_[p_] == '\r')) ++p_;
  }
  bool eat(char c)
  {
    if (p_ < t_.size() && t_[p_] == c)
    {
      ++p_;
      return true;
    }
    return false;
  }
  void literal(const char* word)
  {
    const size_t n = std::strlen(word);
    if (t_.compare(p_, n, word) != 0) fail("unknown literal");
    p_ += n;
  }
  Json value(int depth)
  {
    if (depth > 64) fail("nesting exceeds 64");
    if (p_ >= t_.size()) fail("unexpected end of input");
    const char c = t_[p_];
    if (c == '{') return object(depth);
    if (c == '[') return array(depth);
    if (c == '"') return Json(string());
    if (c == 't') { literal("true"); return Json(true); }
    if (c == 'f') { literal("false"); return Json(false); }
    if (c == 'n') { literal("null"); return Json(); }
    if (c == '-' || (c >= '0' && c <= '9')) return number();
    fail("unexpected character");
  }
  Json object(int depth)
  {
    ++p_;
    Json o = Json::object();
    ws();
    if (eat('}')) return o;
    for (;;)
    {
      ws();
      if (p_ >= t_.size() || t_[p_] != '"') fail("expected an object key");
      std::string key = string();
      if (o.o_.count(key)) fail("duplicate object key '" + key + "'");
      ws();
      if (!eat(':')) fail("expected ':'");
      ws();
      o.o_.emplace(std::move(key), value(depth + 1));
      ws();
      if (eat(',')) continue;
      if (eat('}')) return o;
      fail("expected ',' or '}'");
    }
  }
  Json array(int depth)
  {
    ++p_;
    Json a = Json::array();
    ws();
    if (eat(']')) return a;
    for (;;)
    {
      ws();
      a.a_.push_back(value(depth + 1));
      ws();
      if (eat(',')) continue;
      if (eat(']')) return a;
      fail("expected ',' or ']'");
    }
  }
  unsigned hex4()
  {
    if (p_ + 4 > t_.size()) fail("short \\u escape");
    unsigned v = 0;
    for (int k = 0; k < 4; ++k)
    {
      const char c = t_[p_++];
      v <<= 4;
      if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
      else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
      else fail("bad \\u escape");
    }
    return v;
  }
  static void put_utf8(std::string& o, unsigned cp)
  {
    if (cp < 0x80) o += (char)cp;
    else if (cp < 0x800) { o += (char)(0xC0 | (cp >> 6)); o += (char)(0x80 | (cp & 0x3F)); }
    else if (cp < 0x10000)
    {
      o += (char)(0xE0 | (cp >> 12));
      o += (char)(0x80 | ((cp >> 6) & 0x3F));
      o += (char)(0x80 | (cp & 0x3F));
    }
    else
    {
      o += (char)(0xF0 | (cp >> 18));
      o += (char)(0x80 | ((cp >> 12) & 0x3F));
      o += (char)(0x80 | ((cp >> 6) & 0x3F));
      o += (char)(0x80 | (cp & 0x3F));
    }
  }
  std::string string()
  {
    ++p_;   // opening quote
    std::string o;
    for (;;)
    {
      if (p_ >= t_.size()) fail("unterminated string");
      const unsigned char c = (unsigned char)t_[p_];
      if (c == '"')
      {
        ++p_;
        break;
      }
      if (c < 0x20) fail("control character in a string");
      if (c != '\\')
      {
        o += (char)c;
        ++p_;
        continue;
      }
      ++p_;
      if (p_ >= t_.size()) fail("unterminated escape");
      const char e = t_[p_++];
      switch (e)
      {
        case '"': o += '"'; break;
        case '\\': o += '\\'; break;
        case '/': o += '/'; break;
        case 'b': o += '\b'; break;
        case 'f': o += '\f'; break;
        case 'n': o += '\n'; break;
        case 'r': o += '\r'; break;
        case 't': o += '\t'; break;
        case 'u':
        {
          unsigned cp = hex4();
          if (cp >= 0xD800 && cp <= 0xDBFF)
          {
            if (!(p_ + 1 < t_.size() && t_[p_] == '\\' && t_[p_ + 1] == 'u')) fail("unpaired surrogate");
            p_ += 2;
            const unsigned lo = hex4();
            if (lo < 0xDC00 || lo > 0xDFFF) fail("unpaired surrogate");
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          }
          else if (cp >= 0xDC00 && cp <= 0xDFFF)
            fail("unpaired surrogate");
          put_utf8(o, cp);
          break;
        }
        default: fail("bad escape");
      }
    }
    if (!valid_utf8(o)) fail("string is not valid UTF-8");
    return o;
  }
  Json number()
  {
    const size_t s = p_;
    bool neg = false, frac = false;
    if (eat('-')) neg = true;
    if (p_ >= t_.size()) fail("bad number");
    if (t_[p_] == '0')
      ++p_;
    else if (t_[p_] >= '1' && t_[p_] <= '9')
      while (p_ < t_.size() && t_[p_] >= '0' && t_[p_] <= '9') ++p_;
    else
      fail("bad number");
    if (p_ < t_.size() && t_[p_] == '.')
    {
      frac = true;
      ++p_;
      if (p_ >= t_.size() || t_[p_] < '0' || t_[p_] > '9') fail("bad fraction");
      while (p_ < t_.size() && t_[p_] >= '0' && t_[p_] <= '9') ++p_;
    }
    if (p_ < t_.size() && (t_[p_] == 'e' || t_[p_] == 'E'))
    {
      frac = true;
      ++p_;
      if (p_ < t_.size() && (t_[p_] == '+' || t_[p_] == '-')) ++p_;
      if (p_ >= t_.size() || t_[p_] < '0' || t_[p_] > '9') fail("bad exponent");
      while (p_ < t_.size() && t_[p_] >= '0' && t_[p_] <= '9') ++p_;
    }
    const char* b = t_.data() + s;
    const char* e = t_.data() + p_;
    if (!frac)
    {
      if (neg)
      {
        long long v = 0;
        const auto r = std::from_chars(b, e, v);
        if (r.ec == std::errc() && r.ptr == e) return Json(v);
      }
      else
      {
        unsigned long long v = 0;
        const auto r = std::from_chars(b, e, v);
        if (r.ec == std::errc() && r.ptr == e) return Json(v);
      }
    }
    double d = 0.0;
    const auto r = std::from_chars(b, e, d);
    if (r.ec != std::errc() || r.ptr != e) fail("number out of range");
    return Json(d);
  }
};

Json Json::parse(const std::string& text, const std::string& label)
{
  return JsonParser(text, label).run();
}

}  // namespace dic_cli
