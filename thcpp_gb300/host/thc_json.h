// A small JSON value type with the subset of the nlohmann::json interface that thcpp's
// entry points use (parse from a stream, at(), get<T>(), dump(), json::out_of_range), so
// the reference's constructors keep their `nlohmann::json&` signatures.  Defining
// THC_USE_NLOHMANN_JSON before including this header switches to the real library.
#pragma once

#ifdef THC_USE_NLOHMANN_JSON
#include "json.hpp"
#else

#include <cctype>
#include <cstdlib>
#include <istream>
#include <iterator>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace thc {

class Json {
 public:
  enum class Type { Null, Bool, Number, String, Array, Object };

  struct exception : std::runtime_error {
    using std::runtime_error::runtime_error;
  };
  struct out_of_range : exception {
    using exception::exception;
  };
  struct type_error : exception {
    using exception::exception;
  };
  struct parse_error : exception {
    using exception::exception;
  };

  Json() = default;
  Json(bool b) : t_(Type::Bool), b_(b) {}
  Json(double d) : t_(Type::Number), d_(d) {}
  Json(int i) : t_(Type::Number), d_(i) {}
  Json(const char* s) : t_(Type::String), s_(s) {}
  Json(const std::string& s) : t_(Type::String), s_(s) {}

  Type type() const { return t_; }
  bool is_object() const { return t_ == Type::Object; }

  const Json& at(const std::string& key) const
  {
    if (t_ != Type::Object) throw type_error("[json.exception.type_error] cannot use at() with non-object");
    auto it = o_.find(key);
    if (it == o_.end()) throw out_of_range("[json.exception.out_of_range.403] key '" + key + "' not found");
    return it->second;
  }
  Json& at(const std::string& key)
  {
    return const_cast<Json&>(static_cast<const Json&>(*this).at(key));
  }
  Json& operator[](const std::string& key)
  {
    if (t_ == Type::Null) t_ = Type::Object;
    return o_[key];
  }
  bool contains(const std::string& key) const { return t_ == Type::Object && o_.count(key); }
  size_t size() const { return t_ == Type::Array ? a_.size() : t_ == Type::Object ? o_.size() : 1; }
  const Json& operator[](size_t i) const { return a_.at(i); }

  template <typename T>
  T get() const
  {
    if constexpr (std::is_same<T, std::string>::value) {
      if (t_ != Type::String) throw type_error("[json.exception.type_error.302] type must be string");
      return s_;
    } else if constexpr (std::is_same<T, bool>::value) {
      if (t_ != Type::Bool) throw type_error("[json.exception.type_error.302] type must be boolean");
      return b_;
    } else {
      static_assert(std::is_arithmetic<T>::value, "unsupported get<T>()");
      if (t_ != Type::Number) throw type_error("[json.exception.type_error.302] type must be number");
      return static_cast<T>(d_);
    }
  }

  std::string dump(int indent = -1) const
  {
    std::ostringstream os;
    write(os, indent, 0);
    return os.str();
  }

  static Json parse(const std::string& text)
  {
    size_t p = 0;
    Json v = parse_value(text, p);
    skip(text, p);
    if (p != text.size()) throw parse_error("[json.exception.parse_error] trailing characters");
    return v;
  }

  friend std::istream& operator>>(std::istream& is, Json& j)
  {
    std::string text((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
    j = parse(text);
    return is;
  }

 private:
  Type t_ = Type::Null;
  bool b_ = false;
  double d_ = 0.0;
  std::string s_;
  std::vector<Json> a_;
  std::map<std::string, Json> o_;

  static void skip(const std::string& s, size_t& p)
  {
    while (p < s.size() && std::isspace((unsigned char)s[p])) p++;
  }

  static std::string parse_string(const std::string& s, size_t& p)
  {
    if (s[p] != '"') throw parse_error("[json.exception.parse_error] expected string");
    p++;
    std::string out;
    while (p < s.size() && s[p] != '"') {
      char c = s[p++];
      if (c == '\\' && p < s.size()) {
        char e = s[p++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u': {
            unsigned cp = std::stoul(s.substr(p, 4), nullptr, 16);
            p += 4;
            if (cp < 0x80) out += (char)cp;
            else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
            else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
            break;
          }
          default: out += e;
        }
      } else {
        out += c;
      }
    }
    if (p >= s.size()) throw parse_error("[json.exception.parse_error] unterminated string");
    p++;
    return out;
  }

  static Json parse_value(const std::string& s, size_t& p)
  {
    skip(s, p);
    if (p >= s.size()) throw parse_error("[json.exception.parse_error] unexpected end of input");
    char c = s[p];
    if (c == '{') {
      Json j;
      j.t_ = Type::Object;
      p++;
      skip(s, p);
      if (s[p] == '}') { p++; return j; }
      while (true) {
        skip(s, p);
        std::string k = parse_string(s, p);
        skip(s, p);
        if (s[p] != ':') throw parse_error("[json.exception.parse_error] expected ':'");
        p++;
        j.o_[k] = parse_value(s, p);
        skip(s, p);
        if (s[p] == ',') { p++; continue; }
        if (s[p] == '}') { p++; return j; }
        throw parse_error("[json.exception.parse_error] expected ',' or '}'");
      }
    }
    if (c == '[') {
      Json j;
      j.t_ = Type::Array;
      p++;
      skip(s, p);
      if (s[p] == ']') { p++; return j; }
      while (true) {
        j.a_.push_back(parse_value(s, p));
        skip(s, p);
        if (s[p] == ',') { p++; continue; }
        if (s[p] == ']') { p++; return j; }
        throw parse_error("[json.exception.parse_error] expected ',' or ']'");
      }
    }
    if (c == '"') return Json(parse_string(s, p));
    if (!s.compare(p, 4, "true")) { p += 4; return Json(true); }
    if (!s.compare(p, 5, "false")) { p += 5; return Json(false); }
    if (!s.compare(p, 4, "null")) { p += 4; return Json(); }
    const char* b = s.c_str() + p;
    char* e = nullptr;
    double d = std::strtod(b, &e);
    if (e == b) throw parse_error("[json.exception.parse_error] invalid literal");
    p += (size_t)(e - b);
    return Json(d);
  }

  void write(std::ostringstream& os, int indent, int level) const
  {
    auto nl = [&](int l) {
      if (indent >= 0) { os << '\n'; for (int i = 0; i < l * indent; i++) os << ' '; }
    };
    switch (t_) {
      case Type::Null: os << "null"; break;
      case Type::Bool: os << (b_ ? "true" : "false"); break;
      case Type::Number: {
        if (d_ == (double)(long long)d_ && std::abs(d_) < 1e15) os << (long long)d_;
        else os << d_;
        break;
      }
      case Type::String: os << '"' << s_ << '"'; break;
      case Type::Array: {
        os << '[';
        for (size_t i = 0; i < a_.size(); i++) {
          if (i) os << ',';
          nl(level + 1);
          a_[i].write(os, indent, level + 1);
        }
        if (!a_.empty()) nl(level);
        os << ']';
        break;
      }
      case Type::Object: {
        os << '{';
        size_t i = 0;
        for (auto& kv : o_) {
          if (i++) os << ',';
          nl(level + 1);
          os << '"' << kv.first << "\":" << (indent >= 0 ? " " : "");
          kv.second.write(os, indent, level + 1);
        }
        if (!o_.empty()) nl(level);
        os << '}';
        break;
      }
    }
  }
};

}  // namespace thc

namespace nlohmann {
using json = thc::Json;
}

#endif
