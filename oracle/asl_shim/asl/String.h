// From-scratch stand-in for asl/String.h (see defs.h).  Restated semantics
// (ASL's own implementation is not available, so these are choices, applied
// identically to the oracle's reference build and to the product's loaders):
//   split()            whitespace-separated tokens, empty tokens skipped
//   split(c, out)      fields separated by c, empty fields kept
//   (float)s / (int)s  strtod then cast to float / strtol base 10, 0 if not a number
//   s | def            s if non-empty, else def
#ifndef ASL_SHIM_STRING_H
#define ASL_SHIM_STRING_H
#include "defs.h"
#include "Array.h"
#include <string>
#include <string.h>
#include <ctype.h>
namespace asl {
class String {
  std::string s_;
 public:
  String() {}
  String(const char* s) : s_(s ? s : "") {}
  String(const std::string& s) : s_(s) {}
  String(const char* s, int n) : s_(s, (size_t)n) {}
  const char* operator*() const { return s_.c_str(); }
  const std::string& str() const { return s_; }
  int length() const { return (int)s_.size(); }
  bool ok() const { return !s_.empty(); }
  char operator[](int i) const { return s_[(size_t)i]; }
  bool operator==(const char* b) const { return s_ == b; }
  bool operator==(const String& b) const { return s_ == b.s_; }
  bool operator==(char c) const { return s_.size() == 1 && s_[0] == c; }
  bool operator!=(const char* b) const { return !(*this == b); }
  bool operator!=(const String& b) const { return !(*this == b); }
  bool operator<(const String& b) const { return s_ < b.s_; }
  bool startsWith(char c) const { return !s_.empty() && s_[0] == c; }
  bool startsWith(const char* p) const { return s_.compare(0, strlen(p), p) == 0; }
  operator float() const { return (float)strtod(s_.c_str(), nullptr); }
  operator int() const { return (int)strtol(s_.c_str(), nullptr, 10); }
  String operator|(const char* def) const { return s_.empty() ? String(def) : *this; }
  String operator+(const String& b) const { return String(s_ + b.s_); }
  String operator+(const char* b) const { return String(s_ + b); }
  String& operator<<(const String& b) { s_ += b.s_; return *this; }
  String& operator<<(const char* b) { s_ += b; return *this; }
  String& operator<<(char c) { s_ += c; return *this; }
  String& operator<<(int v) { s_ += std::to_string(v); return *this; }
  static String repeat(char c, int n) { return String(std::string((size_t)n, c)); }
  String replace(char a, char b) const {
    std::string r = s_;
    for (auto& c : r) if (c == a) c = b;
    return String(r);
  }
  String replace(const char* a, const char* b) const {
    std::string r;
    size_t la = strlen(a);
    if (!la) return *this;
    for (size_t i = 0; i < s_.size();) {
      if (s_.compare(i, la, a) == 0) { r += b; i += la; }
      else r += s_[i++];
    }
    return String(r);
  }
  Array<String> split() const {
    Array<String> out;
    size_t i = 0, n = s_.size();
    while (i < n) {
      while (i < n && isspace((unsigned char)s_[i])) i++;
      size_t j = i;
      while (j < n && !isspace((unsigned char)s_[j])) j++;
      if (j > i) out << String(s_.substr(i, j - i));
      i = j;
    }
    return out;
  }
  void split(char sep, Array<String>& out) const {
    out.clear();
    size_t i = 0;
    for (;;) {
      size_t j = s_.find(sep, i);
      if (j == std::string::npos) { out << String(s_.substr(i)); break; }
      out << String(s_.substr(i, j - i));
      i = j + 1;
    }
  }
  template <class T> Array<T> split_() const {
    Array<String> p = split();
    Array<T> out;
    for (int i = 0; i < p.length(); i++) out << (T)p[i];
    return out;
  }
};
inline String operator+(const char* a, const String& b) { return String(a) + b; }
}  // namespace asl
#endif
