// From-scratch stand-in for asl/TextFile.h (see defs.h): a text file read by
// whitespace-separated tokens (>>) or by lines (readLine: up to '\n', a
// trailing '\r' removed).
#ifndef ASL_SHIM_TEXTFILE_H
#define ASL_SHIM_TEXTFILE_H
#include "File.h"
#include <stdarg.h>
namespace asl {
class TextFile : public File {
 public:
  TextFile() {}
  TextFile(const String& name, Mode m = READ) : File(name, m) {}
  TextFile& operator>>(String& tok) {
    std::string s;
    int c;
    while (f_ && (c = fgetc(f_)) != EOF && isspace(c)) {}
    if (f_ && c != EOF) {
      s += (char)c;
      while ((c = fgetc(f_)) != EOF && !isspace(c)) s += (char)c;
      if (c != EOF) ungetc(c, f_);
    }
    tok = String(s);
    return *this;
  }
  bool readLine(String& line) {
    std::string s;
    int c;
    bool any = false;
    while (f_ && (c = fgetc(f_)) != EOF) {
      any = true;
      if (c == '\n') break;
      s += (char)c;
    }
    if (!s.empty() && s.back() == '\r') s.pop_back();
    line = String(s);
    return any;
  }
  String readLine() {
    String l;
    readLine(l);
    return l;
  }
  Array<String> lines() {
    Array<String> out;
    String l;
    while (!end()) {
      readLine(l);
      out << l;
    }
    return out;
  }
  TextFile& operator<<(const String& s) { write(*s, s.length()); return *this; }
  int printf(const char* fmt, ...) {
    if (!f_) return 0;
    va_list ap;
    va_start(ap, fmt);
    int n = vfprintf(f_, fmt, ap);
    va_end(ap);
    return n;
  }
};
}  // namespace asl
#endif
