// From-scratch stand-in for asl/Path.h (see defs.h): '/'-separated paths.
//   directory()        everything before the last '/' ("" if none)
//   hasExtension(e)    the text after the last '.' of the file name equals e, ignoring case
//   noExt()            the path without the file name's extension
#ifndef ASL_SHIM_PATH_H
#define ASL_SHIM_PATH_H
#include "defs.h"
#include "String.h"
#include <strings.h>
namespace asl {
class Path {
  std::string p_;
  size_t name_start() const {
    size_t s = p_.rfind('/');
    return s == std::string::npos ? 0 : s + 1;
  }
  size_t dot() const {
    size_t d = p_.rfind('.');
    return (d == std::string::npos || d < name_start()) ? std::string::npos : d;
  }
 public:
  Path(const String& s) : p_(s.str()) {}
  Path(const char* s) : p_(s) {}
  String directory() const {
    size_t s = p_.rfind('/');
    return s == std::string::npos ? String("") : String(p_.substr(0, s));
  }
  bool hasExtension(const char* e) const {
    size_t d = dot();
    return d != std::string::npos && strcasecmp(p_.c_str() + d + 1, e) == 0;
  }
  String noExt() const {
    size_t d = dot();
    return String(d == std::string::npos ? p_ : p_.substr(0, d));
  }
  String string() const { return String(p_); }
};
}  // namespace asl
#endif
