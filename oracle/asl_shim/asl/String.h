// From-scratch stand-in for asl/String.h (see defs.h): only storage.
#ifndef ASL_SHIM_STRING_H
#define ASL_SHIM_STRING_H
#include "defs.h"
#include <string>
namespace asl {
class String {
  std::string s_;
 public:
  String() {}
  String(const char* s) : s_(s) {}
  const char* operator*() const { return s_.c_str(); }
};
}  // namespace asl
#endif
