// From-scratch stand-in for asl/StreamBuffer.h (see defs.h): little-endian
// binary packing of scalars into a byte buffer, and reading them back.
#ifndef ASL_SHIM_STREAMBUFFER_H
#define ASL_SHIM_STREAMBUFFER_H
#include "defs.h"
#include "Array.h"
#include <string.h>
namespace asl {
class StreamBuffer {
  Array<byte> b_;
  template <class T> StreamBuffer& put(T v) {
    const byte* p = (const byte*)&v;
    for (size_t i = 0; i < sizeof(T); i++) b_ << p[i];
    return *this;
  }
 public:
  StreamBuffer& operator<<(float v) { return put(v); }
  StreamBuffer& operator<<(short v) { return put(v); }
  StreamBuffer& operator<<(int v) { return put(v); }
  int length() const { return b_.length(); }
  void clear() { b_.clear(); }
  const Array<byte>& operator*() const { return b_; }
};
class StreamBufferReader {
  const byte* p_;
  int n_, i_ = 0;
 public:
  StreamBufferReader(const Array<byte>& b) : p_(b.ptr()), n_(b.length()) {}
  template <class T> StreamBufferReader& operator>>(T& v) {
    if (i_ + (int)sizeof(T) <= n_) memcpy(&v, p_ + i_, sizeof(T));
    i_ += (int)sizeof(T);
    return *this;
  }
  void skip(int n) { i_ += n; }
};
}  // namespace asl
#endif
