// From-scratch stand-in for asl/Array.h (see defs.h): a growable array with
// value semantics (the checked sources never mutate a copy after taking it,
// except after dup(), which is then a no-op).
#ifndef ASL_SHIM_ARRAY_H
#define ASL_SHIM_ARRAY_H
#include "defs.h"
#include <vector>
namespace asl {
template <class T>
class Array {
  std::vector<T> v_;
 public:
  Array() {}
  explicit Array(int n) : v_(n) {}
  Array(int n, const T& x) : v_(n, x) {}
  template <class U> Array(const Array<U>& o) {  // element-wise conversion
    v_.reserve(o.length());
    for (int i = 0; i < o.length(); i++) v_.push_back((T)o[i]);
  }
  int length() const { return (int)v_.size(); }
  Array& resize(int n) { v_.resize(n); return *this; }
  void reserve(int n) { v_.reserve(n); }
  void clear() { v_.clear(); }
  void dup() {}
  Array clone() const { return *this; }
  bool operator!() const { return v_.empty(); }
  explicit operator bool() const { return !v_.empty(); }
  T& operator[](int i) { return v_[i]; }
  const T& operator[](int i) const { return v_[i]; }
  Array& operator<<(const T& x) { v_.push_back(x); return *this; }
  T* ptr() { return v_.data(); }
  const T* ptr() const { return v_.data(); }
  typename std::vector<T>::iterator begin() { return v_.begin(); }
  typename std::vector<T>::iterator end() { return v_.end(); }
  typename std::vector<T>::const_iterator begin() const { return v_.begin(); }
  typename std::vector<T>::const_iterator end() const { return v_.end(); }
};
typedef Array<byte> ByteArray;
}  // namespace asl
#endif
