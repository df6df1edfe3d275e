// From-scratch stand-in for asl/Array.h (see defs.h): a growable array with
// value semantics (the checked sources never mutate a copy after taking it).
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
  int length() const { return (int)v_.size(); }
  void resize(int n) { v_.resize(n); }
  void reserve(int n) { v_.reserve(n); }
  void clear() { v_.clear(); }
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
}  // namespace asl
#endif
