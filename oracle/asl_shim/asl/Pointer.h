// From-scratch stand-in for asl/Pointer.h (see defs.h): Shared<T>, a
// reference-counted owner built on std::shared_ptr that converts from a raw
// pointer, from nullptr/NULL and from Shared<Derived>.
#ifndef ASL_SHIM_POINTER_H
#define ASL_SHIM_POINTER_H
#include "defs.h"
#include <memory>
namespace asl {
template <class T>
class Shared {
  template <class U> friend class Shared;
  std::shared_ptr<T> p_;
 public:
  Shared() {}
  Shared(T* p) : p_(p) {}
  template <class U> Shared(const Shared<U>& o) : p_(o.p_) {}
  T* operator->() const { return p_.get(); }
  T& operator*() const { return *p_; }
  T* ptr() const { return p_.get(); }
  explicit operator bool() const { return (bool)p_; }
  bool operator!() const { return !p_; }
};
}  // namespace asl
#endif
