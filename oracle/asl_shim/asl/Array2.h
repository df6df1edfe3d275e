// From-scratch stand-in for asl/Array2.h (see defs.h): a dense row-major
// rows x cols matrix, element (i,j) = row i, column j.
#ifndef ASL_SHIM_ARRAY2_H
#define ASL_SHIM_ARRAY2_H
#include "defs.h"
#include <vector>
namespace asl {
template <class T>
class Array2 {
  std::vector<T> v_;
  int rows_ = 0, cols_ = 0;
 public:
  Array2() {}
  Array2(int rows, int cols) : v_((size_t)rows * cols), rows_(rows), cols_(cols) {}
  void resize(int rows, int cols) { v_.resize((size_t)rows * cols); rows_ = rows; cols_ = cols; }
  void set(const T& x) { for (auto& e : v_) e = x; }
  int rows() const { return rows_; }
  int cols() const { return cols_; }
  T& operator()(int i, int j) { return v_[(size_t)i * cols_ + j]; }
  const T& operator()(int i, int j) const { return v_[(size_t)i * cols_ + j]; }
  T* data() { return v_.data(); }
  const T* data() const { return v_.data(); }
};
}  // namespace asl
#endif
