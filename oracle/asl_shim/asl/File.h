// From-scratch stand-in for asl/File.h (see defs.h): a binary file.  Scalars
// and strings written with << are raw bytes (little-endian scalars, strings
// without terminator); read<T>() reads sizeof(T) raw bytes.
#ifndef ASL_SHIM_FILE_H
#define ASL_SHIM_FILE_H
#include "defs.h"
#include "String.h"
namespace asl {
class File {
 protected:
  FILE* f_ = nullptr;
  bool own_ = false;
  String name_;
 public:
  enum Mode { READ, WRITE, APPEND };
  File() {}
  File(const String& name, Mode m = READ) : name_(name) { open(name, m); }
  ~File() { close(); }
  File(const File&) = delete;
  File& operator=(const File&) = delete;
  bool open(const String& name, Mode m) {
    close();
    name_ = name;
    f_ = fopen(*name, m == READ ? "rb" : m == WRITE ? "wb" : "ab");
    own_ = true;
    return f_ != nullptr;
  }
  void use(FILE* f) { close(); f_ = f; own_ = false; }
  void close() {
    if (f_ && own_) fclose(f_);
    f_ = nullptr;
  }
  explicit operator bool() const { return f_ != nullptr; }
  bool operator!() const { return f_ == nullptr; }
  int read(void* p, int n) { return f_ ? (int)fread(p, 1, (size_t)n, f_) : 0; }
  template <class T> T read() {
    T x{};
    read(&x, (int)sizeof(T));
    return x;
  }
  int write(const void* p, int n) { return f_ ? (int)fwrite(p, 1, (size_t)n, f_) : 0; }
  bool seek(long pos) { return f_ && fseek(f_, pos, SEEK_SET) == 0; }
  bool end() {
    if (!f_) return true;
    int c = fgetc(f_);
    if (c == EOF) return true;
    ungetc(c, f_);
    return false;
  }
  long size() {
    FILE* g = fopen(*name_, "rb");
    if (!g) return 0;
    fseek(g, 0, SEEK_END);
    long s = ftell(g);
    fclose(g);
    return s;
  }
  Array<byte> firstBytes(int n) {
    Array<byte> out;
    FILE* g = fopen(*name_, "rb");
    if (!g) return out;
    out.resize(n);
    int k = (int)fread(out.ptr(), 1, (size_t)n, g);
    fclose(g);
    out.resize(k);
    return out;
  }
  File& operator<<(const String& s) { write(*s, s.length()); return *this; }
  File& operator<<(int v) { write(&v, 4); return *this; }
  File& operator<<(const Array<byte>& b) { write(b.ptr(), b.length()); return *this; }
};
}  // namespace asl
#endif
