// Checkpoint files of 2D and 3D batches: an 8-byte magic, a version and the
// dimension, then raw native-endian arrays in a fixed order (see
// dpm2d_save / dpm3d_save).
#pragma once

#include <cstdio>
#include <cstring>

namespace dpm {

constexpr char kCkptMagic[8] = {'D', 'P', 'M', 'C', 'K', 'P', 'T', '\0'};
constexpr unsigned kCkptVersion = 1;

class CkptFile {
public:
  CkptFile(const char *path, const char *mode) : f_(path ? std::fopen(path, mode) : nullptr) {}
  ~CkptFile() {
    if (f_) std::fclose(f_);
  }
  CkptFile(const CkptFile &) = delete;
  CkptFile &operator=(const CkptFile &) = delete;
  bool open() const { return f_ != nullptr; }
  bool ok() const { return f_ && ok_; }
  template <typename T> void put(const T *p, size_t n) {
    if (ok() && n && std::fwrite(p, sizeof(T), n, f_) != n) ok_ = false;
  }
  template <typename T> void put1(const T &v) { put(&v, 1); }
  template <typename T> void get(T *p, size_t n) {
    if (ok() && n && std::fread(p, sizeof(T), n, f_) != n) ok_ = false;
  }
  // reads n items if they are there; false (and nothing changed) at the end
  // of the file, for optional trailing sections
  template <typename T> bool try_get(T *p, size_t n) {
    return ok() && n && std::fread(p, sizeof(T), n, f_) == n;
  }
  template <typename T> T get1() {
    T v{};
    get(&v, 1);
    return v;
  }
  // header: magic, version, dimension; false if the file is not a
  // checkpoint of that dimension
  void put_header(unsigned dim) {
    put(kCkptMagic, 8);
    put1(kCkptVersion);
    put1(dim);
  }
  bool get_header(unsigned dim) {
    char m[8];
    get(m, 8);
    const unsigned v = get1<unsigned>(), d = get1<unsigned>();
    return ok() && std::memcmp(m, kCkptMagic, 8) == 0 && v == kCkptVersion && d == dim;
  }
  int close() {
    int r = 0;
    if (f_) r = std::fclose(f_);
    f_ = nullptr;
    return r;
  }

private:
  FILE *f_;
  bool ok_ = true;
};

} // namespace dpm
