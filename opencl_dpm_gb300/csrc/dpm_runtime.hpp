// Host-side runtime pieces shared by the 2D and 3D paths.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <atomic>

// A context is shared by the objects created from it: each holds a
// reference, so destroying the context (or the objects) in any order is
// safe; the stream is released with the last reference.
struct dpm_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  std::atomic<int> refs{1};
};

namespace dpm {

const char *last_error();
void ctx_retain(dpm_ctx *ctx);
void ctx_release(dpm_ctx *ctx);

// One device allocation carved into 256-byte aligned arrays.  A batch owns
// its arena; nothing else allocates on the step path.
class DeviceArena {
public:
  DeviceArena() = default;
  DeviceArena(const DeviceArena &) = delete;
  DeviceArena &operator=(const DeviceArena &) = delete;
  ~DeviceArena() {
    if (base_) cudaFree(base_);
  }
  cudaError_t reserve(size_t bytes) {
    cap_ = bytes + 4096;
    return cudaMalloc(&base_, cap_);
  }
  template <typename T> T *take(size_t count) {
    size_t off = (used_ + 255) & ~size_t(255);
    size_t need = off + sizeof(T) * count;
    if (!base_ || need > cap_) {
      ok_ = false;
      return nullptr;
    }
    used_ = need;
    return reinterpret_cast<T *>(static_cast<char *>(base_) + off);
  }
  bool ok() const { return ok_; }
  void *base() const { return base_; }
  size_t used() const { return used_; }
  size_t capacity() const { return cap_; }

private:
  void *base_ = nullptr;
  size_t cap_ = 0, used_ = 0;
  bool ok_ = true;
};

} // namespace dpm
