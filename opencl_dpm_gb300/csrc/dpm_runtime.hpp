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

struct dpm2d_batch;
struct dpm3d_batch;

namespace dpm {

const char *last_error();
void ctx_retain(dpm_ctx *ctx);
void ctx_release(dpm_ctx *ctx);

// ---- slot pools (the server's resident state) ----
// A pool is a batch whose tissues are fixed-capacity slots: a request is
// written into a free slot, runs under a per-tissue step budget inside the
// pool's shared graphs (finished slots freeze in place), and is read back
// and released.  Each pool runs on its own stream.

int pool2d_create(dpm_ctx *ctx, int nslots, int cells_per_slot, int nv_max, dpm2d_batch **out);
int pool2d_assign(dpm2d_batch *b, int slot, int ncells, const unsigned *nv, const float *Ka,
                  const float *Kl, const float *Kb, const float *a0, const float *l0,
                  const float *r0, const float *xy, float L, float Kre, float Kat, int pbc,
                  int nsteps);
int pool2d_run(dpm2d_batch *b, int nsteps, float dt);  // enqueue only
int pool2d_fetch(dpm2d_batch *b, int slot, int ncells, const unsigned *nv, float *xy,
                 float *F);  // synchronizes the pool's stream
int pool2d_release(dpm2d_batch *b, int slot);
int pool2d_sync(dpm2d_batch *b);
size_t pool2d_bytes(const dpm2d_batch *b);
cudaStream_t pool2d_stream(const dpm2d_batch *b);
// Launch over slots [0, nslots) only (the server keeps occupied slots low).
void pool2d_set_active(dpm2d_batch *b, int nslots);

int pool3d_create(dpm_ctx *ctx, int nslots, int cells_per_slot, int nv, int nf,
                  const unsigned *faces, dpm3d_batch **out);
int pool3d_assign(dpm3d_batch *b, int slot, int ncells, const float *Kv, const float *Ka,
                  const float *Ks, const float *v0, const float *a0, const float *l0,
                  const float *Kb, const float *adh, const float *xyz, float L, float Kre,
                  int pbc, int nsteps);
int pool3d_run(dpm3d_batch *b, int nsteps, float dt);
int pool3d_fetch(dpm3d_batch *b, int slot, int ncells, float *xyz, float *F);
int pool3d_release(dpm3d_batch *b, int slot);
int pool3d_sync(dpm3d_batch *b);
size_t pool3d_bytes(const dpm3d_batch *b);
cudaStream_t pool3d_stream(const dpm3d_batch *b);
void pool3d_set_active(dpm3d_batch *b, int nslots);

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
