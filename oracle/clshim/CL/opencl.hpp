// CPU OpenCL host shim: the cl:: C++ wrapper surface the reference uses.
//
// Test infrastructure only.  It lets the reference's own host code
// (src/Tissue2D.cpp:116-241 and src/Tissue3D.cpp:118-522) build and run
// unmodified, with its kernels (shaders/Cell2D_kernel.cl,
// shaders/Cell3D_Kernel.cl) compiled as C++ and executed on the CPU:
//
//  * cl::Buffer       - heap storage shared by all copies of the handle;
//                       CL_MEM_COPY_HOST_PTR copies the host data in.
//  * cl::Program      - keeps the source text; build() checks that the text is
//                       one of the kernel files compiled into this binary
//                       (by checksum), so the program that runs is the one
//                       that was read at run time.
//  * cl::Kernel       - looks the kernel up by name in a registry filled by
//                       the compiled kernel files; setArg() stores the bytes.
//  * enqueueNDRangeKernel runs the kernel serially over the NDRange with
//    dimension 0 fastest.  That gives the reference's kernels their intended
//    race-free reading (a work-group barrier really orders the fi==0 volume
//    write before the other faces read it) and a fixed order for the
//    compare-and-swap float atomics.
//  * enqueueReadBuffer copies out; finish() is a no-op (all work is eager).
#ifndef DPM_CLSHIM_OPENCL_HPP
#define DPM_CLSHIM_OPENCL_HPP

#include "cl.h"

#include <chrono>
#include <cstdint>
#include <cstring>
#include <functional>
#include <initializer_list>
#include <iostream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace cl {

namespace shim {

// One stored kernel argument: either a buffer pointer or up to 16 raw bytes.
struct ArgSlot {
  void *ptr = nullptr;
  unsigned char bytes[16] = {0};
  size_t size = 0;
  bool set = false;
};

using Invoker = void (*)(const ArgSlot *);

struct KernelEntry {
  Invoker invoke = nullptr;
  unsigned nargs = 0;
};

inline std::map<std::string, KernelEntry> &registry() {
  static std::map<std::string, KernelEntry> r;
  return r;
}

inline std::vector<uint64_t> &source_checksums() {
  static std::vector<uint64_t> s;
  return s;
}

// FNV-1a over the source text.
inline uint64_t checksum(const std::string &s) {
  uint64_t h = 1469598103934665603ull;
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

// Work-item state read by get_global_id()/get_global_size() in kernel code.
inline size_t *gid() {
  static thread_local size_t g[3] = {0, 0, 0};
  return g;
}
inline size_t *gsize() {
  static thread_local size_t g[3] = {1, 1, 1};
  return g;
}

struct Registrar {
  Registrar(const char *name, Invoker inv, unsigned nargs) {
    registry()[name] = KernelEntry{inv, nargs};
  }
};
struct SourceRegistrar {
  explicit SourceRegistrar(uint64_t h) { source_checksums().push_back(h); }
};

} // namespace shim

class Platform {
public:
  static Platform getDefault(cl_int *err = nullptr) {
    if (err) *err = CL_SUCCESS;
    return Platform();
  }
};

class Device {
public:
  static Device getDefault(cl_int *err = nullptr) {
    if (err) *err = CL_SUCCESS;
    return Device();
  }
};

class Context {
public:
  Context() = default;
  Context(const std::vector<Device> &, void * = nullptr, void * = nullptr,
          void * = nullptr, cl_int *err = nullptr) {
    if (err) *err = CL_SUCCESS;
  }
};

class Program {
public:
  Program() = default;
  Program(const Context &, const std::string &source, bool = false,
          cl_int *err = nullptr)
      : source_(std::make_shared<std::string>(source)) {
    if (err) *err = CL_SUCCESS;
  }

  cl_int build(const std::vector<Device> &, const char * = nullptr,
               void * = nullptr, void * = nullptr) const {
    if (!source_) return CL_BUILD_PROGRAM_FAILURE;
    uint64_t h = shim::checksum(*source_);
    for (uint64_t k : shim::source_checksums())
      if (k == h) return CL_SUCCESS;
    log_ = "clshim: program source does not match any kernel file compiled "
           "into this binary";
    return CL_BUILD_PROGRAM_FAILURE;
  }

  template <cl_program_build_info name>
  std::string getBuildInfo(const Device &, cl_int *err = nullptr) const {
    if (err) *err = CL_SUCCESS;
    return log_;
  }

private:
  std::shared_ptr<std::string> source_;
  mutable std::string log_;
};

class Buffer {
public:
  Buffer() = default;
  Buffer(const Context &, cl_mem_flags flags, size_t size,
         void *host_ptr = nullptr, cl_int *err = nullptr)
      : data_(std::make_shared<std::vector<unsigned char>>(size, 0)) {
    if ((flags & CL_MEM_COPY_HOST_PTR) && host_ptr)
      std::memcpy(data_->data(), host_ptr, size);
    if (err) *err = CL_SUCCESS;
  }
  void *raw() const { return data_ ? data_->data() : nullptr; }
  size_t size() const { return data_ ? data_->size() : 0; }

private:
  std::shared_ptr<std::vector<unsigned char>> data_;
};

class NDRange {
public:
  NDRange() : dims_(0) {}
  explicit NDRange(size_t a) : dims_(1) { s_[0] = a; }
  NDRange(size_t a, size_t b) : dims_(2) {
    s_[0] = a;
    s_[1] = b;
  }
  NDRange(size_t a, size_t b, size_t c) : dims_(3) {
    s_[0] = a;
    s_[1] = b;
    s_[2] = c;
  }
  size_t dimensions() const { return dims_; }
  size_t operator[](size_t i) const { return i < dims_ ? s_[i] : 1; }

private:
  size_t dims_;
  size_t s_[3] = {1, 1, 1};
};

static const NDRange NullRange;

class Kernel {
public:
  Kernel() = default;
  Kernel(const Program &, const char *name, cl_int *err = nullptr) {
    auto it = shim::registry().find(name);
    if (it == shim::registry().end()) {
      if (err) *err = CL_INVALID_KERNEL_NAME;
      else
        throw std::runtime_error(std::string("clshim: no kernel named ") +
                                 name);
      return;
    }
    entry_ = it->second;
    args_ = std::make_shared<std::vector<shim::ArgSlot>>(entry_.nargs);
    if (err) *err = CL_SUCCESS;
  }

  cl_int setArg(cl_uint index, const Buffer &b) {
    if (!args_ || index >= args_->size()) return CL_INVALID_ARG_INDEX;
    (*args_)[index].ptr = b.raw();
    (*args_)[index].size = sizeof(void *);
    (*args_)[index].set = true;
    return CL_SUCCESS;
  }
  cl_int setArg(cl_uint index, Buffer &b) {
    return setArg(index, static_cast<const Buffer &>(b));
  }

  template <typename T> cl_int setArg(cl_uint index, const T &value) {
    static_assert(sizeof(T) <= 16, "scalar kernel argument too large");
    if (!args_ || index >= args_->size()) return CL_INVALID_ARG_INDEX;
    shim::ArgSlot &s = (*args_)[index];
    std::memset(s.bytes, 0, sizeof(s.bytes));
    std::memcpy(s.bytes, &value, sizeof(T));
    s.size = sizeof(T);
    s.set = true;
    return CL_SUCCESS;
  }

  void run(const NDRange &global) const {
    if (!entry_.invoke) throw std::runtime_error("clshim: empty kernel");
    for (const auto &a : *args_)
      if (!a.set) throw std::runtime_error("clshim: kernel argument not set");
    size_t g0 = global[0], g1 = global[1], g2 = global[2];
    size_t *gs = shim::gsize();
    size_t *id = shim::gid();
    gs[0] = g0;
    gs[1] = g1;
    gs[2] = g2;
    for (size_t k = 0; k < g2; ++k)
      for (size_t j = 0; j < g1; ++j)
        for (size_t i = 0; i < g0; ++i) {
          id[0] = i;
          id[1] = j;
          id[2] = k;
          entry_.invoke(args_->data());
        }
  }

private:
  shim::KernelEntry entry_;
  std::shared_ptr<std::vector<shim::ArgSlot>> args_;
};

class CommandQueue {
public:
  CommandQueue() = default;
  CommandQueue(const Context &, const Device &,
               cl_command_queue_properties = 0, cl_int *err = nullptr) {
    if (err) *err = CL_SUCCESS;
  }

  cl_int enqueueNDRangeKernel(const Kernel &k, const NDRange &,
                              const NDRange &global,
                              const NDRange & = NullRange, void * = nullptr,
                              void * = nullptr) const {
    k.run(global);
    return CL_SUCCESS;
  }

  cl_int enqueueReadBuffer(const Buffer &b, cl_int, size_t offset, size_t size,
                           void *ptr, void * = nullptr,
                           void * = nullptr) const {
    if (offset + size > b.size()) return CL_INVALID_VALUE;
    std::memcpy(ptr, static_cast<unsigned char *>(b.raw()) + offset, size);
    return CL_SUCCESS;
  }

  cl_int enqueueWriteBuffer(const Buffer &b, cl_int, size_t offset,
                            size_t size, const void *ptr, void * = nullptr,
                            void * = nullptr) const {
    if (offset + size > b.size()) return CL_INVALID_VALUE;
    std::memcpy(static_cast<unsigned char *>(b.raw()) + offset, ptr, size);
    return CL_SUCCESS;
  }

  cl_int finish() const { return CL_SUCCESS; }
};

} // namespace cl

#endif
