// OpenCL C prelude for compiling OpenCL kernel text as C++ on the CPU.
//
// Test infrastructure only.  It supplies the OpenCL C built-ins that the
// reference kernels (shaders/Cell2D_kernel.cl, shaders/Cell3D_Kernel.cl) use,
// with the semantics of the OpenCL C specification:
//
//  * float2 (8 bytes) and float3/uint3 (16 bytes, like float4) with
//    component-wise arithmetic and scalar broadcast;
//  * float overloads of sqrt/floor/round/fabs/atan2 that return float, so a
//    float argument stays float while a double literal in an expression
//    promotes it to double, as on an fp64-capable OpenCL device;
//  * dot/cross/length/distance/normalize (normalize of an all-zero vector
//    returns that vector, the specification's special case);
//  * get_global_id/get_global_size, served by the host shim;
//  * barrier() is a no-op and atomic_cmpxchg is a plain compare-and-swap,
//    because the shim runs work-items one at a time.
// Sums are evaluated left to right ((x + y) + z), cross products in the
// textbook component order.  Compile with -ffp-contract=off so that no
// multiply-add is fused.
#ifndef DPM_CLC_PRELUDE_HPP
#define DPM_CLC_PRELUDE_HPP

#include <CL/opencl.hpp>
#include <math.h>

#include <type_traits>
#include <utility>

typedef unsigned int uint;

#define __kernel
#define __global
#define __local
#define __private
#define constant static const
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
#define M_PI_F ((float)3.14159265358979323846)

namespace clc {

inline size_t get_global_id(uint d) { return d < 3 ? cl::shim::gid()[d] : 0; }
inline size_t get_global_size(uint d) {
  return d < 3 ? cl::shim::gsize()[d] : 1;
}
inline void barrier(int) {}

inline int atomic_cmpxchg(volatile int *p, int cmp, int val) {
  int old = *p;
  if (old == cmp) *p = val;
  return old;
}

inline float sqrt(float a) { return ::sqrtf(a); }
inline double sqrt(double a) { return ::sqrt(a); }
inline float floor(float a) { return ::floorf(a); }
inline double floor(double a) { return ::floor(a); }
inline float round(float a) { return ::roundf(a); }
inline double round(double a) { return ::round(a); }
inline float fabs(float a) { return ::fabsf(a); }
inline double fabs(double a) { return ::fabs(a); }
inline float atan2(float y, float x) { return ::atan2f(y, x); }

struct float2 {
  float x, y;
  float2() : x(0.0f), y(0.0f) {}
  float2(float s) : x(s), y(s) {}
  float2(float a, float b) : x(a), y(b) {}
  float2 &operator+=(const float2 &o) {
    x += o.x;
    y += o.y;
    return *this;
  }
  float2 &operator-=(const float2 &o) {
    x -= o.x;
    y -= o.y;
    return *this;
  }
};
static_assert(sizeof(float2) == 8, "float2 must be 8 bytes");

inline float2 operator+(float2 a, float2 b) { return float2(a.x + b.x, a.y + b.y); }
inline float2 operator-(float2 a, float2 b) { return float2(a.x - b.x, a.y - b.y); }
inline float2 operator*(float2 a, float2 b) { return float2(a.x * b.x, a.y * b.y); }
inline float2 operator/(float2 a, float2 b) { return float2(a.x / b.x, a.y / b.y); }
inline float2 operator*(float s, float2 a) { return float2(s * a.x, s * a.y); }
inline float2 operator*(float2 a, float s) { return float2(a.x * s, a.y * s); }
inline float2 operator/(float2 a, float s) { return float2(a.x / s, a.y / s); }
inline float2 round(float2 a) { return float2(round(a.x), round(a.y)); }
inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
inline float length(float2 a) { return sqrt(dot(a, a)); }
inline float2 normalize(float2 a) {
  float l2 = dot(a, a);
  if (l2 == 0.0f) return a;
  return a / sqrt(l2);
}

struct alignas(16) float3 {
  float x, y, z, w;
  float3() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
  float3(float s) : x(s), y(s), z(s), w(0.0f) {}
  float3(float a, float b, float c) : x(a), y(b), z(c), w(0.0f) {}
  float3 &operator+=(const float3 &o) {
    x += o.x;
    y += o.y;
    z += o.z;
    return *this;
  }
  float3 &operator-=(const float3 &o) {
    x -= o.x;
    y -= o.y;
    z -= o.z;
    return *this;
  }
  float3 &operator*=(float s) {
    x *= s;
    y *= s;
    z *= s;
    return *this;
  }
};
static_assert(sizeof(float3) == 16, "float3 must be 16 bytes");

inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(float3 a, float3 b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator*(float s, float3 a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator/(float3 a, float s) { return float3(a.x / s, a.y / s, a.z / s); }
inline float3 round(float3 a) { return float3(round(a.x), round(a.y), round(a.z)); }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 cross(float3 a, float3 b) {
  return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z,
                a.x * b.y - a.y * b.x);
}
inline float length(float3 a) { return sqrt(dot(a, a)); }
inline float distance(float3 a, float3 b) { return length(a - b); }
inline float3 normalize(float3 a) {
  float l2 = dot(a, a);
  if (l2 == 0.0f) return a;
  return a / sqrt(l2);
}

struct alignas(16) uint3 {
  uint x, y, z, w;
};
static_assert(sizeof(uint3) == 16, "uint3 must be 16 bytes");

// Typed view of one stored kernel argument.
template <typename T> inline T arg_as(const cl::shim::ArgSlot &s) {
  if constexpr (std::is_pointer_v<T>) {
    return reinterpret_cast<T>(s.ptr);
  } else {
    T v;
    std::memcpy(&v, s.bytes, sizeof(T));
    return v;
  }
}

template <typename... A, size_t... I>
inline void call_with(void (*f)(A...), const cl::shim::ArgSlot *s,
                      std::index_sequence<I...>) {
  f(arg_as<A>(s[I])...);
}

template <typename... A>
constexpr unsigned arity(void (*)(A...)) {
  return sizeof...(A);
}

template <typename... A>
inline void call(void (*f)(A...), const cl::shim::ArgSlot *s) {
  call_with(f, s, std::index_sequence_for<A...>{});
}

} // namespace clc

// Register kernel NAME (defined in namespace NS) with the shim.  The kernel
// text itself is compiled inside a namespace nested in clc, so that its
// unqualified calls (sqrt, round, dot, ...) resolve to the built-ins above and
// never to the C library's double versions.
#define CLSHIM_REGISTER(NS, NAME)                                              \
  static cl::shim::Registrar clshim_reg_##NAME(                                \
      #NAME, [](const cl::shim::ArgSlot *s) { clc::call(&NS::NAME, s); },      \
      clc::arity(&NS::NAME));

#endif
