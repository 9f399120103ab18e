// Shared definitions of the GB300 DPM library: error reporting, device
// layouts and small device helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/dpm_gb300.h"

namespace dpm {

// ---- error reporting (thread-local message, int status) ----
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define DPM_CUDA_TRY(expr)                                                     \
  do {                                                                         \
    cudaError_t _e = (expr);                                                   \
    if (_e != cudaSuccess) return ::dpm::cuda_fail(_e, #expr);                 \
  } while (0)

// ---- 2D device layouts ----

// Per-cell constants of a 2D cell (48 bytes).  The derived spring constants
// are formed on the host with the reference's float operations:
// kA = Ka / sqrtf(a0) (Cell2D_kernel.cl:38), kL = Kl * sqrtf(a0 / l0)
// (Cell2D_kernel.cl:118).
struct alignas(16) Cell2D {
  uint32_t voff;   // first vertex of the cell
  uint32_t nv;     // vertices
  uint32_t tissue; // owning tissue
  uint32_t pad0;
  float a0, l0, kA, kL;
  float Kb, r0;
  float inv_l0;  // 1 / l0
  float inv_2r0; // 1 / (2 r0)
};

// Per-tissue constants and cell-list state of a 2D tissue (80 bytes).
struct alignas(16) Tissue2D {
  float L, Kre, Kat, l0max;  // l0max: largest l0 (attraction range)
  int pbc;
  int cell_begin, cell_end;  // active cells [begin, end) in batch cell order
  int cap;                   // upper bound on bins per axis
  float skin;                // neighbour-list skin (absolute)
  float binw;                // bin width of the last rebuild
  int nbx, nby;              // bins per axis of the last rebuild
  float gminx, gmaxx, gminy, gmaxy; // raw extent at the last rebuild
  int cell_cap;   // end of the tissue's cell slots (>= cell_end)
  int steps_left; // step budget; each rebuild takes run_now steps from it
  int run_now;    // steps of the current rebuild period this tissue runs
  int pad;
};

// A step budget that never runs out (ordinary batches).
constexpr int kStepsUnlimited = 0x3fffffff;

// Per-cell geometry at the current positions: circle (centre, radius)
// around the vertices, the cell area, and the axis-aligned box.
struct alignas(16) Geom2D {
  float cx, cy, R, area;
  float minx, maxx, miny, maxy;
};

constexpr int kMaxNV2D = 256;    // vertices per 2D cell
constexpr int kMaxNB2D = 96;     // neighbour-list capacity per 2D cell
constexpr int kNbOverflow = -1;  // neighbour count meaning "scan the tissue"
constexpr int kLocalBinBits = 20; // key = tissue << 20 | local bin
constexpr int kMaxBinsAxis = 1024;

// ---- 3D ----
constexpr int kMaxNV3D = 642; // subdivision 3
// Per-cell constants of a 3D cell (48 bytes).  sa_scale is the surface
// spring prefactor Ka*sqrtf(a0)/l0*0.3f formed in the reference's order
// (Cell3D_Kernel.cl:167); adh is the adhesion range (2*l0 unless set).
struct alignas(16) Cell3D {
  float Kv, Ka, Ks, v0;
  float a0, l0, Kb, adh;
  float sa_scale;
  uint32_t tissue;
  uint32_t active; // 0: an empty slot
  uint32_t pad1;
};
struct alignas(16) Tissue3D {
  float L, Kre, skin, binw;
  int pbc, cell_begin, cell_end, cap; // active cells [begin, end)
  int nb, cell_cap, steps_left, run_now;
  // AllVertAttraction (opt-in; the reference's step loop never runs it):
  // strength, and the pair range it needs (2 * largest l0, 0 when off)
  float Kat, arange;
  int pad0, pad1;
};
// Centre of mass, largest vertex distance from it, and the longest mesh
// edge (the reference's winding sum drops faces whose denominator is below
// 1e-8, which happens only within ~0.77 * longest edge of a face, so points
// up to R + emax from the centre can get a non-zero winding number).
// rin > 0: the mesh winds exactly `wind` (+1 or -1, the sign of the
// reference's face terms) times around every point closer than rin to the
// centre; rin = 0: no such ball is known.
struct alignas(16) Geom3D {
  float cx, cy, cz, R;
  float emax, rin, wind, pad0;
};
constexpr int kMaxNB3D = 64;

// ---- device helpers ----
#ifdef __CUDACC__
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Warp-wide float max/min in one instruction (redux.sync .f32, sm_100a and
// later): the same value as a shuffle tree of fmaxf/fminf (NaN inputs
// ignored, -0 below +0), since a maximum does not depend on the order.
__device__ __forceinline__ float warp_max(float v) {
  float r;
  asm("redux.sync.max.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
  return r;
}
__device__ __forceinline__ float warp_min(float v) {
  float r;
  asm("redux.sync.min.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
  return r;
}
__device__ __forceinline__ int warp_sum_i(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// x - L*floor(x/L), with each operation rounded separately.
__device__ __forceinline__ float wrap_rn(float x, float L) {
  return __fsub_rn(x, __fmul_rn(L, floorf(__fdiv_rn(x, L))));
}
#endif

} // namespace dpm
