// Dispersion of cell centres on the device: the soft-disc relaxation that
// Tissue2D::Disperse (src/Tissue2D.cpp:42-114) and Tissue3D::Disperse2D
// (src/Tissue3D.cpp:40-116) run on the host before a simulation, for many
// independent systems at once (one thread block per system, the whole
// relaxation loop inside one launch).
//
// Bit-exact with the reference.  Per iteration the reference loops over all
// ordered pairs (i, j), i outer, and for a pair in contact subtracts the
// pair force from F[i] and adds it to F[j]; the energy U is one float sum in
// that same order.  Because the wrapped offset of (j, i) is exactly the
// negation of that of (i, j), cell k's force is the float sum, in order, of
// -f(k, j) over its contacts j < k, then over all its contacts, then over its
// contacts j > k (rows i < k add to F[k] before row k, rows i > k after).
// Each thread folds that sequence for its cells, every operation rounded as
// in the reference (float, with the reference's double sub-expressions);
// one thread then adds the U terms in row order.  Contacts come from
// per-cell lists of the cells within the contact distance plus a skin,
// rebuilt when some centre has moved by half the skin, and kept in
// ascending order; the contact test itself is the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "dpm_common.cuh"
#include "dpm_runtime.hpp"

namespace dpm {
namespace {

constexpr int kDispThreads = 256;
constexpr int kDispMaxNb = 48;       // list capacity per cell (more: scan all)
constexpr int kDispMaxCells = 4096;  // per system (shared-memory staging)
constexpr int kDispMaxIter = 100000; // the reference's cap (count > 1e5)

struct DisperseArgs {
  const int *begin;    // [nsys + 1] first cell of each system
  const float *radius; // [ncells]
  const float *L;      // [nsys]
  float *X, *Y;        // [ncells] in: start; out: relaxed
  int *count;          // [nsys] iterations run
  int *nb;             // [ncells * kDispMaxNb] contact candidates, ascending
  int *nn;             // [ncells] candidate count, -1: scan every cell
  float *inner;        // [ncells * kDispMaxNb] U terms of each row's contacts
};

// The reference's wrapped offset from (xi, yi) to (xj, yj), distance, and
// contact test dist <= ri + rj.
__device__ __forceinline__ bool contact(float xi, float yi, float ri, float xj, float yj,
                                        float rj, float L, float &dx, float &dy, float &dist) {
  dx = __fsub_rn(xj, xi);
  dx = __double2float_rn(
      __dsub_rn((double)dx, __dmul_rn((double)L, round((double)__fdiv_rn(dx, L)))));
  dy = __fsub_rn(yj, yi);
  dy = __double2float_rn(
      __dsub_rn((double)dy, __dmul_rn((double)L, round((double)__fdiv_rn(dy, L)))));
  dist = __double2float_rn(__dsqrt_rn((double)__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy))));
  return dist <= __fadd_rn(ri, rj);
}

// Pair force (fx, fy) of the reference for a pair in contact.
__device__ __forceinline__ void pair_force(float dx, float dy, float dist, float ri, float rj,
                                           float &fx, float &fy) {
  const float ux = __fdiv_rn(dx, dist), uy = __fdiv_rn(dy, dist);
  const float s = __fadd_rn(ri, rj);
  const float q = __fdiv_rn(dist, s);
  const float ftmp = __double2float_rn(__ddiv_rn(__dsub_rn(1.0, (double)q), (double)s));
  fx = __fmul_rn(ftmp, ux);
  fy = __fmul_rn(ftmp, uy);
}

// The reference's energy term 1 - q (1 - q), q = dist / (ri + rj), in float.
__device__ __forceinline__ float u_term(float dist, float ri, float rj) {
  const float q = __fdiv_rn(dist, __fadd_rn(ri, rj));
  return __fsub_rn(1.0f, __fmul_rn(q, __fsub_rn(1.0f, q)));
}

__global__ void __launch_bounds__(kDispThreads) k_disperse(DisperseArgs a) {
  extern __shared__ float sm[];
  __shared__ int s_rebuild, s_stop;
  const int sys = blockIdx.x;
  const int c0 = a.begin[sys], n = a.begin[sys + 1] - c0;
  const float L = a.L[sys];
  float *X = sm, *Y = X + n, *X0 = Y + n, *Y0 = X0 + n, *R = Y0 + n;
  const int tid = threadIdx.x;
  float rmin = INFINITY;
  for (int k = tid; k < n; k += kDispThreads) {
    X[k] = a.X[c0 + k];
    Y[k] = a.Y[c0 + k];
    R[k] = a.radius[c0 + k];
    rmin = fminf(rmin, R[k]);
  }
  // skin of the contact lists: a fraction of the smallest radius
  __shared__ float s_red[kDispThreads / 32];
  rmin = warp_min(rmin);
  if ((tid & 31) == 0) s_red[tid >> 5] = rmin;
  if (tid == 0) {
    s_rebuild = 1;
    s_stop = 0;
  }
  __syncthreads();
  float skin = INFINITY;
  for (int w = 0; w < kDispThreads / 32; ++w) skin = fminf(skin, s_red[w]);
  skin *= 0.5f;
  int *nb = a.nb + (size_t)c0 * kDispMaxNb, *nn = a.nn + c0;
  float *inner = a.inner + (size_t)c0 * kDispMaxNb;

  float oldU = 100.0f;
  int count = 0;
  for (;;) {
    // contact lists (conservative: every pair within the contact distance
    // plus the skin; centres move by at most skin/2 before the next rebuild)
    if (s_rebuild) {
      for (int k = tid; k < n; k += kDispThreads) {
        const float xk = X[k], yk = Y[k], rk = R[k];
        int m = 0;
        for (int j = 0; j < n && m >= 0; ++j) {
          if (j == k) continue;
          float dx, dy, dist;
          contact(xk, yk, rk, X[j], Y[j], R[j], L, dx, dy, dist);
          if (dist <= __fadd_rn(__fadd_rn(rk, R[j]), skin)) {
            if (m < kDispMaxNb) nb[(size_t)k * kDispMaxNb + m++] = j;
            else m = -1;
          }
        }
        nn[k] = m;
        X0[k] = xk;
        Y0[k] = yk;
      }
      __syncthreads();
      if (tid == 0) s_rebuild = 0;
    }
    __syncthreads();

    // forces of this iteration, folded in the reference's order
    float fxk[(kDispMaxCells + kDispThreads - 1) / kDispThreads];
    float fyk[(kDispMaxCells + kDispThreads - 1) / kDispThreads];
#pragma unroll 1
    for (int t = 0, k = tid; k < n; ++t, k += kDispThreads) {
      const float xk = X[k], yk = Y[k], rk = R[k];
      const int m = nn[k];
      const int *lst = nb + (size_t)k * kDispMaxNb;
      const int cnt = m < 0 ? n : m;
      float Fx = 0.0f, Fy = 0.0f;
      // segment 1: contacts j < k; segment 2: all contacts (storing the U
      // terms of row k); segment 3: contacts j > k
      for (int seg = 0; seg < 3; ++seg) {
        int u = 0;
        for (int p = 0; p < cnt; ++p) {
          const int j = m < 0 ? p : lst[p];
          if (j == k) continue;
          if (seg == 0 && j > k) break;
          if (seg == 2 && j < k) continue;
          float dx, dy, dist;
          if (!contact(xk, yk, rk, X[j], Y[j], R[j], L, dx, dy, dist)) continue;
          float fx, fy;
          pair_force(dx, dy, dist, rk, R[j], fx, fy);
          Fx = __fsub_rn(Fx, fx);
          Fy = __fsub_rn(Fy, fy);
          if (seg == 1 && m >= 0) inner[(size_t)k * kDispMaxNb + u++] = u_term(dist, rk, R[j]);
        }
        if (seg == 1 && m >= 0) nn[k] = m | (u << 16);
      }
      fxk[t] = Fx;
      fyk[t] = Fy;
    }
    __syncthreads();

    // U in row order (one thread), positions (every thread)
    if (tid == 0) {
      float U = 0.0f;
      for (int k = 0; k < n; ++k) {
        const int m = nn[k];
        if (m >= 0) {
          const int u = m >> 16;
          for (int p = 0; p < u; ++p)
            U = __double2float_rn(
                __dadd_rn((double)U, __dmul_rn(0.5, (double)inner[(size_t)k * kDispMaxNb + p])));
        } else {
          for (int j = 0; j < n; ++j) {
            if (j == k) continue;
            float dx, dy, dist;
            if (!contact(X[k], Y[k], R[k], X[j], Y[j], R[j], L, dx, dy, dist)) continue;
            U = __double2float_rn(
                __dadd_rn((double)U, __dmul_rn(0.5, (double)u_term(dist, R[k], R[j]))));
          }
        }
      }
      float dU = __fsub_rn(U, oldU);
      if (dU < 0.0f) dU = -dU;
      oldU = U;
      ++count;
      s_stop = !((double)dU > 1e-6) || count > kDispMaxIter;
    }
    __syncthreads();
    bool moved = false;
#pragma unroll 1
    for (int t = 0, k = tid; k < n; ++t, k += kDispThreads) {
      X[k] = __double2float_rn(__dadd_rn((double)X[k], __dmul_rn(0.01, (double)fxk[t])));
      Y[k] = __double2float_rn(__dadd_rn((double)Y[k], __dmul_rn(0.01, (double)fyk[t])));
      const float d = fabsf(X[k] - X0[k]) + fabsf(Y[k] - Y0[k]);
      moved |= !(d <= 0.5f * skin);
      if (nn[k] >= 0) nn[k] &= 0xffff;
    }
    const bool any = __syncthreads_or(moved) != 0;
    if (tid == 0 && any) s_rebuild = 1;
    __syncthreads();
    if (s_stop) break;
  }
  for (int k = tid; k < n; k += kDispThreads) {
    a.X[c0 + k] = X[k];
    a.Y[c0 + k] = Y[k];
  }
  if (tid == 0) a.count[sys] = count;
}

} // namespace
} // namespace dpm

using namespace dpm;

extern "C" int dpm_disperse(dpm_ctx *ctx, int nsystems, const int *ncells, const float *radius,
                            const float *L, float *X, float *Y, int *iterations) {
  if (!ctx || !ncells || !radius || !L || !X || !Y) return fail(DPM_EINVAL, "null argument");
  if (nsystems <= 0) return fail(DPM_EINVAL, "no systems");
  std::vector<int> begin(nsystems + 1, 0);
  int nmax = 0;
  for (int s = 0; s < nsystems; ++s) {
    if (ncells[s] < 1) return fail(DPM_EINVAL, "a system needs at least one cell");
    if (ncells[s] > kDispMaxCells) return fail(DPM_ECAPACITY, "more than 4096 cells in a system");
    if (!(L[s] > 0.0f) || !std::isfinite(L[s])) return fail(DPM_EINVAL, "L must be positive");
    begin[s + 1] = begin[s] + ncells[s];
    nmax = std::max(nmax, ncells[s]);
  }
  const size_t N = (size_t)begin[nsystems];
  for (size_t i = 0; i < N; ++i)
    if (!(radius[i] > 0.0f)) return fail(DPM_EINVAL, "radii must be positive");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  DeviceArena A;
  DPM_CUDA_TRY(A.reserve(sizeof(int) * (nsystems + 1) + sizeof(float) * (4 * N + nsystems) +
                         sizeof(int) * (nsystems + N) +
                         (sizeof(int) + sizeof(float)) * N * kDispMaxNb + 16 * 256));
  int *d_begin = A.take<int>(nsystems + 1);
  float *d_r = A.take<float>(N), *d_L = A.take<float>(nsystems);
  float *d_X = A.take<float>(N), *d_Y = A.take<float>(N);
  int *d_count = A.take<int>(nsystems), *d_nn = A.take<int>(N);
  int *d_nb = A.take<int>(N * kDispMaxNb);
  float *d_inner = A.take<float>(N * kDispMaxNb);
  if (!A.ok()) return fail(DPM_ECAPACITY, "device arena exhausted");
  DPM_CUDA_TRY(cudaMemcpyAsync(d_begin, begin.data(), sizeof(int) * (nsystems + 1),
                               cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(d_r, radius, sizeof(float) * N, cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(d_L, L, sizeof(float) * nsystems, cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(d_X, X, sizeof(float) * N, cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(d_Y, Y, sizeof(float) * N, cudaMemcpyHostToDevice, s));
  DisperseArgs a{d_begin, d_r, d_L, d_X, d_Y, d_count, d_nb, d_nn, d_inner};
  const size_t smem = sizeof(float) * 5 * (size_t)nmax;
  DPM_CUDA_TRY(cudaFuncSetAttribute(k_disperse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)std::max<size_t>(smem, 1)));
  k_disperse<<<nsystems, kDispThreads, smem, s>>>(a);
  DPM_CUDA_TRY(cudaGetLastError());
  DPM_CUDA_TRY(cudaMemcpyAsync(X, d_X, sizeof(float) * N, cudaMemcpyDeviceToHost, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(Y, d_Y, sizeof(float) * N, cudaMemcpyDeviceToHost, s));
  std::vector<int> cnt(nsystems);
  DPM_CUDA_TRY(cudaMemcpyAsync(cnt.data(), d_count, sizeof(int) * nsystems,
                               cudaMemcpyDeviceToHost, s));
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  if (iterations) std::copy(cnt.begin(), cnt.end(), iterations);
  return DPM_OK;
}
