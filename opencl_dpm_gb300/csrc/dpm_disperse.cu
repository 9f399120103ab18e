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
// in the reference; one thread then adds the U terms in row order.
// Contacts come from per-cell lists of the cells within the contact distance
// plus a skin, rebuilt when some centre has moved by half the skin, kept in
// ascending order; the contact test itself is the reference's.
//
// Where the reference rounds a double expression of float operands to float
// and the double operation is exact (or is a correctly rounded sqrt, which
// rounds to float without double-rounding error since 53 >= 2*24 + 2), the
// same bits come from the float operation; only the force magnitude
// (1 - q)/(ri + rj) and the position update x + 0.01 F stay in double.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "dpm_common.cuh"
#include "dpm_runtime.hpp"

namespace dpm {
namespace {

constexpr int kDispThreads = 256;
constexpr int kDispMaxNb = 48;       // list capacity per cell (more: scan all)
constexpr int kDispMaxCells = 4096;  // per system (shared-memory staging)
constexpr int kDispMaxIter = 100000; // the reference's cap (count > 1e5)
constexpr int kDispTerms = 6;        // U terms per row kept in shared memory
constexpr int kDispContacts = 24;    // contacts per cell folded from registers

struct DisperseArgs {
  const int *begin;    // [nsys + 1] first cell of each system
  const float *radius; // [ncells]
  const float *L;      // [nsys]
  float *X, *Y;        // [ncells] in: start; out: relaxed
  int *count;          // [nsys] iterations run
  int *nb;             // [ncells * kDispMaxNb] contact candidates, ascending
  int *nn;             // [ncells] candidate count, -1: scan every cell
  float *inner;        // [ncells * kDispMaxNb] U terms of rows with many contacts
};

// x - L round(x / L), rounded to float as the reference's
// (float)((double)x - (double)L * round((double)(x / L))).
__device__ __forceinline__ float wrap_ref(float x, float L) {
  const float r = roundf(__fdiv_rn(x, L));
  if (r == 0.0f) return x;
  if (fabsf(r) == 1.0f) return __fsub_rn(x, r == 1.0f ? L : -L);  // exact in double
  return __double2float_rn(__dsub_rn((double)x, __dmul_rn((double)L, (double)r)));
}

// The reference's wrapped offset from (xi, yi) to (xj, yj), distance, and
// contact test dist <= ri + rj.
__device__ __forceinline__ bool contact(float xi, float yi, float ri, float xj, float yj,
                                        float rj, float L, float &dx, float &dy, float &dist) {
  dx = wrap_ref(__fsub_rn(xj, xi), L);
  dy = wrap_ref(__fsub_rn(yj, yi), L);
  dist = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
  return dist <= __fadd_rn(ri, rj);
}

// Pair force (fx, fy) and energy term 1 - q (1 - q), q = dist / (ri + rj),
// of the reference for a pair in contact.
__device__ __forceinline__ void pair_terms(float dx, float dy, float dist, float ri, float rj,
                                           float &fx, float &fy, float &u) {
  const float ux = __fdiv_rn(dx, dist), uy = __fdiv_rn(dy, dist);
  const float s = __fadd_rn(ri, rj);
  const float q = __fdiv_rn(dist, s);
  const float ftmp = __double2float_rn(__ddiv_rn(__dsub_rn(1.0, (double)q), (double)s));
  fx = __fmul_rn(ftmp, ux);
  fy = __fmul_rn(ftmp, uy);
  u = __fsub_rn(1.0f, __fmul_rn(q, __fsub_rn(1.0f, q)));
}

__global__ void __launch_bounds__(kDispThreads) k_disperse(DisperseArgs a) {
  extern __shared__ float sm[];
  __shared__ int s_rebuild, s_stop;
  __shared__ float s_red[kDispThreads / 32];
  const int sys = blockIdx.x;
  const int c0 = a.begin[sys], n = a.begin[sys + 1] - c0;
  const float L = a.L[sys];
  float *X = sm, *Y = X + n, *X0 = Y + n, *Y0 = X0 + n, *R = Y0 + n;
  float *T = R + n;                              // [n * kDispTerms] U terms
  int *tc = reinterpret_cast<int *>(T + (size_t)n * kDispTerms);  // [n] U term counts
  const int tid = threadIdx.x;
  float rmin = INFINITY;
  for (int k = tid; k < n; k += kDispThreads) {
    X[k] = a.X[c0 + k];
    Y[k] = a.Y[c0 + k];
    R[k] = a.radius[c0 + k];
    rmin = fminf(rmin, R[k]);
  }
  // skin of the contact lists: half the smallest radius
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
    bool rescan = false;  // a U row must be rescanned from the positions
#pragma unroll 1
    for (int t = 0, k = tid; k < n; ++t, k += kDispThreads) {
      const float xk = X[k], yk = Y[k], rk = R[k];
      const int m = nn[k];
      const int *lst = nb + (size_t)k * kDispMaxNb;
      const int cnt = m < 0 ? n : m;
      // contacts of row k in ascending order: pair force and U term
      float cfx[kDispContacts], cfy[kDispContacts];
      int nc = 0, nlt = 0;
      bool many = false;
      float Fx = 0.0f, Fy = 0.0f;
      for (int p = 0; p < cnt; ++p) {
        const int j = m < 0 ? p : lst[p];
        if (j == k) continue;
        float dx, dy, dist;
        if (!contact(xk, yk, rk, X[j], Y[j], R[j], L, dx, dy, dist)) continue;
        float fx, fy, u;
        pair_terms(dx, dy, dist, rk, R[j], fx, fy, u);
        if (nc < kDispTerms) T[(size_t)k * kDispTerms + nc] = u;
        else if (m >= 0) inner[(size_t)k * kDispMaxNb + nc] = u;
        if (nc < kDispContacts) {
          cfx[nc] = fx;
          cfy[nc] = fy;
        } else {
          many = true;
        }
        nlt += j < k ? 1 : 0;
        ++nc;
      }
      tc[k] = m < 0 && nc > kDispTerms ? -1 : nc;
      rescan |= tc[k] < 0;
      if (!many) {
        // segment 1: j < k; segment 2: all; segment 3: j > k
#pragma unroll 1
        for (int p = 0; p < nlt; ++p) {
          Fx = __fsub_rn(Fx, cfx[p]);
          Fy = __fsub_rn(Fy, cfy[p]);
        }
#pragma unroll 1
        for (int p = 0; p < nc; ++p) {
          Fx = __fsub_rn(Fx, cfx[p]);
          Fy = __fsub_rn(Fy, cfy[p]);
        }
#pragma unroll 1
        for (int p = nlt; p < nc; ++p) {
          Fx = __fsub_rn(Fx, cfx[p]);
          Fy = __fsub_rn(Fy, cfy[p]);
        }
      } else {
        // more contacts than registers hold: recompute per segment
        for (int seg = 0; seg < 3; ++seg)
          for (int p = 0; p < cnt; ++p) {
            const int j = m < 0 ? p : lst[p];
            if (j == k || (seg == 0 && j > k) || (seg == 2 && j < k)) continue;
            float dx, dy, dist;
            if (!contact(xk, yk, rk, X[j], Y[j], R[j], L, dx, dy, dist)) continue;
            float fx, fy, u;
            pair_terms(dx, dy, dist, rk, R[j], fx, fy, u);
            Fx = __fsub_rn(Fx, fx);
            Fy = __fsub_rn(Fy, fy);
          }
      }
      fxk[t] = Fx;
      fyk[t] = Fy;
    }
    // without rescans the U sum reads only stored terms, so the position
    // update below may overlap it
    const bool any_rescan = __syncthreads_or(rescan) != 0;

    // U in row order (one thread): U = (float)((double)U + 0.5 * inner) is
    // the float sum U + 0.5f * inner, the double sum being exact
    if (tid == 0) {
      float U = 0.0f;
      for (int k = 0; k < n; ++k) {
        const int u = tc[k];
        if (u >= 0) {
          const float *row = T + (size_t)k * kDispTerms;
#pragma unroll
          for (int p = 0; p < kDispTerms; ++p)
            if (p < u) U = __fadd_rn(U, __fmul_rn(0.5f, row[p]));
          for (int p = kDispTerms; p < u; ++p)
            U = __fadd_rn(U, __fmul_rn(0.5f, inner[(size_t)k * kDispMaxNb + p]));
        } else {
          // a row scanned in full with more terms than the buffers hold
          for (int j = 0; j < n; ++j) {
            if (j == k) continue;
            float dx, dy, dist;
            if (!contact(X[k], Y[k], R[k], X[j], Y[j], R[j], L, dx, dy, dist)) continue;
            float fx, fy, uu;
            pair_terms(dx, dy, dist, R[k], R[j], fx, fy, uu);
            U = __fadd_rn(U, __fmul_rn(0.5f, uu));
          }
        }
      }
      float dU = __fsub_rn(U, oldU);
      if (dU < 0.0f) dU = -dU;
      oldU = U;
      ++count;
      s_stop = !((double)dU > 1e-6) || count > kDispMaxIter;
    }
    if (any_rescan) __syncthreads();
    bool moved = false;
#pragma unroll 1
    for (int t = 0, k = tid; k < n; ++t, k += kDispThreads) {
      X[k] = __double2float_rn(__dadd_rn((double)X[k], __dmul_rn(0.01, (double)fxk[t])));
      Y[k] = __double2float_rn(__dadd_rn((double)Y[k], __dmul_rn(0.01, (double)fyk[t])));
      const float d = fabsf(X[k] - X0[k]) + fabsf(Y[k] - Y0[k]);
      moved |= !(d <= 0.5f * skin);
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
  // positions, starts, radii, U terms and their counts of the largest system
  const size_t smem = sizeof(float) * (5 + kDispTerms + 1) * (size_t)nmax;
  {
    // the kernel's limit is shared by concurrent calls: only ever raised
    static std::mutex mu;
    static size_t granted[64] = {0};
    int dev = 0;
    DPM_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || smem > granted[dev]) {
      DPM_CUDA_TRY(cudaFuncSetAttribute(k_disperse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
      if (dev >= 0 && dev < 64) granted[dev] = smem;
    }
  }
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
