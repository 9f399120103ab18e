// 2D DPM kernels for sm_103a: initial geometry, diagnostics, the cell list
// (bin keys, neighbour lists) and the dispatch of the fused step.
//
// One warp owns one cell per launch.  A time step is ONE fused kernel
// (k2d_step, in dpm2d_step.cuh): it reads the cell's vertex ring once,
// computes the area, perimeter and bending forces from the ring held in
// shared memory, the attraction and repulsion against the cells of its
// neighbour list, applies the overdamped Euler update, writes the new
// positions, and -- as its epilogue -- the geometry of the new positions
// (centre, enclosing radius, area, box) that the next step's neighbour tests
// read.  The force field is never stored unless the caller asks for the last
// step's forces.
//
// Physics follows the reference kernels (shaders/Cell2D_kernel.cl); the
// repulsion's containment test uses the reference's exact crossing
// arithmetic (each operation rounded separately, no contraction), so that a
// vertex is flagged inside another cell on exactly the same inputs as the
// reference flags it.  Candidate cells are pruned with tests that are proved
// conservative (see `vertex_candidate` in dpm2d_device.cuh), so pruning
// never changes a flag; the neighbour lists below only ever hold more cells
// than those tests need.
#include "dpm2d_kernels.cuh"

#include <math.h>

#include "dpm2d_device.cuh"

namespace dpm {

namespace {

// ---------------------------------------------------------------------------
// Initial geometry
// ---------------------------------------------------------------------------

constexpr int kGeomWarps = 8;

__global__ void __launch_bounds__(kGeomWarps * 32)
    k2d_geom(const Cell2D *__restrict__ cells, const float2 *__restrict__ pos,
             Geom2D *__restrict__ geom, int ncells) {
  __shared__ float shx[kGeomWarps][kMaxNV2D], shy[kGeomWarps][kMaxNV2D];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * kGeomWarps + w;
  if (c >= ncells) return;
  const Cell2D cp = cells[c];
  const int n = (int)cp.nv;
  if (n == 0) return;  // an empty slot
  for (int k = lane; k < n; k += 32) {
    const float2 v = pos[cp.voff + k];
    shx[w][k] = v.x;
    shy[w][k] = v.y;
  }
  __syncwarp();
  const Geom2D g = ring_geom(shx[w], shy[w], n, lane);
  if (lane == 0) geom[c] = g;
}

// ---------------------------------------------------------------------------
// Diagnostics (double precision, one warp per cell)
// ---------------------------------------------------------------------------

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Per cell: |area| (shoelace), perimeter, sum over edges of (l/l0 - 1)^2 and
// sum over vertices of |s_i|^2, s_i = (x_{i+1} - x_i) - (x_i - x_{i-1}).
__global__ void __launch_bounds__(kGeomWarps * 32)
    k2d_diag(const Cell2D *__restrict__ cells, const float2 *__restrict__ pos, Diag2D *out,
             int ncells) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * kGeomWarps + w;
  if (c >= ncells) return;
  const Cell2D cp = cells[c];
  const int n = (int)cp.nv;
  if (n == 0) {
    if (lane == 0) out[c] = Diag2D{0.0, 0.0, 0.0, 0.0};
    return;
  }
  const float2 *p = pos + cp.voff;
  double A = 0.0, P = 0.0, Ul = 0.0, Ub = 0.0;
  for (int i = lane; i < n; i += 32) {
    const int j = i + 1 == n ? 0 : i + 1, k = i == 0 ? n - 1 : i - 1;
    const double xi = p[i].x, yi = p[i].y, xj = p[j].x, yj = p[j].y, xk = p[k].x, yk = p[k].y;
    A += xi * yj - xj * yi;
    const double l = sqrt((xj - xi) * (xj - xi) + (yj - yi) * (yj - yi));
    P += l;
    const double dl = l / (double)cp.l0 - 1.0;
    Ul += dl * dl;
    const double sx = (xj - xi) - (xi - xk), sy = (yj - yi) - (yi - yk);
    Ub += sx * sx + sy * sy;
  }
  A = warp_sum_d(A);
  P = warp_sum_d(P);
  Ul = warp_sum_d(Ul);
  Ub = warp_sum_d(Ub);
  if (lane == 0) out[c] = Diag2D{fabs(0.5 * A), P, Ul, Ub};
}

// ---------------------------------------------------------------------------
// Cell list: per-tissue bins and keys
// ---------------------------------------------------------------------------

__device__ __forceinline__ int bin_count_dev(float L, float w, int cap) {
  int nb = (int)floorf(__fdiv_rn(L, w));
  return max(1, min(nb, cap));
}

__device__ __forceinline__ int bin_of(float x, float L, float inv, int nb) {
  int b = (int)floorf(__fmul_rn(wrap_rn(x, L), inv));
  return max(0, min(b, nb - 1));
}

__device__ __forceinline__ float block_reduce_max(float v, float *sh) {
  v = warp_max(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  float r = -INFINITY;
  for (int i = 0; i < nw; ++i) r = fmaxf(r, sh[i]);
  return r;
}
__device__ __forceinline__ float block_reduce_min(float v, float *sh) {
  return -block_reduce_max(-v, sh);
}

__global__ void __launch_bounds__(256) k2d_binprep(Rebuild2DArgs a, int local_bits) {
  __shared__ float red[32];
  const int t = blockIdx.x;
  const Tissue2D T = a.tissues[t];
  float dmax = 0.f, mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
  for (int c = T.cell_begin + threadIdx.x; c < T.cell_end; c += blockDim.x) {
    const Geom2D g = a.geom[c];
    dmax = fmaxf(dmax, 2.0f * g.R);
    mnx = fminf(mnx, g.minx);
    mxx = fmaxf(mxx, g.maxx);
    mny = fminf(mny, g.miny);
    mxy = fmaxf(mxy, g.maxy);
  }
  dmax = block_reduce_max(dmax, red);
  mnx = block_reduce_min(mnx, red);
  mxx = block_reduce_max(mxx, red);
  mny = block_reduce_min(mny, red);
  mxy = block_reduce_max(mxy, red);
  float w = __fadd_rn(dmax, T.skin);
  w = __fadd_rn(w, __fadd_rn(__fmul_rn(1e-3f, dmax), __fmul_rn(1e-5f, T.L)));
  if (T.Kat != 0.0f) w = __fadd_rn(w, T.l0max);
  const int nb = bin_count_dev(T.L, w, T.cap);
  if (threadIdx.x == 0) {
    Tissue2D *o = a.tissues + t;
    o->binw = w;
    o->nbx = nb;
    o->nby = nb;
    o->gminx = mnx;
    o->gmaxx = mxx;
    o->gminy = mny;
    o->gmaxy = mxy;
    a.stale[t] = 0;
    // the tissue's share of the rebuild period that follows
    if (a.block_len > 0) {
      const int run = min(T.steps_left, a.block_len);
      o->run_now = run;
      if (T.steps_left < kStepsUnlimited) o->steps_left = T.steps_left - run;
    }
  }
  const float inv = __fdiv_rn((float)nb, T.L);
  for (int c = T.cell_begin + threadIdx.x; c < T.cell_end; c += blockDim.x) {
    const Geom2D g = a.geom[c];
    const int bx = bin_of(g.cx, T.L, inv, nb), by = bin_of(g.cy, T.L, inv, nb);
    a.keys[c] = ((uint32_t)t << local_bits) | (uint32_t)(by * nb + bx);
    a.vals[c] = (uint32_t)c;
  }
  // empty slots sort after the tissue's cells
  for (int c = T.cell_end + threadIdx.x; c < T.cell_cap; c += blockDim.x) {
    a.keys[c] = ((uint32_t)t << local_bits) | ((1u << local_bits) - 1u);
    a.vals[c] = (uint32_t)c;
  }
}

// ---------------------------------------------------------------------------
// Cell list: neighbour lists
// ---------------------------------------------------------------------------

constexpr int kNbWarps = 8;
constexpr int kNbBuf = 128;
static_assert(kNbBuf >= kMaxNB2D + 32, "neighbour buffer too small");

__device__ __forceinline__ int lower_bound_u32(const uint32_t *a, int lo, int hi, uint32_t key) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Does pair (i, j) need to be in i's list for the next rebuild period?
// Distances may change by at most the skin before the list is rebuilt or
// declared stale (each cell's box and circle move by at most skin/2).
// The rebuild tests below use separately rounded operations only, in a fixed
// order, so that a host rebuild with IEEE float32 arithmetic reproduces the
// neighbour lists bit for bit.
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }

// Slack of the rebuild tests: well above the per-step tests' margins.
__device__ __forceinline__ float rebuild_margin(const Geom2D &gi, const Geom2D &gj,
                                                const Tissue2D &T) {
  const float mag =
      fa(fa(fa(fa(fabsf(gi.cx), fabsf(gi.cy)), fabsf(gj.cx)), fabsf(gj.cy)), T.L);
  return fa(fm(1e-3f, fa(gi.R, gj.R)), fm(1e-4f, mag));
}

__device__ __forceinline__ float round_away(float x) { return roundf(x); }

__device__ __forceinline__ bool pair_near(const Geom2D &gi, const Geom2D &gj,
                                          const Tissue2D &T, float l0) {
  const float dx = fs(gi.cx, gj.cx), dy = fs(gi.cy, gj.cy);
  const float m = rebuild_margin(gi, gj, T);
  const float r = fa(fa(fa(gi.R, gj.R), T.skin), m);
  if (fa(fm(dx, dx), fm(dy, dy)) <= fm(r, r)) return true;
  if (T.Kat != 0.0f) {
    float ex = dx, ey = dy;
    if (T.pbc) {
      ex = fs(ex, fm(T.L, round_away(__fdiv_rn(ex, T.L))));
      ey = fs(ey, fm(T.L, round_away(__fdiv_rn(ey, T.L))));
    }
    const float ra = fa(r, fmaxf(l0, T.l0max));
    if (fa(fm(ex, ex), fm(ey, ey)) <= fm(ra, ra)) return true;
  }
  return false;
}

__device__ __forceinline__ bool pair_far(const Geom2D &gi, const Geom2D &gj, const Tissue2D &T) {
  if (!T.pbc) return false;
  const float lim = fs(fs(T.L, T.skin), rebuild_margin(gi, gj, T));
  return fs(gi.maxx, gj.minx) >= lim || fs(gj.maxx, gi.minx) >= lim ||
         fs(gi.maxy, gj.miny) >= lim || fs(gj.maxy, gi.miny) >= lim;
}

__device__ __forceinline__ bool cell_on_boundary(const Geom2D &gi, const Tissue2D &T) {
  if (!T.pbc) return false;
  // any far partner j passes the pair test against the tissue extent, with
  // a margin at least as large as rebuild_margin(gi, gj)
  const float ext = fa(fa(fa(fabsf(T.gminx), fabsf(T.gmaxx)), fabsf(T.gminy)), fabsf(T.gmaxy));
  const float own = fa(fa(fabsf(gi.cx), fabsf(gi.cy)), T.L);
  const float m = fa(fa(fm(2e-3f, fa(gi.R, T.binw)), fm(1e-4f, own)), fm(2e-4f, ext));
  const float lim = fs(fs(T.L, T.skin), m);
  return fs(gi.maxx, T.gminx) >= lim || fs(T.gmaxx, gi.minx) >= lim ||
         fs(gi.maxy, T.gminy) >= lim || fs(T.gmaxy, gi.miny) >= lim;
}

__global__ void __launch_bounds__(kNbWarps * 32) k2d_neighbors(Rebuild2DArgs a, int local_bits) {
  __shared__ int buf[kNbWarps][kNbBuf];
  __shared__ unsigned char uniq[kNbWarps][kNbBuf];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * kNbWarps + w;
  if (c >= a.ncells) return;
  const Cell2D cp = a.cells[c];
  if (cp.nv == 0) {  // an empty slot
    if (lane == 0) a.nn[c] = 0;
    return;
  }
  const int t = (int)cp.tissue;
  const Tissue2D T = a.tissues[t];
  const Geom2D gi = a.geom[c];
  const unsigned lt = (1u << lane) - 1u;
  int cnt = 0;

  const int nb = T.nbx;
  const float inv = __fdiv_rn((float)nb, T.L);
  const int bx = bin_of(gi.cx, T.L, inv, nb), by = bin_of(gi.cy, T.L, inv, nb);
  // distinct bin offsets along an axis with nb bins; lane l finds the
  // sorted range of the l-th neighbouring bin (the searches run side by
  // side), then their cells are tested in bin order, 32 at a time
  const int lo_off = nb >= 3 ? -1 : 0, hi_off = nb >= 3 ? 1 : nb - 1;
  const int nax = hi_off - lo_off + 1, nbins = nax * nax;
  int blo = 0, bhi = 0;
  if (lane < nbins) {
    const int yy = (by + lo_off + lane / nax + nb) % nb;
    const int xx = (bx + lo_off + lane % nax + nb) % nb;
    const uint32_t key = ((uint32_t)t << local_bits) | (uint32_t)(yy * nb + xx);
    blo = lower_bound_u32(a.sorted_keys, T.cell_begin, T.cell_end, key);
    bhi = lower_bound_u32(a.sorted_keys, blo, T.cell_end, key + 1u);
  }
  // the bins' cells as one flat range over the lanes (prefix sum of the
  // bin sizes; a lane finds its bin by binary search over the prefix)
  const int bsize = bhi - blo;
  int bincl = bsize;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, bincl, o);
    if (lane >= o) bincl += y;
  }
  const int btotal = __shfl_sync(kFull, bincl, 31);
  const int bexcl = bincl - bsize;
  for (int t0 = 0; t0 < btotal; t0 += 32) {
    const int tt = t0 + lane;
    int ob = 0;
#pragma unroll
    for (int st = 16; st > 0; st >>= 1)
      if (__shfl_sync(kFull, bexcl, ob + st) <= tt) ob += st;
    const int q = __shfl_sync(kFull, blo, ob) + tt - __shfl_sync(kFull, bexcl, ob);
    const int j = tt < btotal ? (int)a.sorted_vals[q] : -1;
    const bool ok = j >= 0 && j != c && pair_near(gi, a.geom[j], T, cp.l0);
    const unsigned m = __ballot_sync(kFull, ok);
    const int pos = cnt + __popc(m & lt);
    if (ok && pos < kNbBuf) buf[w][pos] = j;
    cnt += __popc(m);
  }
  // pairs whose raw offsets can exceed L (the reference's shifted edges)
  if (cell_on_boundary(gi, T)) {
    for (int base = T.cell_begin; base < T.cell_end; base += 32) {
      const int j = base + lane;
      const bool ok = j < T.cell_end && j != c && pair_far(gi, a.geom[j], T);
      const unsigned m = __ballot_sync(kFull, ok);
      const int pos = cnt + __popc(m & lt);
      if (ok && pos < kNbBuf) buf[w][pos] = j;
      cnt += __popc(m);
    }
  }
  __syncwarp();
  int nout;
  if (cnt > kNbBuf) {
    nout = kNbOverflow;
  } else {
    // drop duplicates, then place each unique id at its rank (ascending ids)
    for (int i = lane; i < cnt; i += 32) {
      const int v = buf[w][i];
      bool first = true;
      for (int k = 0; k < i; ++k) first &= buf[w][k] != v;
      uniq[w][i] = first ? 1 : 0;
    }
    __syncwarp();
    int nu = 0;
    for (int i = 0; i < cnt; ++i) nu += uniq[w][i];
    if (nu > kMaxNB2D) {
      nout = kNbOverflow;
    } else {
      int *out = a.nbr + (size_t)c * kMaxNB2D;
      for (int i = lane; i < cnt; i += 32) {
        if (!uniq[w][i]) continue;
        const int v = buf[w][i];
        int rank = 0;
        for (int k = 0; k < cnt; ++k) rank += (uniq[w][k] && buf[w][k] < v) ? 1 : 0;
        out[rank] = v;
      }
      nout = nu;
    }
  }
  if (lane == 0) {
    a.nn[c] = nout;
    a.geom0[c] = gi;
  }
}

// ---------------------------------------------------------------------------
// Compression: a tissue rescaled to a packing fraction
// ---------------------------------------------------------------------------

// The host Tissue2D::SetPackingFraction (an extension: the reference has no
// way to change its box) on the device, with the host's arithmetic so that
// both give the same bits: each cell's float shoelace area in the
// reference's order (src/cell.cpp:35-47), summed in double in cell order;
// L' = sqrt(sum / phi); every vertex moved by its cell's vertex-mean centroid
// (double) times L'/L - 1 and rounded to float.  One block per tissue;
// phi <= 0 leaves the tissue as it is.  The tissue's neighbour lists are
// marked stale (the step scans the whole tissue until the next rebuild).
__global__ void __launch_bounds__(256)
    k2d_rescale(const Cell2D *__restrict__ cells, Tissue2D *tissues, const float *phi,
                float2 *pos, int *stale) {
  __shared__ float area[256];
  __shared__ double scale_m1;
  const int t = blockIdx.x;
  const float ph = phi[t];
  if (!(ph > 0.0f)) return;  // the same for the whole block
  const Tissue2D T = tissues[t];
  double sum = 0.0;  // thread 0's, in cell order
  for (int base = T.cell_begin; base < T.cell_end; base += blockDim.x) {
    const int c = base + (int)threadIdx.x;
    float a = 0.0f;
    if (c < T.cell_end) {
      const Cell2D cp = cells[c];
      const int n = (int)cp.nv;
      const float2 *p = pos + cp.voff;
      for (int i = 0, j = n - 1; i < n; j = i++) {
        const float s = __fadd_rn(p[j].x, p[i].x), d = __fsub_rn(p[j].y, p[i].y);
        a = (float)__dadd_rn((double)a, __dmul_rn(0.5, (double)__fmul_rn(s, d)));
      }
      a = a < 0.0f ? -a : a;
    }
    area[threadIdx.x] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
      const int m = min((int)blockDim.x, T.cell_end - base);
      for (int k = 0; k < m; ++k) sum = __dadd_rn(sum, (double)area[k]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double Lnew = sqrt(__ddiv_rn(sum, (double)ph));
    scale_m1 = __dsub_rn(__ddiv_rn(Lnew, (double)T.L), 1.0);
    tissues[t].L = (float)Lnew;
    stale[t] = 1;
  }
  __syncthreads();
  const double sm1 = scale_m1;
  for (int c = T.cell_begin + (int)threadIdx.x; c < T.cell_end; c += blockDim.x) {
    const Cell2D cp = cells[c];
    const int n = (int)cp.nv;
    if (n == 0) continue;
    float2 *p = pos + cp.voff;
    double cx = 0.0, cy = 0.0;
    for (int i = 0; i < n; ++i) {
      cx = __dadd_rn(cx, (double)p[i].x);
      cy = __dadd_rn(cy, (double)p[i].y);
    }
    const double dx = __dmul_rn(__ddiv_rn(cx, (double)n), sm1);
    const double dy = __dmul_rn(__ddiv_rn(cy, (double)n), sm1);
    for (int i = 0; i < n; ++i)
      p[i] = make_float2((float)__dadd_rn((double)p[i].x, dx),
                         (float)__dadd_rn((double)p[i].y, dy));
  }
}

} // namespace

cudaError_t launch_rescale2d(const Cell2D *cells, Tissue2D *tissues, const float *phi,
                             float2 *pos, int *stale, int ntissues, cudaStream_t s) {
  k2d_rescale<<<ntissues, 256, 0, s>>>(cells, tissues, phi, pos, stale);
  return cudaGetLastError();
}

int bin_axis_count(float L, float w, int cap) {
  int nb = (int)floorf(L / w);
  return nb < 1 ? 1 : (nb > cap ? cap : nb);
}

cudaError_t launch_geom2d(const Cell2D *cells, const float2 *pos, Geom2D *geom, int ncells,
                          int maxnv, cudaStream_t s) {
  (void)maxnv;
  const int grid = (ncells + kGeomWarps - 1) / kGeomWarps;
  k2d_geom<<<grid, kGeomWarps * 32, 0, s>>>(cells, pos, geom, ncells);
  return cudaGetLastError();
}

cudaError_t launch_diag2d(const Cell2D *cells, const float2 *pos, Diag2D *out, int ncells,
                          cudaStream_t s) {
  const int grid = (ncells + kGeomWarps - 1) / kGeomWarps;
  k2d_diag<<<grid, kGeomWarps * 32, 0, s>>>(cells, pos, out, ncells);
  return cudaGetLastError();
}

cudaError_t launch_binprep2d(const Rebuild2DArgs &a, int local_bits, cudaStream_t s) {
  k2d_binprep<<<a.ntissues, 256, 0, s>>>(a, local_bits);
  return cudaGetLastError();
}

cudaError_t launch_neighbors2d(const Rebuild2DArgs &a, int local_bits, cudaStream_t s) {
  const int grid = (a.ncells + kNbWarps - 1) / kNbWarps;
  k2d_neighbors<<<grid, kNbWarps * 32, 0, s>>>(a, local_bits);
  return cudaGetLastError();
}

size_t resident2d_smem_bytes(int ncmax, int nvmax) {
  return 128 + sizeof(Cell2D) * (size_t)ncmax + 2 * sizeof(Geom2D) * (size_t)ncmax +
         2 * sizeof(float2) * (size_t)nvmax;
}

cudaError_t launch_resident2d(const Resident2DArgs &r, int ntissues, int maxnv, int variant,
                              cudaStream_t s) {
  if (maxnv <= 32) return launch_resident2d_s1(r, ntissues, variant, s);
  return launch_resident2d_s2(r, ntissues, variant, s);
}

cudaError_t launch_step2d(const Step2DArgs &a, int maxnv, int warps, int occ, cudaStream_t s) {
  if (maxnv <= 32) return launch_step2d_s1(a, warps, occ, s);
  if (maxnv <= 64) return launch_step2d_s2(a, warps, occ, s);
  if (maxnv <= 128) return launch_step2d_s4(a, warps, occ, s);
  return launch_step2d_s8(a, warps, occ, s);
}

} // namespace dpm
