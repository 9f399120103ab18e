// 2D DPM kernels for sm_103a.
//
// One warp owns one cell per launch.  A time step is ONE fused kernel
// (k2d_step): it reads the cell's vertex ring once, computes the area,
// perimeter and bending forces from the ring held in shared memory, the
// attraction and repulsion against the cells of its neighbour list, applies
// the overdamped Euler update, writes the new positions, and -- as its
// epilogue -- the geometry of the new positions (centre, enclosing radius,
// area, box) that the next step's neighbour tests read.  The force field is
// never stored unless the caller asks for the last step's forces.
//
// Physics follows the reference kernels (shaders/Cell2D_kernel.cl); the
// repulsion's containment test uses the reference's exact crossing
// arithmetic (each operation rounded separately, no contraction), so that a
// vertex is flagged inside another cell on exactly the same inputs as the
// reference flags it.  Candidate cells are pruned with tests that are proved
// conservative (see `vertex_candidate`), so pruning never changes a flag.
#include "dpm2d_kernels.cuh"

#include <math.h>

namespace dpm {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr float kRelMargin = 1e-5f;  // relative slack of the pruning tests
constexpr float kAbsMargin = 1e-6f;  // per unit of coordinate magnitude

// Geometry of the ring (sx, sy)[0..n) in shared memory: vertex mean, largest
// distance to it, |shoelace area| (Cell2D_kernel.cl:25-36 form), box.
__device__ Geom2D ring_geom(const float *sx, const float *sy, int n, int lane) {
  float sumx = 0.f, sumy = 0.f, ar = 0.f;
  float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
  for (int k = lane; k < n; k += 32) {
    const float x = sx[k], y = sy[k];
    const int km = k == 0 ? n - 1 : k - 1;
    sumx += x;
    sumy += y;
    ar += 0.5f * ((sx[km] + x) * (sy[km] - y));
    mnx = fminf(mnx, x);
    mxx = fmaxf(mxx, x);
    mny = fminf(mny, y);
    mxy = fmaxf(mxy, y);
  }
  Geom2D g;
  g.cx = warp_sum(sumx) / (float)n;
  g.cy = warp_sum(sumy) / (float)n;
  g.area = fabsf(warp_sum(ar));
  g.minx = warp_min(mnx);
  g.maxx = warp_max(mxx);
  g.miny = warp_min(mny);
  g.maxy = warp_max(mxy);
  float r2 = 0.f;
  for (int k = lane; k < n; k += 32) {
    const float dx = sx[k] - g.cx, dy = sy[k] - g.cy;
    r2 = fmaxf(r2, dx * dx + dy * dy);
  }
  g.R = sqrtf(warp_max(r2));
  return g;
}

// One edge of the reference's crossing-number test (Cell2D_kernel.cl:171-195)
// for the point (X, Y) and the edge (P_i, P_j), j = i-1: offsets d = v - P,
// shifted per axis by L*floor (x) or L*round (y) when that edge has |d| > L,
// then the half-open y test and the sign of the x intercept.  Every
// operation is rounded on its own, as in the reference.
__device__ __forceinline__ unsigned edge_crosses(float X, float Y, float pix, float piy,
                                                 float pjx, float pjy, bool pbc, float L) {
  float dix = __fsub_rn(X, pix), diy = __fsub_rn(Y, piy);
  float djx = __fsub_rn(X, pjx), djy = __fsub_rn(Y, pjy);
  if (pbc) {
    if (fabsf(dix) > L || fabsf(djx) > L) {
      dix = __fsub_rn(dix, __fmul_rn(L, floorf(__fdiv_rn(dix, L))));
      djx = __fsub_rn(djx, __fmul_rn(L, floorf(__fdiv_rn(djx, L))));
    }
    if (fabsf(diy) > L || fabsf(djy) > L) {
      diy = __fsub_rn(diy, __fmul_rn(L, roundf(__fdiv_rn(diy, L))));
      djy = __fsub_rn(djy, __fmul_rn(L, roundf(__fdiv_rn(djy, L))));
    }
  }
  if ((diy > 0.0f) == (djy > 0.0f)) return 0u;
  const float r = __fadd_rn(
      __fdiv_rn(__fmul_rn(__fsub_rn(djx, dix), __fsub_rn(0.0f, diy)), __fsub_rn(djy, diy)),
      dix);
  return 0.0f < r ? 1u : 0u;
}

// Can the reference's crossing test flag (X, Y) inside cell j?
//  * If no edge of j is shifted (every |X - P.x| <= L and |Y - P.y| <= L),
//    an odd count needs miny < Y <= maxy (the y test compares exact signs)
//    and (X, Y) within the enclosing circle: outside it, (X, Y) is farther
//    than the margin from every edge, so every x intercept has its true
//    sign and the count equals the even-odd containment, which is 0.
//  * A shift happens only if some vertex is more than L away on an axis;
//    by monotone rounding that is decided exactly by the box corners.
//  * If only x offsets can be shifted, the y test still compares the raw
//    signs of Y - P.y, so again an odd count needs miny < Y <= maxy.
//  * If y offsets can be shifted: the reference shifts an edge's y offsets d
//    by L*round(d/L) (each endpoint by its own rounding) when an endpoint has
//    |d| > L.  d ranges over [fl(Y - maxy), fl(Y - miny)] and round(d/L) is
//    monotone in d; when it is one k (|k| <= 2, so L*k is exact) over the
//    range, unshifted edges have both offsets of k's sign (no crossing) and
//    shifted ones have offsets fl(d - kL), so a crossing needs the image
//    level Y - kL inside the box (exactly, by the same monotone bounds), and
//    with no x offset shifted the count is the plain test of the image point
//    (X, Y - kL), to which the circle test applies -- with one exception for
//    k = -1: a vertex of the ring at offset exactly -L is not shifted in an
//    edge whose other end is not, where the image test would count a
//    crossing.  Such points are kCheckY: candidates only if a ring vertex
//    lies within a few ulps of Y + L.
//  * If only x offsets can be shifted and the point is right of the ring by
//    more than L somewhere (but less than 1.5 L, and right of every vertex
//    by L/4), every offset after the reference's floor shift is >= 0, and
//    the computed x intercept r of an edge whose y signs differ exceeds the
//    smaller end offset minus 3.2 ulp(L); so r > 0 unless a ring vertex has
//    x offset within 8 ulp(L) of L, and the count is the number of sign
//    changes around the ring, even.  Such points are kCheckX.
//    (Left of the ring by more than L, the floor shift tears the ring and
//    the count can be odd: those points are evaluated.)
constexpr int kNotCandidate = 0, kCandidate = 1, kCheckY = 2, kCheckX = 3;

__device__ __forceinline__ int shifted_y_candidate(float X, float Y, const Geom2D &gj, float L) {
  const float dlo = __fsub_rn(Y, gj.maxy), dhi = __fsub_rn(Y, gj.miny);
  const float k = roundf(__fdiv_rn(dlo, L));
  if (k != roundf(__fdiv_rn(dhi, L)) || k == 0.0f || fabsf(k) > 2.0f) return kCandidate;
  const float kL = __fmul_rn(L, k);
  if (!(__fsub_rn(dlo, kL) <= 0.0f && __fsub_rn(dhi, kL) > 0.0f)) return kNotCandidate;
  // an x shift would tear the ring: evaluate the reference's test
  if (__fsub_rn(X, gj.minx) > L || __fsub_rn(gj.maxx, X) > L) return kCandidate;
  const float Ys = __fsub_rn(Y, kL);
  const float dx = X - gj.cx, dy = Ys - gj.cy;
  const float rm = gj.R * (1.0f + kRelMargin) +
                   kAbsMargin * (fabsf(gj.cx) + fabsf(gj.cy) + fabsf(X) + fabsf(Y) + L);
  const float bm = kRelMargin * (gj.maxx - gj.minx) +
                   kAbsMargin * (fabsf(gj.minx) + fabsf(gj.maxx) + fabsf(X));
  if (X >= gj.minx - bm && X <= gj.maxx + bm && dx * dx + dy * dy <= rm * rm) return kCandidate;
  // left of the ring every x intercept is to the right: nothing is counted
  return k == -1.0f && X >= gj.minx - bm ? kCheckY : kNotCandidate;
}

__device__ __forceinline__ int vertex_candidate(float X, float Y, const Geom2D &gj, bool near,
                                                bool far, float L) {
  const bool band = Y > gj.miny && Y <= gj.maxy;
  if (far) {
    const bool fy = __fsub_rn(Y, gj.miny) > L || __fsub_rn(gj.maxy, Y) > L;
    if (fy) return shifted_y_candidate(X, Y, gj, L);
    if (__fsub_rn(gj.maxx, X) > L) return band ? kCandidate : kNotCandidate;
    const float xr = __fsub_rn(X, gj.minx);
    if (xr > L) {
      if (!band) return kNotCandidate;
      return __fsub_rn(X, gj.maxx) > 0.25f * L && xr < 1.5f * L ? kCheckX : kCandidate;
    }
  }
  if (near && band) {
    const float dx = X - gj.cx, dy = Y - gj.cy;
    const float rm = gj.R * (1.0f + kRelMargin) +
                     kAbsMargin * (fabsf(gj.cx) + fabsf(gj.cy) + fabsf(X) + fabsf(Y));
    const float bm = kRelMargin * (gj.maxx - gj.minx) +
                     kAbsMargin * (fabsf(gj.minx) + fabsf(gj.maxx) + fabsf(X));
    if (X >= gj.minx - bm && X <= gj.maxx + bm && dx * dx + dy * dy <= rm * rm)
      return kCandidate;
  }
  return kNotCandidate;
}

__device__ __forceinline__ void normalize2(float x, float y, float &ox, float &oy) {
  const float l2 = x * x + y * y;
  if (l2 == 0.0f) {
    ox = x;
    oy = y;
    return;
  }
  const float l = sqrtf(l2);
  ox = x / l;
  oy = y / l;
}

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
  // distinct bin offsets along an axis with nb bins
  const int lo_off = nb >= 3 ? -1 : 0, hi_off = nb >= 3 ? 1 : nb - 1;
  for (int oy = lo_off; oy <= hi_off; ++oy) {
    const int yy = (by + oy + nb) % nb;
    for (int ox = lo_off; ox <= hi_off; ++ox) {
      const int xx = (bx + ox + nb) % nb;
      const uint32_t key = ((uint32_t)t << local_bits) | (uint32_t)(yy * nb + xx);
      const int lo = lower_bound_u32(a.sorted_keys, T.cell_begin, T.cell_end, key);
      const int hi = lower_bound_u32(a.sorted_keys, lo, T.cell_end, key + 1u);
      for (int base = lo; base < hi; base += 32) {
        const int q = base + lane;
        const int j = q < hi ? (int)a.sorted_vals[q] : -1;
        const bool ok = j >= 0 && j != c && pair_near(gi, a.geom[j], T, cp.l0);
        const unsigned m = __ballot_sync(kFull, ok);
        const int pos = cnt + __popc(m & lt);
        if (ok && pos < kNbBuf) buf[w][pos] = j;
        cnt += __popc(m);
      }
    }
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
// Fused step
// ---------------------------------------------------------------------------

// Occupancy variants: with OCC = 1 the register budget is capped so that
// 32 warps per SM stay resident (16 for more than 2 vertex slots per lane);
// with OCC = 0 the compiler chooses.  The tuner picks per batch.
template <int S, int W, int OCC> struct StepOcc {
  static constexpr int kThreads = S <= 2 ? 1024 : 512;
  static constexpr int kBlocks =
      OCC == 0 ? 1 : (kThreads / (W * 32) > 0 ? kThreads / (W * 32) : 1);
};

// One step of cell c by one warp; (sx, sy), (nxs, nys) and sf are the warp's
// shared-memory ring, neighbour ring and containment flags (32*S entries).
template <int S>
__device__ __forceinline__ void step_cell(const Step2DArgs &a, const int c, const int lane,
                                          float *sx, float *sy, float *nxs, float *nys,
                                          unsigned char *sf) {
  const Cell2D cp = a.cells[c];
  const int n = (int)cp.nv;
  if (n == 0) return;  // an empty slot
  const int tid = (int)cp.tissue;
  const Tissue2D T = a.tissues[tid];
  if (a.step_index >= T.run_now) {
    // the tissue's step budget is spent: carry its state over unchanged
    for (int k = lane; k < n; k += 32) a.pos_out[cp.voff + k] = a.pos_in[cp.voff + k];
    if (lane == 0) a.geom_out[c] = a.geom_in[c];
    return;
  }
  // outputs of this step: for every cell when asked, else at the tissue's last step
  const bool write_out =
      a.all_forces != 0 || (a.step_index == T.run_now - 1 && T.steps_left == 0);
  const float L = T.L;
  const bool pbc = T.pbc != 0;

  float vx[S], vy[S], fx[S], fy[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int k = lane + 32 * s;
    vx[s] = vy[s] = fx[s] = fy[s] = 0.0f;
    if (k < n) {
      const float2 v = a.pos_in[cp.voff + k];
      vx[s] = v.x;
      vy[s] = v.y;
      sx[k] = v.x;
      sy[k] = v.y;
      sf[k] = 0;
    }
  }
  __syncwarp();
  const Geom2D gi = a.geom_in[c];

  // -- shape forces: area (AreaForceUpdates, with the reference's sign of
  // the y term), perimeter (PerimeterForceUpdates), bending
  // (BendingForceUpdates); summed in the reference's order.
  const float strain = gi.area / cp.a0 - 1.0f;
  const float ka = cp.kA * 0.5f * strain;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int k = lane + 32 * s;
    if (k < n) {
      const int im1 = k == 0 ? n - 1 : k - 1;
      const int ip1 = k == n - 1 ? 0 : k + 1;
      const int im2 = im1 == 0 ? n - 1 : im1 - 1;
      const int ip2 = ip1 == n - 1 ? 0 : ip1 + 1;
      const float x = vx[s], y = vy[s];
      const float xm = sx[im1], ym = sy[im1], xp = sx[ip1], yp = sy[ip1];
      const float xmm = sx[im2], ymm = sy[im2], xpp = sx[ip2], ypp = sy[ip2];
      const float ax = ka * (ym - yp), ay = ka * (xm - xp);
      const float lvx = xp - x, lvy = yp - y, lmx = x - xm, lmy = y - ym;
      const float len = sqrtf(lvx * lvx + lvy * lvy), lenm = sqrtf(lmx * lmx + lmy * lmy);
      // unit vectors and strains with reciprocals (within 1 ulp of the
      // reference's divisions)
      const float il = 1.0f / len, ilm = 1.0f / lenm;
      const float dl = len * cp.inv_l0 - 1.0f, dlm = lenm * cp.inv_l0 - 1.0f;
      const float px = cp.kL * (dl * (lvx * il) - dlm * (lmx * ilm));
      const float py = cp.kL * (dl * (lvy * il) - dlm * (lmy * ilm));
      const float six = lvx - lmx, siy = lvy - lmy;
      const float sixp = (xpp - xp) - lvx, siyp = (ypp - yp) - lvy;
      const float sixm = lmx - (xm - xmm), siym = lmy - (ym - ymm);
      const float bx = cp.Kb * (2.0f * six - sixm - sixp);
      const float by = cp.Kb * (2.0f * siy - siym - siyp);
      fx[s] = (ax + px) + bx;
      fy[s] = (ay + py) + by;
    }
  }

  // -- attraction and repulsion against the neighbour list (cells in
  // ascending order, as the reference loops over them).
  const int nnc = a.nn[c];
  const bool scan_all =
      nnc == kNbOverflow || *((volatile const int *)(a.stale + tid)) != 0;
  const int count = scan_all ? (T.cell_end - T.cell_begin) : nnc;
  const int *list = a.nbr + (size_t)c * kMaxNB2D;
  const bool att = T.Kat != 0.0f;
  // Lanes screen up to 32 list entries at once (one geometry load each, in
  // parallel); the cells that pass are then processed one by one, in list
  // order, with their geometry broadcast by shuffles.
  for (int base = 0; base < count; base += 32) {
    const int q = base + lane;
    int jl = -1;
    unsigned pflags = 0u;
    Geom2D gl;
    gl.cx = gl.cy = gl.R = gl.area = gl.minx = gl.maxx = gl.miny = gl.maxy = 0.0f;
    if (q < count) {
      jl = scan_all ? T.cell_begin + q : list[q];
      if (jl != c) {
        gl = a.geom_in[jl];
        const float dcx = gi.cx - gl.cx, dcy = gi.cy - gl.cy;
        const float rr = gi.R + gl.R;
        const float mm = kRelMargin * rr + kAbsMargin * (fabsf(gi.cx) + fabsf(gi.cy) +
                                                         fabsf(gl.cx) + fabsf(gl.cy));
        // own y range must meet (miny_j, maxy_j] unless y offsets can shift
        const bool yover = gi.maxy > gl.miny && gi.miny <= gl.maxy;
        const bool near = yover && dcx * dcx + dcy * dcy <= (rr + mm) * (rr + mm);
        const bool farx = pbc && (__fsub_rn(gi.maxx, gl.minx) > L || __fsub_rn(gl.maxx, gi.minx) > L);
        const bool fary = pbc && (__fsub_rn(gi.maxy, gl.miny) > L || __fsub_rn(gl.maxy, gi.miny) > L);
        const bool far = fary || (farx && yover);
        bool attp = false;
        if (att) {
          float ex = dcx, ey = dcy;
          if (pbc) {
            ex -= L * roundf(ex / L);
            ey -= L * roundf(ey / L);
          }
          const float ra = rr + cp.l0 + mm;
          attp = ex * ex + ey * ey <= ra * ra;
        }
        pflags = (near ? 1u : 0u) | (far ? 2u : 0u) | (attp ? 4u : 0u);
      }
    }
    unsigned pm = __ballot_sync(kFull, pflags != 0u);
    while (pm) {
    const int src = __ffs(pm) - 1;
    pm &= pm - 1u;
    const int j = __shfl_sync(kFull, jl, src);
    const unsigned fl = __shfl_sync(kFull, pflags, src);
    const bool near = fl & 1u, far = fl & 2u, attp = fl & 4u;
    Geom2D gj;
    gj.cx = __shfl_sync(kFull, gl.cx, src);
    gj.cy = __shfl_sync(kFull, gl.cy, src);
    gj.R = __shfl_sync(kFull, gl.R, src);
    gj.area = 0.0f;
    gj.minx = __shfl_sync(kFull, gl.minx, src);
    gj.maxx = __shfl_sync(kFull, gl.maxx, src);
    gj.miny = __shfl_sync(kFull, gl.miny, src);
    gj.maxy = __shfl_sync(kFull, gl.maxy, src);
    const float mm = kRelMargin * (gi.R + gj.R) +
                     kAbsMargin * (fabsf(gi.cx) + fabsf(gi.cy) + fabsf(gj.cx) + fabsf(gj.cy));

    unsigned cm[S], am[S];
    int code[S];
    bool anyc = false, anya = false, anyx = false;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      cm[s] = am[s] = 0u;
      code[s] = kNotCandidate;
      if (32 * s >= n) continue;  // empty slot (uniform over the warp)
      const int k = lane + 32 * s;
      bool ac = false;
      if (k < n) {
        if (!sf[k]) code[s] = vertex_candidate(vx[s], vy[s], gj, near, far, L);
        if (attp) {
          float ex = gj.cx - vx[s], ey = gj.cy - vy[s];
          if (pbc) {
            ex -= L * roundf(ex / L);
            ey -= L * roundf(ey / L);
          }
          const float ra = gj.R + cp.l0 + mm;
          ac = ex * ex + ey * ey <= ra * ra;
        }
      }
      cm[s] = __ballot_sync(kFull, code[s] == kCandidate);
      anyc |= cm[s] != 0u;
      anyx |= __any_sync(kFull, code[s] >= kCheckY);
      if (att) {
        am[s] = __ballot_sync(kFull, ac);
        anya |= am[s] != 0u;
      }
    }
    if (!anyc && !anya && !anyx) continue;
    const uint4 jr = *reinterpret_cast<const uint4 *>(a.cells + j);
    const int nj = (int)jr.y;
    const float2 *pj = a.pos_in + jr.x;
    if (anyx) {
      // kCheckY points are candidates only if a ring vertex has y offset
      // exactly -L; kCheckX points only if one has x offset within 8 ulp(L)
      // of L.  One point at a time, the lanes scan the ring.
      const float win = 8.0f * __int_as_float(__float_as_int(L) & 0x7f800000) * 0x1p-23f;
      float px[S], py[S];
#pragma unroll
      for (int s2 = 0; s2 < S; ++s2) {
        const int e = lane + 32 * s2;
        const float2 p = e < nj ? pj[e] : make_float2(0.0f, 0.0f);
        px[s2] = p.x;
        py[s2] = p.y;
      }
#pragma unroll
      for (int s = 0; s < S; ++s) {
        unsigned my = __ballot_sync(kFull, code[s] == kCheckY);
        unsigned mx = __ballot_sync(kFull, code[s] == kCheckX);
        while (my) {
          const int l = __ffs(my) - 1;
          my &= my - 1u;
          const float Y = __shfl_sync(kFull, vy[s], l);
          bool hit = false;
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2)
            hit |= lane + 32 * s2 < nj && __fsub_rn(Y, py[s2]) == -L;
          if (__ballot_sync(kFull, hit)) cm[s] |= 1u << l;
        }
        while (mx) {
          const int l = __ffs(mx) - 1;
          mx &= mx - 1u;
          const float X = __shfl_sync(kFull, vx[s], l);
          bool hit = false;
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2)
            hit |= lane + 32 * s2 < nj && fabsf(__fsub_rn(__fsub_rn(X, px[s2]), L)) <= win;
          if (__ballot_sync(kFull, hit)) cm[s] |= 1u << l;
        }
        anyc |= cm[s] != 0u;
      }
      if (!anyc && !anya) continue;
    }

    if (anya) {
      // stage the neighbour's ring for the per-vertex attraction loops
      for (int k = lane; k < nj; k += 32) {
        const float2 v = pj[k];
        nxs[k] = v.x;
        nys[k] = v.y;
      }
      __syncwarp();
      // AttractionForceUpdate (Cell2D_kernel.cl:251-267)
      const float kat = T.Kat / (float)n;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        if (!((am[s] >> lane) & 1u)) continue;
        for (int v = 0; v < nj; ++v) {
          float rx = nxs[v] - vx[s], ry = nys[v] - vy[s];
          if (pbc) {
            rx -= L * roundf(rx / L);
            ry -= L * roundf(ry / L);
          }
          const float dist = sqrtf(rx * rx + ry * ry);
          if (dist < cp.l0) {
            const float ftmp = kat * dist / cp.l0;
            float ux, uy;
            normalize2(rx, ry, ux, uy);
            fx[s] += ftmp * ux;
            fy[s] += ftmp * uy;
          }
        }
      }
    }
    if (anyc) {
      // RepulsionForceUpdate containment (Cell2D_kernel.cl:166-202):
      // lanes take the edges (P_e, P_{e-1}) of the neighbour, held in
      // registers for all candidates; a ballot gives the crossing parity.
      // Edges can be shifted only for "far" pairs, so the plain test is
      // used otherwise.
      float ex[S], ey[S], qx[S], qy[S];
#pragma unroll
      for (int s2 = 0; s2 < S; ++s2) {
        const int e = lane + 32 * s2;
        ex[s2] = ey[s2] = qx[s2] = qy[s2] = 0.0f;
        if (e < nj) {
          const float2 p = pj[e], pp = pj[e == 0 ? nj - 1 : e - 1];
          ex[s2] = p.x;
          ey[s2] = p.y;
          qx[s2] = pp.x;
          qy[s2] = pp.y;
        }
      }
#pragma unroll
      for (int s = 0; s < S; ++s) {
        unsigned msk = cm[s];
        while (msk) {
          const int l = __ffs(msk) - 1;
          msk &= msk - 1u;
          const float X = __shfl_sync(kFull, vx[s], l), Y = __shfl_sync(kFull, vy[s], l);
          unsigned par = 0u;
          if (far) {
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2)
              if (lane + 32 * s2 < nj)
                par ^= edge_crosses(X, Y, ex[s2], ey[s2], qx[s2], qy[s2], true, L);
          } else {
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2)
              if (lane + 32 * s2 < nj)
                par ^= edge_crosses(X, Y, ex[s2], ey[s2], qx[s2], qy[s2], false, L);
          }
          const unsigned bal = __ballot_sync(kFull, par != 0u);
          if ((__popc(bal) & 1) && lane == 0) sf[l + 32 * s] = 1;
        }
      }
    }
    __syncwarp();
    }
  }

  // -- repulsion force toward the own centre (Cell2D_kernel.cl:205-219)
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int k = lane + 32 * s;
    if (k < n && sf[k]) {
      float dx = gi.cx - vx[s], dy = gi.cy - vy[s];
      // d -= L*round(d/L); for |d| <= 0.49 L the rounded quotient is 0
      if (pbc && fabsf(dx) > 0.49f * L) dx -= L * roundf(dx / L);
      if (pbc && fabsf(dy) > 0.49f * L) dy -= L * roundf(dy / L);
      const float d2 = dx * dx + dy * dy;
      const float dist = sqrtf(d2);
      const float xij = dist * cp.inv_2r0;
      const float ftmp = T.Kre * (1.0f - xij);
      // normalize(d), with the zero vector mapped to itself
      const float inv = d2 == 0.0f ? 1.0f : 1.0f / dist;
      fx[s] += 0.5f * ftmp * (dx * inv);
      fy[s] += 0.5f * ftmp * (dy * inv);
    }
  }

  // -- Euler update (EulerUpdate, Cell2D_kernel.cl:279) and outputs
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int k = lane + 32 * s;
    if (k < n) {
      const float nxv = __fadd_rn(vx[s], __fmul_rn(fx[s], a.dt));
      const float nyv = __fadd_rn(vy[s], __fmul_rn(fy[s], a.dt));
      a.pos_out[cp.voff + k] = make_float2(nxv, nyv);
      if (a.force_out && write_out) a.force_out[cp.voff + k] = make_float2(fx[s], fy[s]);
      if (a.flags_out && write_out) a.flags_out[cp.voff + k] = sf[k];
      sx[k] = nxv;
      sy[k] = nyv;
    }
  }
  __syncwarp();

  // -- epilogue: geometry of the new positions for the next step
  const Geom2D g = ring_geom(sx, sy, n, lane);
  if (lane == 0) {
    a.geom_out[c] = g;
    if (!(isfinite(g.cx) && isfinite(g.cy) && isfinite(g.R))) atomicOr(a.err, 1);
    const Geom2D g0 = a.geom0[c];
    const float dc = sqrtf((g.cx - g0.cx) * (g.cx - g0.cx) + (g.cy - g0.cy) * (g.cy - g0.cy));
    float d = dc + fmaxf(0.0f, g.R - g0.R);
    d = fmaxf(d, fmaxf(fabsf(g.minx - g0.minx), fabsf(g.maxx - g0.maxx)));
    d = fmaxf(d, fmaxf(fabsf(g.miny - g0.miny), fabsf(g.maxy - g0.maxy)));
    if (!(d <= 0.5f * T.skin)) atomicOr(a.stale + tid, 1);
  }
}

// Static schedule: warp w of block b takes cell b*W + w.
template <int S, int W, int OCC>
__global__ void __launch_bounds__(W * 32, (StepOcc<S, W, OCC>::kBlocks))
    k2d_step(Step2DArgs a) {
  constexpr int M = 32 * S;
  __shared__ float sh_x[W][M], sh_y[W][M], sh_nx[W][M], sh_ny[W][M];
  __shared__ unsigned char sh_f[W][M];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * W + w;
  if (c >= a.ncells) return;
  step_cell<S>(a, c, lane, sh_x[w], sh_y[w], sh_nx[w], sh_ny[w], sh_f[w]);
}

// Dynamic schedule: a grid of exactly the resident blocks whose warps take
// the next cell from a counter until none is left.  The work per cell varies
// with its neighbours, so no warp idles while cells remain and no block is
// held resident by one slow warp.  The last warp to finish resets the two
// counters (next cell, finished warps) for the next launch.
template <int S, int W, int OCC>
__global__ void __launch_bounds__(W * 32, (StepOcc<S, W, OCC>::kBlocks))
    k2d_step_dyn(Step2DArgs a) {
  constexpr int M = 32 * S;
  __shared__ float sh_x[W][M], sh_y[W][M], sh_nx[W][M], sh_ny[W][M];
  __shared__ unsigned char sh_f[W][M];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    int c = 0;
    if (lane == 0) c = atomicAdd(a.sched, 1);
    c = __shfl_sync(kFull, c, 0);
    if (c >= a.ncells) break;
    step_cell<S>(a, c, lane, sh_x[w], sh_y[w], sh_nx[w], sh_ny[w], sh_f[w]);
    __syncwarp();
  }
  if (lane == 0) {
    const int warps = (int)gridDim.x * W;
    if (atomicAdd(a.sched + 1, 1) == warps - 1) {
      atomicExch(a.sched, 0);
      atomicExch(a.sched + 1, 0);
    }
  }
}

template <int S, int W, int OCC>
cudaError_t launch_step_sw(const Step2DArgs &a, bool dyn, cudaStream_t s) {
  if (dyn && a.sched) {
    // resident blocks per SM of this variant, and the device's SM count
    static int per_sm = 0, sms = 0;
    if (per_sm == 0) {
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, k2d_step_dyn<S, W, OCC>, W * 32, 0);
      if (e != cudaSuccess) return e;
      int dev = 0;
      e = cudaGetDevice(&dev);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      if (per_sm < 1) per_sm = 1;
    }
    const int need = (a.ncells + W - 1) / W;
    const int grid = need < per_sm * sms ? need : per_sm * sms;
    k2d_step_dyn<S, W, OCC><<<grid, W * 32, 0, s>>>(a);
    return cudaGetLastError();
  }
  const int grid = (a.ncells + W - 1) / W;
  k2d_step<S, W, OCC><<<grid, W * 32, 0, s>>>(a);
  return cudaGetLastError();
}

template <int S, int OCC>
cudaError_t launch_step_so(const Step2DArgs &a, int warps, bool dyn, cudaStream_t s) {
  // 16 warps of 8 slots would exceed the static shared-memory limit
  if (warps == 4) return launch_step_sw<S, 4, OCC>(a, dyn, s);
  if (warps == 16 && S <= 4) return launch_step_sw<S, (S <= 4 ? 16 : 8), OCC>(a, dyn, s);
  return launch_step_sw<S, 8, OCC>(a, dyn, s);
}

// variant bit 0: register cap for occupancy; bit 1: dynamic schedule
template <int S>
cudaError_t launch_step_s(const Step2DArgs &a, int warps, int variant, cudaStream_t s) {
  const bool dyn = (variant & 2) != 0;
  return (variant & 1) ? launch_step_so<S, 1>(a, warps, dyn, s)
                       : launch_step_so<S, 0>(a, warps, dyn, s);
}

} // namespace

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

cudaError_t launch_step2d(const Step2DArgs &a, int maxnv, int warps, int occ, cudaStream_t s) {
  if (maxnv <= 32) return launch_step_s<1>(a, warps, occ, s);
  if (maxnv <= 64) return launch_step_s<2>(a, warps, occ, s);
  if (maxnv <= 128) return launch_step_s<4>(a, warps, occ, s);
  return launch_step_s<8>(a, warps, occ, s);
}

} // namespace dpm
