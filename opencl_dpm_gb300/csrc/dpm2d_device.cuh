// Device helpers shared by the 2D kernels: the reference's crossing test,
// the conservative candidate tests, ring geometry.  Included by the
// translation units of the 2D kernels; everything is internal to each.
#pragma once

#include <math.h>

#include "dpm2d_kernels.cuh"

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

} // namespace
} // namespace dpm
