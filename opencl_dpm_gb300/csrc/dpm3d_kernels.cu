// 3D DPM kernels for sm_103a.
//
// One thread block owns one cell per step and keeps the cell's mesh in
// shared memory.  A step is one fused kernel (k3d_step):
//   * centre of mass (from the previous step's epilogue) and volume (block
//     reduction over faces);
//   * volume, surface-area and substrate forces per vertex, gathered over
//     the vertex's incident faces in ascending face order -- the order in
//     which the reference's compare-and-swap adds reach a vertex when its
//     work-items run in order -- so no atomics are needed and the result is
//     deterministic (shaders/Cell3D_Kernel.cl:66-247);
//   * optional triangle bending (extension);
//   * repulsion by winding number against the cells of the neighbour list
//     (Cell3D_Kernel.cl:251-310): the neighbour's vertices are staged in
//     shared memory with the bounding spheres of their patches, candidate
//     vertices within its winding reach are compacted, and one warp decides
//     each candidate's winding number -- by a separating plane (outside) or
//     the neighbour's inner ball (inside), adding only the terms of the faces
//     the reference drops -- or defers it to a sum over every face that the
//     whole block evaluates (winding_at);
//   * opt-in AllVertAttraction (Cell3D_Kernel.cl:313-364);
//   * Euler update x += F*dt (Cell3D_Kernel.cl:371-381) and, as epilogue, the
//     centre, bounding radius, longest edge and inner ball of the new mesh for
//     the next step.
#include "dpm3d_kernels.cuh"

#include <math.h>

#include <mutex>

namespace dpm {

namespace {

// Threads per cell of k3d_step (NT): 512 (16 warps) by default -- the
// winding candidates of a cell (one warp each) are the bulk of the work, and
// a few hundred cells must fill 152 SMs (measured on the 256-cell monolayer
// at subdivision 3: 512 threads 27% faster than 256); meshes whose shared
// memory lets four or eight cells share an SM take 256 or 128 threads.
// Every block-wide sum is formed in the order of a 512-thread block
// (block_sum_v), so the block size changes no bit of the results.
// k3d_geom and k3d_diag run 512 threads.
constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kSumThreads = 512;
constexpr unsigned kFull = 0xffffffffu;

struct f3 {
  float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// normalize with the OpenCL special case: the zero vector maps to itself
// (one reciprocal square root for the three components; within the parity
// tolerance of the reference's divisions)
__device__ __forceinline__ f3 normalize(f3 a) {
  const float l2 = dot(a, a);
  if (l2 == 0.0f) return a;
  const float r = rsqrtf(l2);
  return mk(a.x * r, a.y * r, a.z * r);
}

// Block sum of per-thread partials, added as a kSumThreads-thread block
// adds them: v[r] is the partial of virtual thread threadIdx.x + r * NT (a
// block of NT threads runs kSumThreads / NT virtual threads per thread);
// the 32 virtual threads of a virtual warp are summed by the warp's
// butterfly, then the virtual warps' sums in order.
template <int NT>
__device__ float block_sum_v(const float (&v)[kSumThreads / NT], float *red) {
  constexpr int R = kSumThreads / NT;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float ws[R];
#pragma unroll
  for (int r = 0; r < R; ++r) ws[r] = warp_sum(v[r]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) red[w + r * (NT / 32)] = ws[r];
  }
  __syncthreads();
  float t = 0.0f;
  for (int i = 0; i < kSumThreads / 32; ++i) t += red[i];
  return t;
}
// NS block sums (each formed as block_sum_v forms it) and NM block maxima of
// per-thread values in one pass: two barriers instead of two per value.
// red holds 16 NS + (NT / 32) NM floats (at most 64).
template <int NT, int NS, int NM>
__device__ void block_reduce(const float (&sv)[NS][kSumThreads / NT], float (&so)[NS],
                             const float (&mv)[NM], float (&mo)[NM], float *red) {
  constexpr int R = kSumThreads / NT, VW = kSumThreads / 32, W = NT / 32;
  static_assert(NS * VW + NM * W <= 64, "reduction scratch");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float ws[NS][R], wm[NM];
#pragma unroll
  for (int k = 0; k < NS; ++k)
#pragma unroll
    for (int r = 0; r < R; ++r) ws[k][r] = warp_sum(sv[k][r]);
#pragma unroll
  for (int k = 0; k < NM; ++k) wm[k] = warp_max(mv[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NS; ++k)
#pragma unroll
      for (int r = 0; r < R; ++r) red[k * VW + w + r * W] = ws[k][r];
#pragma unroll
    for (int k = 0; k < NM; ++k) red[NS * VW + k * W + w] = wm[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    float t = 0.0f;
    for (int i = 0; i < VW; ++i) t += red[k * VW + i];
    so[k] = t;
  }
#pragma unroll
  for (int k = 0; k < NM; ++k) {
    float t = -INFINITY;
    for (int i = 0; i < W; ++i) t = fmaxf(t, red[NS * VW + k * W + i]);
    mo[k] = t;
  }
}

// Centre of mass (sum times 1/NV, Cell3D_Kernel.cl:35-44), bounding radius
// and longest edge of the mesh held in shared memory.
template <int NT, typename FaceIdx>
__device__ Geom3D mesh_geom(const float *px, const float *py, const float *pz, int nv,
                            const FaceIdx *faces, int nf, float *red) {
  constexpr int R = kSumThreads / NT;
  // pass 1: longest edge (maximum) and the vertex sums (centre)
  float e2[1] = {0.f};
  for (int f = threadIdx.x; f < nf; f += NT) {
    const int i0 = faces[3 * f], i1 = faces[3 * f + 1], i2 = faces[3 * f + 2];
    const int a[3] = {i0, i1, i2}, b[3] = {i1, i2, i0};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float dx = px[a[k]] - px[b[k]], dy = py[a[k]] - py[b[k]], dz = pz[a[k]] - pz[b[k]];
      e2[0] = fmaxf(e2[0], dx * dx + dy * dy + dz * dz);
    }
  }
  float sxyz[3][R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    sxyz[0][r] = sxyz[1][r] = sxyz[2][r] = 0.f;
    for (int v = threadIdx.x + r * NT; v < nv; v += kSumThreads) {
      sxyz[0][r] += px[v];
      sxyz[1][r] += py[v];
      sxyz[2][r] += pz[v];
    }
  }
  float sums[3], maxs[1];
  block_reduce<NT, 3, 1>(sxyz, sums, e2, maxs, red);
  const float inv = 1.0f / (float)nv;
  Geom3D g;
  g.cx = sums[0] * inv;
  g.cy = sums[1] * inv;
  g.cz = sums[2] * inv;
  g.emax = sqrtf(maxs[0]);
  // pass 2: bounding radius and the inner ball.  With the centre as
  // origin, face (a, b, c) has the triple product t = a.(b x c), whose sign
  // is the sign of the reference's face term at the centre, and its plane
  // lies |t| / |n| from the centre (n = (b - a) x (c - a)).  If every t has
  // the same sign and the solid angles sum to less than 8 pi (each is at
  // most area / plane distance^2), the mesh winds exactly once around the
  // centre, and no face comes closer than the smallest plane distance, so
  // the same holds in that ball.  (dmin is -1 once any face is degenerate,
  // whatever the order.)
  float mx[2] = {0.f, INFINITY};  // r2 and dmin (reduced as maxima of r2, -dmin)
  for (int v = threadIdx.x; v < nv; v += NT) {
    const float dx = px[v] - g.cx, dy = py[v] - g.cy, dz = pz[v] - g.cz;
    mx[0] = fmaxf(mx[0], dx * dx + dy * dy + dz * dz);
  }
  float bn[2][R];  // bound, count of positive triple products
#pragma unroll
  for (int r = 0; r < R; ++r) {
    bn[0][r] = bn[1][r] = 0.f;
    for (int f = threadIdx.x + r * NT; f < nf; f += kSumThreads) {
      const int i0 = faces[3 * f], i1 = faces[3 * f + 1], i2 = faces[3 * f + 2];
      const f3 a = mk(px[i0] - g.cx, py[i0] - g.cy, pz[i0] - g.cz);
      const f3 b = mk(px[i1] - g.cx, py[i1] - g.cy, pz[i1] - g.cz);
      const f3 c = mk(px[i2] - g.cx, py[i2] - g.cy, pz[i2] - g.cz);
      const f3 n = cross(b - a, c - a);
      const float nl = sqrtf(dot(n, n));
      const float t = dot(a, cross(b, c));
      const float d = fabsf(t) / nl;  // NaN or 0 for a degenerate face
      mx[1] = d > 0.0f ? fminf(mx[1], d) : -1.0f;
      bn[0][r] += 0.5f * nl / (d * d);
      bn[1][r] += t > 0.0f ? 1.0f : 0.0f;
    }
  }
  mx[1] = -mx[1];
  float s2[2], m2[2];
  block_reduce<NT, 2, 2>(bn, s2, mx, m2, red);
  g.R = sqrtf(m2[0]);
  const float dmin = -m2[1];
  const float bsum = s2[0], ns = s2[1];
  const bool one_sign = ns == (float)nf || ns == 0.0f;
  const bool ok = one_sign && dmin > 0.0f && bsum < 8.0f * (float)M_PI * 0.999f;
  g.rin = ok ? dmin * (1.0f - 1e-4f) : 0.0f;
  g.wind = ns == (float)nf ? 1.0f : -1.0f;
  g.pad0 = 0.0f;
  return g;
}

// Radius around a cell's centre beyond which the reference's winding number
// of a point is certainly below its 1e-6 threshold: outside the bounding
// sphere every face lies farther than the point's distance to the sphere,
// a face subtends more than pi steradians (denominator <= 0, dropped by the
// reference) only from within 1.155 * its circumradius <= 0.77 * its
// longest edge, and with no face dropped the sum over the closed mesh
// cancels to rounding noise.
__device__ __forceinline__ float winding_reach(const Geom3D &g) {
  return g.R + 1.05f * g.emax;
}

// Per-warp bit mask of a neighbour's vertices near the point under test,
// and the list of their ids (when they are at most kNearList).
constexpr int kNearWords = (kMaxNV3D + 31) / 32;
constexpr int kNearList = 32;
// Candidates whose winding number needs the sum over every face are summed
// by the whole block after the neighbour's other candidates, up to kDefer
// of them (more are summed by their warp).
constexpr int kDefer = 64;

// Shared-memory layout of k3d_step (see step3d_smem_bytes).  The staged
// neighbour (q*, pb), its candidate list and its geometry and centre (nbg, nbc)
// exist twice: the repulsion works on one buffer while it fills the other
// (staged_view selects one).
struct Smem3D {
  float4 *pb;  // bounding sphere (centre, radius) of each patch of the neighbour
  Geom3D *nbg; // the neighbour's geometry
  float4 *nbc; // the neighbour's centre, shifted to the image nearest this cell
  float *px, *py, *pz, *fx, *fy, *fz, *qx, *qy, *qz, *red;
  float *bnx, *bny, *bnz, *bnl, *bgx, *bgy, *bgz;
  int *ncand, *poff;
  unsigned *near;
  uint16_t *faces, *cand, *pvert, *nlist, *defer;
  float *terms; // [2][nf] face terms of a deferred candidate
  float *ex, *ey, *ez, *eL; // unit vector (lower id -> higher id) and length of each edge
  unsigned char *wnc;
  int qstride;  // floats from one staged buffer's q* to the other's
};

// Counters in Smem3D::ncand: the candidates of a neighbour and the next
// candidate to take, each rotating over three neighbours (a counter is zeroed
// one neighbour after its last read and two before its next write, with a
// barrier on either side), and the deferred candidates of a neighbour,
// alternating over two (the next neighbour's warps may add theirs while a
// slow thread still reads this one's count).  That is the pipelined loop of
// 512-thread blocks; the two-barrier loop of smaller blocks alternates the
// first two candidate counters and uses the first deferred counter.
constexpr int kCntCand = 0, kCntTake = 3, kCntDefer = 6, kNumCounters = 8;

__host__ __device__ __forceinline__ int q_region(int nv, int nf, int ne) {
  const int a = 6 * nv + 2 * nf, b = 4 * ne;
  return a > b ? a : b;
}

template <int NT>
__device__ __forceinline__ Smem3D carve(char *base, int nv, int nf, int ne, bool bend) {
  Smem3D s;
  s.pb = reinterpret_cast<float4 *>(base);
  s.nbg = reinterpret_cast<Geom3D *>(s.pb + 2 * kMaxPatches3D);
  s.nbc = reinterpret_cast<float4 *>(s.nbg + 2);
  float *f = reinterpret_cast<float *>(s.nbc + 2);
  s.px = f; f += nv;
  s.py = f; f += nv;
  s.pz = f; f += nv;
  s.fx = f; f += nv;
  s.fy = f; f += nv;
  s.fz = f; f += nv;
  // one region, two lives: the unit vectors and lengths of the mesh edges
  // while the shape forces are formed, then the staged neighbour and the
  // face terms of deferred candidates during the repulsion
  s.qx = f;
  s.qy = f + nv;
  s.qz = f + 2 * nv;
  s.qstride = 3 * nv;
  s.terms = f + 6 * nv;
  s.ex = f;
  s.ey = f + ne;
  s.ez = f + 2 * ne;
  s.eL = f + 3 * ne;
  f += q_region(nv, nf, ne);
  s.red = f; f += 64;
  s.near = reinterpret_cast<unsigned *>(f);
  f += (NT / 32) * kNearWords;
  if (bend) {
    s.bnx = f; f += nf;
    s.bny = f; f += nf;
    s.bnz = f; f += nf;
    s.bnl = f; f += nf;
    s.bgx = f; f += nf;
    s.bgy = f; f += nf;
    s.bgz = f; f += nf;
  } else {
    s.bnx = s.bny = s.bnz = s.bnl = s.bgx = s.bgy = s.bgz = nullptr;
  }
  s.ncand = reinterpret_cast<int *>(f);
  f += kNumCounters;
  s.poff = reinterpret_cast<int *>(f);
  f += kMaxPatches3D + 4;
  uint16_t *h = reinterpret_cast<uint16_t *>(f);
  s.faces = h;
  h += 3 * nf;
  s.cand = h;
  h += 2 * nv;
  s.pvert = h;
  h += nv;
  s.nlist = h;
  h += (NT / 32) * kNearList;
  s.defer = h;
  h += kDefer;
  s.wnc = reinterpret_cast<unsigned char *>(h);
  return s;
}

// The view of s whose staged neighbour (q*, pb, cand, nbg, nbc) is buffer b.
__device__ __forceinline__ Smem3D staged_view(const Smem3D &s, int b) {
  Smem3D v = s;
  const int o = b * s.qstride;
  v.qx += o;
  v.qy += o;
  v.qz += o;
  v.pb += b * kMaxPatches3D;
  v.nbg += b;
  v.nbc += b;
  v.cand += b * (s.qstride / 3);
  return v;
}

__device__ __forceinline__ f3 vtx(const Smem3D &s, int i) { return mk(s.px[i], s.py[i], s.pz[i]); }
__device__ __forceinline__ f3 nbv(const Smem3D &s, int i) { return mk(s.qx[i], s.qy[i], s.qz[i]); }
// unit vector of edge id g & 0x7fff, negated when bit 15 is set
__device__ __forceinline__ f3 edge_unit(const Smem3D &s, int g) {
  const int i = g & 0x7fff;
  const f3 n = mk(s.ex[i], s.ey[i], s.ez[i]);
  return (g & 0x8000) ? mk(-n.x, -n.y, -n.z) : n;
}

// RepellingForces' contribution of one hit (Cell3D_Kernel.cl:299-308): the
// vertex is pushed towards its own centre by |wn| Kc / 2.
__device__ __forceinline__ void repel(const Smem3D &s, int v, float wn, f3 C, f3 pt, float Kre) {
  const f3 dir = normalize(C - pt);
  const float sc = fabsf(wn) * 0.5f * Kre;
  s.fx[v] += sc * dir.x;
  s.fy[v] += sc * dir.y;
  s.fz[v] += sc * dir.z;
  s.wnc[v] = (unsigned char)min(255, s.wnc[v] + 1);
}

// One face term of the reference's winding sum (Cell3D_Kernel.cl:281-297):
// unit vectors from the point to the corners, the denominator of the
// triangle's half solid angle, and its numerator.
__device__ __forceinline__ void face_term(const Smem3D &s, int i0, int i1, int i2, f3 pt,
                                          float &num, float &denom) {
  const f3 u = normalize(nbv(s, i0) - pt), vv = normalize(nbv(s, i1) - pt),
           ww = normalize(nbv(s, i2) - pt);
  denom = 1.0f + dot(u, vv) + dot(vv, ww) + dot(ww, u);
  num = dot(u, cross(vv, ww));
}

__device__ __forceinline__ bool near_bit(const unsigned *m, int i) {
  return (m[i >> 5] >> (i & 31)) & 1u;
}

// Whether the plane through pt along the most outward-facing face around
// the nearest near vertex separates pt from every staged neighbour vertex
// (pt then lies outside the neighbour's convex hull).  Vertices are
// visited patch by patch as in winding_at; `span` bounds |q - pt|.
__device__ __forceinline__ bool face_plane_separates(const Smem3D &s, const Mesh3D &m, int NP,
                                                     f3 pt, float span, const uint16_t *nlist,
                                                     int nnear, int lane) {
  // nearest near vertex (lowest lane on ties)
  float dd = INFINITY;
  int k = 0;
  if (lane < nnear) {
    k = nlist[lane];
    const f3 d = nbv(s, k) - pt;
    dd = dot(d, d);
  }
  const float dbest = warp_min(dd);
  const int src = __ffs(__ballot_sync(kFull, dd == dbest)) - 1;
  const int k0 = __shfl_sync(kFull, k, src);
  // its incident face with the largest signed distance of pt
  float best = -INFINITY;
  f3 nb = mk(0.f, 0.f, 0.f);
  for (int e = m.inc_off[k0] + lane; e < m.inc_off[k0 + 1]; e += 32) {
    const int f = m.inc_face[e];
    const f3 a = nbv(s, s.faces[3 * f]), b = nbv(s, s.faces[3 * f + 1]),
             c = nbv(s, s.faces[3 * f + 2]);
    const f3 n = cross(b - a, c - a);
    const float l = sqrtf(dot(n, n));
    if (l > 0.0f) {
      const f3 nh = n / l;
      const float sd = dot(pt - a, nh);
      if (sd > best) {
        best = sd;
        nb = nh;
      }
    }
  }
  const float top = warp_max(best);
  if (!(top > 0.0f)) return false;
  const int win = __ffs(__ballot_sync(kFull, best == top)) - 1;
  const f3 n = mk(__shfl_sync(kFull, nb.x, win), __shfl_sync(kFull, nb.y, win),
                  __shfl_sync(kFull, nb.z, win));
  // every vertex must lie below the plane by the margin
  const float M = 1e-5f * (1.0f + span);
  bool need = false;
  if (lane < NP) {
    const float4 b = s.pb[lane];
    need = !(dot(mk(b.x, b.y, b.z) - pt, n) + b.w < -M);
  }
  unsigned todo = __ballot_sync(kFull, need);
  bool bad = false;
  while (todo) {
    const int p = __ffs(todo) - 1;
    todo &= todo - 1u;
    const int o = s.poff[p], cnt = s.poff[p + 1] - o;
    if (lane < cnt) bad |= !(dot(nbv(s, s.pvert[o + lane]) - pt, n) < -M);
  }
  return !__any_sync(kFull, bad);
}

// The reference's winding number of point pt with respect to the staged
// neighbour mesh (s.q*), as the sum over its faces of 2 atan2(num, denom) /
// 4 pi, leaving out faces with denom < 1e-8.  One warp; every lane returns
// the value.
//
// Over a closed mesh the full sum is 4 pi times the topological winding
// number, 0 for a point outside.  A face's term can be dropped (its solid
// angle is at least ~pi) only from within 1.155 r of the centre of its
// smallest enclosing circle (radius r <= longest edge / sqrt 3), i.e. within
// 1.25 x the mesh's longest edge of each of its corners.  So when a plane
// separates pt from every neighbour vertex (pt outside the convex hull), the
// reference's sum equals minus the sum of the dropped terms, up to the
// rounding of the reference's own summation: only faces with a corner near
// pt are evaluated.  Otherwise every face is summed as the reference does.
//
// The support and the near vertices are found patch by patch: a patch whose
// bounding sphere lies below the separating plane with the margin, and
// farther than the drop range from pt, cannot change either, so only the
// vertices of the other patches are visited.
__device__ __forceinline__ float winding_at(const Smem3D &s, const Mesh3D &m, int NV, int NF,
                                            int NP, f3 pt, f3 cj, const Geom3D &gj,
                                            unsigned *nearm, uint16_t *nlist, int lane,
                                            bool may_defer, bool &deferred) {
  deferred = false;
  const float four_pi = 4.0f * (float)M_PI;
  const float emax = gj.emax;
  const f3 du = pt - cj;
  const float r = sqrtf(dot(du, du));
  bool outside = false, inside = false;
  int nnear = 0;
  if (r > 0.0f) {
    // support of the neighbour's vertices along u = (pt - cj)/|pt - cj|,
    // and the vertices within the drop range of pt
    const f3 u = du / r;
    const float dn = 1.3f * emax;
    const float dn2 = dn * dn;
    if (lane < kNearWords) nearm[lane] = 0u;
    bool need = false;
    if (lane < NP) {
      // every vertex q of the patch has (q - cj).u <= (c - cj).u + radius
      // and |q - pt| >= |c - pt| - radius
      const float4 b = s.pb[lane];
      const f3 cp = mk(b.x, b.y, b.z);
      const float B = dot(cp - cj, u) + b.w;
      const f3 d = cp - pt;
      need = !(r > B + 1e-5f * (1.0f + r + fabsf(B))) ||
             !(sqrtf(dot(d, d)) > (b.w + dn) * (1.0f + 1e-5f));
    }
    unsigned todo = __ballot_sync(kFull, need);
    __syncwarp();
    float h = -INFINITY;
    while (todo) {
      const int p = __ffs(todo) - 1;
      todo &= todo - 1u;
      const int o = s.poff[p], n = s.poff[p + 1] - o;
      bool nr = false;
      int k = 0;
      if (lane < n) {
        k = s.pvert[o + lane];
        const f3 q = nbv(s, k);
        h = fmaxf(h, dot(q - cj, u));
        const f3 d = q - pt;
        nr = dot(d, d) <= dn2;
      }
      const unsigned bal = __ballot_sync(kFull, nr);
      if (nr) {
        atomicOr(nearm + (k >> 5), 1u << (k & 31));
        const int at = nnear + __popc(bal & ((1u << lane) - 1u));
        if (at < kNearList) nlist[at] = (uint16_t)k;
      }
      nnear += __popc(bal);
    }
    h = warp_max(h);
    // rounding of the dot products is far below this margin; with no patch
    // visited every patch already clears it
    outside = h == -INFINITY || r > h + 1e-5f * (1.0f + r + fabsf(h));
    __syncwarp();
    if (!outside && nnear <= kNearList) {
      const float mag = fabsf(pt.x) + fabsf(pt.y) + fabsf(pt.z) + fabsf(cj.x) + fabsf(cj.y) +
                        fabsf(cj.z);
      // inside the neighbour's inner ball: the mesh winds gj.wind times
      // around pt (the staged vertices differ from the neighbour's own by
      // the rounding of the periodic shift, covered by the mag term)
      inside = r < gj.rin - (1e-5f * (1.0f + r + gj.rin) + 1e-6f * mag);
      if (!inside && nnear > 0)
        outside = face_plane_separates(s, m, NP, pt, r + gj.R, nlist, nnear, lane);
    }
  }
  if ((outside || inside) && nnear <= kNearList) {
    // (near vertex, incident face) pairs, 32 at a time over the lanes;
    // each face once, at its lowest-numbered near corner
    float sum = 0.0f;
    int a0 = 0, e0 = 0, deg = 0;
    if (lane < nnear) {
      a0 = nlist[lane];
      e0 = m.inc_off[a0];
      deg = m.inc_off[a0 + 1] - e0;
    }
    int incl = deg;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    const int excl = incl - deg;
    for (int t0 = 0; t0 < total; t0 += 32) {
      const int t = t0 + lane;
      // the last near vertex whose pairs start at or before t
      int o = 0;
#pragma unroll
      for (int st = 16; st > 0; st >>= 1)
        if (__shfl_sync(kFull, excl, o + st) <= t) o += st;
      const int va = __shfl_sync(kFull, a0, o);
      const int ve = __shfl_sync(kFull, e0, o) + t - __shfl_sync(kFull, excl, o);
      if (t < total) {
        const int f = m.inc_face[ve];
        const int i0 = s.faces[3 * f], i1 = s.faces[3 * f + 1], i2 = s.faces[3 * f + 2];
        int low = NV;
        if (near_bit(nearm, i0)) low = min(low, i0);
        if (near_bit(nearm, i1)) low = min(low, i1);
        if (near_bit(nearm, i2)) low = min(low, i2);
        // A face subtends at most what the disc around its centroid through
        // its farthest corner subtends, and a disc of radius rho subtends
        // pi steradians or more only within rho of its centre: farther
        // away (here with a 25% margin) the reference's denominator is
        // clearly positive and the face is kept.
        const f3 A = nbv(s, i0), B = nbv(s, i1), Cc = nbv(s, i2);
        const f3 g = (1.0f / 3.0f) * (A + B + Cc);
        const f3 ga = A - g, gb = B - g, gc = Cc - g, gp = pt - g;
        const float rho2 = fmaxf(dot(ga, ga), fmaxf(dot(gb, gb), dot(gc, gc)));
        if (low == va && dot(gp, gp) <= 1.5625f * rho2) {
          float num, denom;
          face_term(s, i0, i1, i2, pt, num, denom);
          if (denom < 1e-8f) sum += 2.0f * atan2f(num, denom);
        }
      }
    }
    __syncwarp();
    return (inside ? gj.wind : 0.0f) - warp_sum(sum) / four_pi;
  }
  if (outside) {
    float sum = 0.0f;
    for (int wd = 0; wd < (NV + 31) / 32; ++wd) {
      unsigned bits = nearm[wd];
      while (bits) {
        const int a0 = wd * 32 + __ffs(bits) - 1;
        bits &= bits - 1u;
        const int e0 = m.inc_off[a0], e1 = m.inc_off[a0 + 1];
        for (int e = e0 + lane; e < e1; e += 32) {
          const int f = m.inc_face[e];
          const int i0 = s.faces[3 * f], i1 = s.faces[3 * f + 1], i2 = s.faces[3 * f + 2];
          // each face once: at its lowest-numbered near corner
          int low = NV;
          if (near_bit(nearm, i0)) low = min(low, i0);
          if (near_bit(nearm, i1)) low = min(low, i1);
          if (near_bit(nearm, i2)) low = min(low, i2);
          if (low != a0) continue;
          float num, denom;
          face_term(s, i0, i1, i2, pt, num, denom);
          if (denom < 1e-8f) sum += 2.0f * atan2f(num, denom);
        }
      }
    }
    __syncwarp();
    return -warp_sum(sum) / four_pi;
  }
  if (may_defer) {
    // the block sums it after this neighbour's candidates
    deferred = true;
    return 0.0f;
  }
  float part = 0.0f;
  for (int f = lane; f < NF; f += 32) {
    float num, denom;
    face_term(s, s.faces[3 * f], s.faces[3 * f + 1], s.faces[3 * f + 2], pt, num, denom);
    if (denom < 1e-8f) continue;
    part += 2.0f * atan2f(num, denom);
  }
  return warp_sum(part) / four_pi;
}

// Two blocks per SM by registers (64 a thread, no spills).
// Stages cell j's vertices, shifted to the periodic image nearest this cell,
// into s.q*, and the bounding spheres of its patches, from the same shifted
// coordinates, into s.pb (the whole block; no barrier).
template <int NT>
__device__ __forceinline__ void stage_neighbour(const Smem3D &s, const Step3DArgs &a, int j,
                                                f3 shift, int NV, int NP, int tid, int w,
                                                int lane) {
  const size_t bj = (size_t)j * NV;
  for (int k = tid; k < NV; k += NT) {
    s.qx[k] = a.xin[bj + k] + shift.x;
    s.qy[k] = a.yin[bj + k] + shift.y;
    s.qz[k] = a.zin[bj + k] + shift.z;
  }
  for (int p = w; p < NP; p += NT / 32) {
    const int o = s.poff[p], n = s.poff[p + 1] - o;
    f3 q = mk(0.f, 0.f, 0.f);
    if (lane < n) {
      const int k = s.pvert[o + lane];
      q = mk(a.xin[bj + k] + shift.x, a.yin[bj + k] + shift.y, a.zin[bj + k] + shift.z);
    }
    const float inv = 1.0f / (float)n;
    const f3 cp = mk(warp_sum(q.x) * inv, warp_sum(q.y) * inv, warp_sum(q.z) * inv);
    const f3 d = q - cp;
    const float rad = warp_max(lane < n ? sqrtf(dot(d, d)) : 0.0f);
    if (lane == 0) s.pb[p] = make_float4(cp.x, cp.y, cp.z, rad * (1.0f + 1e-6f));
  }
}

// Shift of cell j to its periodic image nearest the centre (cx, cy, cz).
__device__ __forceinline__ f3 image_shift(const Geom3D &gi, const Geom3D &gj, const Tissue3D &T) {
  if (!T.pbc) return mk(0.f, 0.f, 0.f);
  const float L = T.L;
  return mk(__fmul_rn(L, roundf(__fdiv_rn(__fsub_rn(gi.cx, gj.cx), L))),
            __fmul_rn(L, roundf(__fdiv_rn(__fsub_rn(gi.cy, gj.cy), L))),
            __fmul_rn(L, roundf(__fdiv_rn(__fsub_rn(gi.cz, gj.cz), L))));
}

// One ordered pair of AllVertAttraction as the reference computes it
// (Cell3D_Kernel.cl:339-361), seen from vertex p of the cell with rest
// length L0i: delta = q - p from the raw positions, wrapped by
// L*round(delta/L); -tmp(L0i) from this cell's visit and +tmp'(L0j), built on
// -delta, from the other cell's visit, each added to (fx, fy, fz) as the
// reference's atomics add them.
__device__ __forceinline__ void attract_pair(f3 p, f3 q, float L0i, float L0j, float Kat,
                                             float L, bool pbc, float &fx, float &fy,
                                             float &fz) {
  float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
  if (pbc) {
    dx = __fsub_rn(dx, __fmul_rn(L, roundf(__fdiv_rn(dx, L))));
    dy = __fsub_rn(dy, __fmul_rn(L, roundf(__fdiv_rn(dy, L))));
    dz = __fsub_rn(dz, __fmul_rn(L, roundf(__fdiv_rn(dz, L))));
  }
  const float dist =
      __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
  const float k2 = __fmul_rn(Kat, 0.5f);
  if (dist < L0i * 2.0f && dist > 1e-12f) {
    const float t = __fmul_rn(k2, __fsub_rn(__fdiv_rn(dist, L0i), 1.0f));
    fx = __fadd_rn(fx, -__fmul_rn(t, __fdiv_rn(dx, dist)));
    fy = __fadd_rn(fy, -__fmul_rn(t, __fdiv_rn(dy, dist)));
    fz = __fadd_rn(fz, -__fmul_rn(t, __fdiv_rn(dz, dist)));
  }
  if (dist < L0j * 2.0f && dist > 1e-12f) {
    const float t = __fmul_rn(k2, __fsub_rn(__fdiv_rn(dist, L0j), 1.0f));
    fx = __fadd_rn(fx, __fmul_rn(t, __fdiv_rn(-dx, dist)));
    fy = __fadd_rn(fy, __fmul_rn(t, __fdiv_rn(-dy, dist)));
    fz = __fadd_rn(fz, __fmul_rn(t, __fdiv_rn(-dz, dist)));
  }
}

// One winding candidate v of the staged neighbour (view sb: its mesh,
// centre cj and geometry gj), decided by one warp: the hit lands on v's
// force, or v is queued in sb.defer (counter *ndefer) for the block-wide
// full sum after the neighbour's other candidates (beyond kDefer of them
// the warp sums every face itself).
__device__ __forceinline__ void decide_candidate(const Smem3D &sb, const Mesh3D &m, int NV,
                                                 int NF, int NP, int v, f3 cj,
                                                 const Geom3D &gj, f3 C, float Kre,
                                                 unsigned *nearm, uint16_t *nlist, int lane,
                                                 int *ndefer) {
  const f3 pt = vtx(sb, v);
  bool deferred;
  float wn = winding_at(sb, m, NV, NF, NP, pt, cj, gj, nearm, nlist, lane, true, deferred);
  if (deferred) {
    int slot = 0;
    if (lane == 0) slot = atomicAdd(ndefer, 1);
    slot = __shfl_sync(kFull, slot, 0);
    if (slot < kDefer) {
      if (lane == 0) sb.defer[slot] = (uint16_t)v;
      return;
    }
    wn = winding_at(sb, m, NV, NF, NP, pt, cj, gj, nearm, nlist, lane, false, deferred);
  }
  if (lane == 0 && !(fabsf(wn) < 1e-6f)) repel(sb, v, wn, C, pt, Kre);
}

// The deferred candidates of the staged neighbour (view sb), one after the
// other: the block evaluates the face terms into a buffer, then one warp
// adds them up in the order of the warp-level sum (lane l: faces l, l + 32,
// ...; then the butterfly), so the result is the one that warp would give;
// two buffers let that warp add while the block evaluates the next.  The
// counter is zeroed after its last read.  Returns how many were summed (the
// last one's hit lands after the last barrier here).
template <int NT>
__device__ __forceinline__ int deferred_sums(const Smem3D &sb, int NF, int *ndefer, f3 C,
                                             float Kre, int tid, int w, int lane) {
  const int nd = min(*ndefer, kDefer);
  for (int d = 0; d < nd; ++d) {
    float *tb = sb.terms + (d & 1) * NF;
    const int v = sb.defer[d];
    const f3 pt = vtx(sb, v);
    for (int f = tid; f < NF; f += NT) {
      float num, denom;
      face_term(sb, sb.faces[3 * f], sb.faces[3 * f + 1], sb.faces[3 * f + 2], pt, num, denom);
      tb[f] = denom < 1e-8f ? 0.0f : 2.0f * atan2f(num, denom);
    }
    __syncthreads();
    if (tid == 0 && d == nd - 1) *ndefer = 0;
    if (w == d % (NT / 32)) {
      float part = 0.0f;
      for (int f = lane; f < NF; f += 32) part += tb[f];
      const float wn = warp_sum(part) / (4.0f * (float)M_PI);
      if (lane == 0 && !(fabsf(wn) < 1e-6f)) repel(sb, v, wn, C, pt, Kre);
    }
  }
  return nd;
}

template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k3d_step(Step3DArgs a) {
  constexpr int kW = NT / 32;  // warps per cell
  extern __shared__ __align__(16) char smem3d[];
  const int c = blockIdx.x;
  const int NV = a.mesh.nv, NF = a.mesh.nf;
  const bool bend_any = a.bend != 0;
  Smem3D s = carve<NT>(smem3d, NV, NF, a.mesh.ne, bend_any);
  const Cell3D P = a.cells[c];
  if (!P.active) return;  // an empty slot (uniform over the block)
  const Tissue3D T = a.tissues[P.tissue];
  const size_t base = (size_t)c * NV;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (a.step_index >= T.run_now) {
    // the tissue's step budget is spent: carry its state over unchanged
    for (int v = tid; v < NV; v += NT) {
      a.xout[base + v] = a.xin[base + v];
      a.yout[base + v] = a.yin[base + v];
      a.zout[base + v] = a.zin[base + v];
    }
    if (tid == 0) a.geom_out[c] = a.geom_in[c];
    return;
  }
  const bool write_out =
      a.all_forces != 0 || (a.step_index == T.run_now - 1 && T.steps_left == 0);

  for (int v = tid; v < NV; v += NT) {
    s.px[v] = a.xin[base + v];
    s.py[v] = a.yin[base + v];
    s.pz[v] = a.zin[base + v];
    s.wnc[v] = 0;
  }
  for (int i = tid; i < 3 * NF; i += NT) s.faces[i] = a.mesh.faces[i];
  const int NP = a.mesh.np;
  for (int i = tid; i < NV; i += NT) s.pvert[i] = a.mesh.pvert[i];
  if (tid <= NP) s.poff[tid] = a.mesh.poff[tid];
  if (tid < kNumCounters) s.ncand[tid] = 0;
  __syncthreads();

  const Geom3D gi = a.geom_in[c];
  const f3 C = mk(gi.cx, gi.cy, gi.cz);

  // volume (getVolume, Cell3D_Kernel.cl:46-64)
  float vpart[kSumThreads / NT];
#pragma unroll
  for (int r = 0; r < kSumThreads / NT; ++r) {
    vpart[r] = 0.0f;
    for (int f = tid + r * NT; f < NF; f += kSumThreads) {
      const f3 P0 = vtx(s, s.faces[3 * f]), P1 = vtx(s, s.faces[3 * f + 1]),
               P2 = vtx(s, s.faces[3 * f + 2]);
      vpart[r] += dot(cross(P0, P1), P2) / 6.0f;
    }
  }
  const float volume = fabsf(block_sum_v<NT>(vpart, s.red));
  const float kvol = -P.Kv * (volume / P.v0 - 1.0f);

  // edge pass of SurfaceAreaForceUpdate: every face term uses the unit
  // vector and length of its edges, formed here once per edge
  if (!(P.Ka < 1e-8f)) {
    for (int e = tid; e < a.mesh.ne; e += NT) {
      const f3 lv = vtx(s, a.mesh.eva[2 * e + 1]) - vtx(s, a.mesh.eva[2 * e]);
      const float L = sqrtf(dot(lv, lv));
      const f3 n = lv / L;
      s.ex[e] = n.x;
      s.ey[e] = n.y;
      s.ez[e] = n.z;
      s.eL[e] = L;
    }
  }
  // triangle bending, face pass (extension): unit normals, then G per face
  const bool bend = bend_any && P.Kb != 0.0f;
  if (bend) {
    for (int f = tid; f < NF; f += NT) {
      const f3 p0 = vtx(s, s.faces[3 * f]), p1 = vtx(s, s.faces[3 * f + 1]),
               p2 = vtx(s, s.faces[3 * f + 2]);
      const f3 n = cross(p1 - p0, p2 - p0);
      const float l = sqrtf(dot(n, n));
      const f3 nh = l > 0.0f ? n / l : mk(0.f, 0.f, 0.f);
      s.bnx[f] = nh.x;
      s.bny[f] = nh.y;
      s.bnz[f] = nh.z;
      s.bnl[f] = l;
    }
  }
  __syncthreads();
  if (bend) {
    for (int f = tid; f < NF; f += NT) {
      f3 G = mk(0.f, 0.f, 0.f);
      const float l = s.bnl[f];
      if (l != 0.0f) {
        const f3 nf = mk(s.bnx[f], s.bny[f], s.bnz[f]);
        for (int e = 0; e < 3; ++e) {
          const int g = a.mesh.adj[3 * f + e];
          if (g < 0) continue;
          const f3 ng = mk(s.bnx[g], s.bny[g], s.bnz[g]);
          const float cth = dot(nf, ng);
          G = G + (ng - cth * nf) / l;
        }
      }
      s.bgx[f] = G.x;
      s.bgy[f] = G.y;
      s.bgz[f] = G.z;
    }
    __syncthreads();
  }

  // per-vertex shape forces, in the reference's accumulation order
  const float range = P.adh;
  for (int v = tid; v < NV; v += NT) {
    f3 F = mk(0.f, 0.f, 0.f);
    const int e0 = a.mesh.inc_off[v], e1 = a.mesh.inc_off[v + 1];
    // VolumeForceUpdate (Cell3D_Kernel.cl:95-111)
    if (P.Kv != 0.0f) {
      for (int e = e0; e < e1; ++e) {
        const int f = a.mesh.inc_face[e], k = a.mesh.inc_corner[e];
        const f3 A = vtx(s, s.faces[3 * f + 1]) - C, B = vtx(s, s.faces[3 * f + 2]) - C,
                 Cc = vtx(s, s.faces[3 * f]) - C;
        const f3 g = k == 0 ? cross(A, B) : (k == 1 ? cross(B, Cc) : cross(Cc, A));
        F = F + (kvol * g) / 6.0f;
      }
    }
    // SurfaceAreaForceUpdate (Cell3D_Kernel.cl:129-176)
    if (!(P.Ka < 1e-8f)) {
      for (int e = e0; e < e1; ++e) {
        const int f = a.mesh.inc_face[e], k = a.mesh.inc_corner[e];
        // edge i runs from corner i to corner i+1: lv_i = p_{i+1} - p_i,
        // L_i = |lv_i|, n_i = lv_i / L_i (from the edge pass, negated when
        // the face runs the edge the other way)
        const int g0 = a.mesh.fedge[3 * f], g1 = a.mesh.fedge[3 * f + 1],
                  g2 = a.mesh.fedge[3 * f + 2];
        const float L0 = s.eL[g0 & 0x7fff], L1 = s.eL[g1 & 0x7fff], L2 = s.eL[g2 & 0x7fff];
        if (L0 < 1e-12f || L1 < 1e-12f || L2 < 1e-12f) continue;
        // corner k: g = d_k n_k - d_{k-1} n_{k-1}, d_i = L_i / l0 - 1
        const int ga = k == 0 ? g0 : (k == 1 ? g1 : g2);
        const int gb = k == 0 ? g2 : (k == 1 ? g0 : g1);
        const float La = k == 0 ? L0 : (k == 1 ? L1 : L2);
        const float Lb = k == 0 ? L2 : (k == 1 ? L0 : L1);
        const f3 na = edge_unit(s, ga), nb = edge_unit(s, gb);
        const float da = La / P.l0 - 1.0f, db = Lb / P.l0 - 1.0f;
        const f3 g = da * na - db * nb;
        F = F + P.sa_scale * g;
      }
    }
    // StickToSurface (Cell3D_Kernel.cl:196-246)
    if (!(P.Ks < 1e-12f)) {
      for (int e = e0; e < e1; ++e) {
        const int f = a.mesh.inc_face[e], k = a.mesh.inc_corner[e];
        const f3 p0 = vtx(s, s.faces[3 * f]), p1 = vtx(s, s.faces[3 * f + 1]),
                 p2 = vtx(s, s.faces[3 * f + 2]);
        // z of the unit normal (normalize's other components are unused)
        const f3 nn = cross(p1 - p0, p2 - p0);
        const float nl2 = dot(nn, nn);
        const float unz = nl2 == 0.0f ? nn.z : nn.z / sqrtf(nl2);
        if (!(unz < -0.1f)) continue;
        const f3 pos = k == 0 ? p0 : (k == 1 ? p1 : p2);
        if (pos.z < 0.0f) F.z += P.Ks * fabsf(pos.z);
        if (fabsf(pos.z) < range) {
          const f3 c2v = mk(pos.x, pos.y, 0.0f) - C;
          const float dd = sqrtf(0.0f * 0.0f + 0.0f * 0.0f + pos.z * pos.z);
          const float ftmp = (float)((double)P.Ks * (1.0 - (double)(dd / P.l0)));
          const f3 n = normalize(c2v);
          F = F + mk(n.x * ftmp, n.y * ftmp, n.z * ftmp);
        }
      }
    }
    // triangle bending, vertex gather (extension)
    if (bend) {
      for (int e = e0; e < e1; ++e) {
        const int f = a.mesh.inc_face[e], k = a.mesh.inc_corner[e];
        const f3 p0 = vtx(s, s.faces[3 * f]), p1 = vtx(s, s.faces[3 * f + 1]),
                 p2 = vtx(s, s.faces[3 * f + 2]);
        const f3 G = mk(s.bgx[f], s.bgy[f], s.bgz[f]);
        const f3 t = k == 0 ? cross(p1 - p2, G) : (k == 1 ? cross(p2 - p0, G) : cross(G, p1 - p0));
        F = F + P.Kb * t;
      }
    }
    s.fx[v] = F.x;
    s.fy[v] = F.y;
    s.fz[v] = F.z;
  }
  __syncthreads();

  // RepellingForces (Cell3D_Kernel.cl:251-310) over the neighbour list.
  // With 16 warps per cell (NT = 512) the neighbours within winding reach go
  // through two staging buffers: the warps take the candidates of the
  // neighbour in one buffer from a shared counter (one warp each; the first
  // by warp index), and every thread, once the counter runs dry, compacts
  // and stages its share of the next such neighbour into the other buffer;
  // one barrier closes both.  With fewer warps (many small-mesh cells, four
  // blocks per SM) each neighbour is staged, then its candidates taken in
  // warp order, with a barrier after each phase: there the pipeline measured
  // slower (4% on served pools of subdivision-2 requests).  Either way a
  // vertex is a candidate of a neighbour at most once and its hits land
  // neighbour by neighbour in list order (barriers separate them), so every
  // vertex sums its forces in the reference's order and both loops give the
  // same bits.
  if (T.Kre != 0.0f) {
    const int nnc = a.nn[c];
    const bool scan_all =
        nnc == kNbOverflow || *((volatile const int *)(a.stale + P.tissue)) != 0;
    const int count = scan_all ? (T.cell_end - T.cell_begin) : nnc;
    const int *list = a.nbr + (size_t)c * kMaxNB3D;
    if constexpr (NT == 512) {
      // the first listed neighbour at or after list position q whose winding
      // reach meets this cell (count when there is none), with its id, its
      // geometry and its shift to the periodic image nearest this cell
      auto next_in_reach = [&](int q, int &j, Geom3D &gj, f3 &shift) {
        for (; q < count; ++q) {
          j = scan_all ? T.cell_begin + q : list[q];
          if (j == c) continue;
          gj = a.geom_in[j];
          shift = image_shift(gi, gj, T);
          const f3 cj = mk(gj.cx + shift.x, gj.cy + shift.y, gj.cz + shift.z);
          const f3 dc = C - cj;
          const float mag = fabsf(cj.x) + fabsf(cj.y) + fabsf(cj.z) + fabsf(C.x) + fabsf(C.y) +
                            fabsf(C.z);
          const float reach = winding_reach(gj);
          const float rr = gi.R + reach + 1e-4f * (gi.R + reach) + 1e-5f * mag;
          if (dot(dc, dc) <= rr * rr) return q;
        }
        return count;
      };
      // this thread's share of neighbour k (id j) in buffer b: the candidate
      // vertices within its winding reach, its staged mesh and patch spheres,
      // its geometry and shifted centre
      auto fill = [&](int b, int k, int j, const Geom3D &gj, f3 shift) {
        const Smem3D sb = staged_view(s, b);
        const f3 cj = mk(gj.cx + shift.x, gj.cy + shift.y, gj.cz + shift.z);
        const float mag = fabsf(cj.x) + fabsf(cj.y) + fabsf(cj.z) + fabsf(C.x) + fabsf(C.y) +
                          fabsf(C.z);
        const float rj = winding_reach(gj) * (1.0f + 1e-4f) + 1e-5f * mag;
        int *cnt = s.ncand + kCntCand + k % 3;
        for (int v = tid; v < NV; v += NT) {
          const f3 d = vtx(s, v) - cj;
          if (dot(d, d) <= rj * rj) sb.cand[atomicAdd(cnt, 1)] = (uint16_t)v;
        }
        stage_neighbour<NT>(sb, a, j, shift, NV, NP, tid, w, lane);
        if (tid == 0) {
          sb.nbg[0] = gj;
          sb.nbc[0] = make_float4(cj.x, cj.y, cj.z, 0.0f);
        }
      };
      int j = 0;
      Geom3D gn;
      f3 shift;
      int q = next_in_reach(0, j, gn, shift);
      if (q < count) fill(0, 0, j, gn, shift);
      __syncthreads();
      for (int k = 0; q < count; ++k) {
        const Smem3D sb = staged_view(s, k & 1);
        const int ncand = s.ncand[kCntCand + k % 3];
        // the counters of neighbour k - 1: read before the last barrier,
        // written next for neighbour k + 2 after the coming one
        if (tid == 0) {
          s.ncand[kCntCand + (k + 2) % 3] = 0;
          s.ncand[kCntTake + (k + 2) % 3] = 0;
        }
        if (ncand > 0) {
          const Geom3D &gj = sb.nbg[0];
          const float4 c4 = sb.nbc[0];
          const f3 cj = mk(c4.x, c4.y, c4.z);
          unsigned *nearm = s.near + w * kNearWords;
          int *take = s.ncand + kCntTake + k % 3;
          bool first = true;
          for (;;) {
            int i = w;
            if (!first) {
              if (lane == 0) i = kW + atomicAdd(take, 1);
              i = __shfl_sync(kFull, i, 0);
            }
            first = false;
            if (i >= ncand) break;
            decide_candidate(sb, a.mesh, NV, NF, NP, sb.cand[i], cj, gj, C, T.Kre, nearm,
                             s.nlist + w * kNearList, lane, s.ncand + kCntDefer + (k & 1));
            __syncwarp();
          }
        }
        const int qn = next_in_reach(q + 1, j, gn, shift);
        if (qn < count) fill((k + 1) & 1, k + 1, j, gn, shift);
        __syncthreads();
        const int nd = deferred_sums<NT>(sb, NF, s.ncand + kCntDefer + (k & 1), C, T.Kre, tid,
                                         w, lane);
        // the last deferred hit lands before the next neighbour's hits
        if (nd > 0) __syncthreads();
        q = qn;
      }
    } else {
      int par = 0;
      for (int q = 0; q < count; ++q) {
        const int j = scan_all ? T.cell_begin + q : list[q];
        if (j == c) continue;
        const Geom3D gj = a.geom_in[j];
        const f3 shift = image_shift(gi, gj, T);
        const f3 cj = mk(gj.cx + shift.x, gj.cy + shift.y, gj.cz + shift.z);
        const f3 dc = C - cj;
        const float mag = fabsf(cj.x) + fabsf(cj.y) + fabsf(cj.z) + fabsf(C.x) + fabsf(C.y) +
                          fabsf(C.z);
        const float reach = winding_reach(gj);
        const float rr = gi.R + reach + 1e-4f * (gi.R + reach) + 1e-5f * mag;
        if (!(dot(dc, dc) <= rr * rr)) continue;
        // candidate compaction and staging of the neighbour's mesh (buffer
        // 0) in one phase.  Two candidate counters alternate between
        // neighbours: the one in use was zeroed during the previous
        // neighbour's evaluation, when nobody reads it.
        int *cnt = s.ncand + kCntCand + par;
        const float rj = reach * (1.0f + 1e-4f) + 1e-5f * mag;
        for (int v = tid; v < NV; v += NT) {
          const f3 d = vtx(s, v) - cj;
          if (dot(d, d) <= rj * rj) s.cand[atomicAdd(cnt, 1)] = (uint16_t)v;
        }
        stage_neighbour<NT>(s, a, j, shift, NV, NP, tid, w, lane);
        __syncthreads();
        const int ncand = *cnt;
        if (tid == 0) s.ncand[kCntCand + (par ^ 1)] = 0;
        par ^= 1;
        if (ncand > 0) {
          unsigned *nearm = s.near + w * kNearWords;
          for (int i = w; i < ncand; i += kW) {
            decide_candidate(s, a.mesh, NV, NF, NP, s.cand[i], cj, gj, C, T.Kre, nearm,
                             s.nlist + w * kNearList, lane, s.ncand + kCntDefer);
            __syncwarp();
          }
        }
        __syncthreads();
        deferred_sums<NT>(s, NF, s.ncand + kCntDefer, C, T.Kre, tid, w, lane);
      }
      // the last deferred sum's force lands after the loop's last barrier
      __syncthreads();
    }
  }

  // AllVertAttraction (Cell3D_Kernel.cl:313-364), opt-in (Kat != 0): after
  // the repulsion, every vertex gathers its pairs with the vertices of the
  // cells on the list, neighbour by neighbour and patch by patch.  Pairs are
  // skipped only where the reference's own test must fail: beyond
  // 2 max(l0_i, l0_j) (with margins for the rounding of the periodic shift),
  // judged in the frame of the centres' nearest image when every vertex pair
  // of the two cells lies within L/2 of it on each axis (so the reference's
  // per-pair wrap picks that same image); otherwise every pair is evaluated.
  if (T.Kat != 0.0f) {
    const int nnc = a.nn[c];
    const bool scan_all =
        nnc == kNbOverflow || *((volatile const int *)(a.stale + P.tissue)) != 0;
    const int count = scan_all ? (T.cell_end - T.cell_begin) : nnc;
    const int *list = a.nbr + (size_t)c * kMaxNB3D;
    const float L = T.L;
    const float L0i = fmaxf(P.l0, 1e-12f);
    for (int q = 0; q < count; ++q) {
      const int j = scan_all ? T.cell_begin + q : list[q];
      if (j == c) continue;
      const Geom3D gj = a.geom_in[j];
      const f3 shift = image_shift(gi, gj, T);
      const f3 cj = mk(gj.cx + shift.x, gj.cy + shift.y, gj.cz + shift.z);
      const f3 dc = C - cj;
      const float mag = fabsf(cj.x) + fabsf(cj.y) + fabsf(cj.z) + fabsf(C.x) + fabsf(C.y) +
                        fabsf(C.z);
      const float L0j = fmaxf(a.cells[j].l0, 1e-12f);
      const float range = 2.0f * fmaxf(L0i, L0j) * (1.0f + 1e-4f) + 1e-5f * mag;
      const float rr = (gi.R + gj.R) * (1.0f + 1e-4f) + range;
      if (!(dot(dc, dc) <= rr * rr)) continue;
      const float ext = gi.R + gj.R + range;
      const bool prune = !T.pbc || (fabsf(dc.x) + ext < 0.49f * L &&
                                    fabsf(dc.y) + ext < 0.49f * L &&
                                    fabsf(dc.z) + ext < 0.49f * L);
      stage_neighbour<NT>(s, a, j, shift, NV, NP, tid, w, lane);
      __syncthreads();
      const size_t bj = (size_t)j * NV;
      const float range2 = range * range;
      for (int v = tid; v < NV; v += NT) {
        const f3 p = vtx(s, v);
        const f3 d0 = p - cj;
        const float rj = gj.R * (1.0f + 1e-4f) + range;
        if (prune && !(dot(d0, d0) <= rj * rj)) continue;
        float fx = s.fx[v], fy = s.fy[v], fz = s.fz[v];
        for (int pp = 0; pp < NP; ++pp) {
          if (prune) {
            const float4 b = s.pb[pp];
            const f3 d = p - mk(b.x, b.y, b.z);
            const float rp = b.w + range;
            if (!(dot(d, d) <= rp * rp)) continue;
          }
          const int o = s.poff[pp], n = s.poff[pp + 1] - o;
          for (int i = 0; i < n; ++i) {
            const int k = s.pvert[o + i];
            if (prune) {
              const f3 d = nbv(s, k) - p;
              if (!(dot(d, d) <= range2)) continue;
            }
            const f3 qr = mk(a.xin[bj + k], a.yin[bj + k], a.zin[bj + k]);
            attract_pair(p, qr, L0i, L0j, T.Kat, L, T.pbc != 0, fx, fy, fz);
          }
        }
        s.fx[v] = fx;
        s.fy[v] = fy;
        s.fz[v] = fz;
      }
      __syncthreads();
    }
  }

  // EulerPosition (Cell3D_Kernel.cl:371-381) and outputs
  for (int v = tid; v < NV; v += NT) {
    const float nx = __fadd_rn(s.px[v], __fmul_rn(s.fx[v], a.dt));
    const float ny = __fadd_rn(s.py[v], __fmul_rn(s.fy[v], a.dt));
    const float nz = __fadd_rn(s.pz[v], __fmul_rn(s.fz[v], a.dt));
    a.xout[base + v] = nx;
    a.yout[base + v] = ny;
    a.zout[base + v] = nz;
    if (a.fx && write_out) {
      a.fx[base + v] = s.fx[v];
      a.fy[base + v] = s.fy[v];
      a.fz[base + v] = s.fz[v];
    }
    if (a.wn_out && write_out) a.wn_out[base + v] = s.wnc[v];
    s.px[v] = nx;
    s.py[v] = ny;
    s.pz[v] = nz;
  }
  __syncthreads();
  const Geom3D g = mesh_geom<NT>(s.px, s.py, s.pz, NV, s.faces, NF, s.red);
  if (tid == 0) {
    a.geom_out[c] = g;
    if (!(isfinite(g.cx) && isfinite(g.cy) && isfinite(g.cz) && isfinite(g.R)))
      atomicOr(a.err, 1);
    // the list stays valid while every cell's winding reach moved by at
    // most skin/2 (centre shift plus growth of R + 1.05 emax)
    const Geom3D g0 = a.geom0[c];
    const float dx = g.cx - g0.cx, dy = g.cy - g0.cy, dz = g.cz - g0.cz;
    const float d = sqrtf(dx * dx + dy * dy + dz * dz) +
                    fmaxf(0.0f, winding_reach(g) - winding_reach(g0)) + fmaxf(0.0f, g.R - g0.R);
    if (!(d <= 0.5f * T.skin)) atomicOr(a.stale + P.tissue, 1);
  }
}

__global__ void __launch_bounds__(kThreads)
    k3d_geom(const float *x, const float *y, const float *z, const uint16_t *faces, int nf,
             const Cell3D *cells, Geom3D *geom, int nv) {
  __shared__ float px[kMaxNV3D], py[kMaxNV3D], pz[kMaxNV3D], red[64];
  if (!cells[blockIdx.x].active) return;  // an empty slot
  const size_t base = (size_t)blockIdx.x * nv;
  for (int v = threadIdx.x; v < nv; v += kThreads) {
    px[v] = x[base + v];
    py[v] = y[base + v];
    pz[v] = z[base + v];
  }
  __syncthreads();
  const Geom3D g = mesh_geom<kThreads>(px, py, pz, nv, faces, nf, red);
  if (threadIdx.x == 0) geom[blockIdx.x] = g;
}

// ---------------------------------------------------------------------------
// Diagnostics (double precision, one block per cell)
// ---------------------------------------------------------------------------

__device__ double block_sum_d(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double r = 0.0;
  for (int i = 0; i < kWarps; ++i) r += red[i];
  return r;
}

// Per cell: enclosed volume, surface area and the energy
// Kv/2 (V/v0 - 1)^2 + Ka/2 sum_edges (l/l0 - 1)^2 + Kb sum_edges (1 - n1.n2)
// (project-defined; the reference defines no energy), all in double.
__global__ void __launch_bounds__(kThreads)
    k3d_diag(const float *x, const float *y, const float *z, Mesh3D mesh, const Cell3D *cells,
             double *out, int nv) {
  __shared__ double red[kWarps];
  const Cell3D P = cells[blockIdx.x];
  double *o = out + 3 * (size_t)blockIdx.x;
  if (!P.active) {
    if (threadIdx.x == 0) o[0] = o[1] = o[2] = 0.0;
    return;
  }
  const size_t base = (size_t)blockIdx.x * nv;
  auto vd = [&](int i) {
    return make_double3((double)x[base + i], (double)y[base + i], (double)z[base + i]);
  };
  auto normal = [&](int f, double3 &n) {
    const double3 a = vd(mesh.faces[3 * f]), b = vd(mesh.faces[3 * f + 1]),
                  d = vd(mesh.faces[3 * f + 2]);
    const double ux = b.x - a.x, uy = b.y - a.y, uz = b.z - a.z;
    const double wx = d.x - a.x, wy = d.y - a.y, wz = d.z - a.z;
    n = make_double3(uy * wz - uz * wy, uz * wx - ux * wz, ux * wy - uy * wx);
    return sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
  };
  double V = 0.0, A = 0.0, Ue = 0.0, Eb = 0.0;
  for (int f = threadIdx.x; f < mesh.nf; f += kThreads) {
    const int i0 = mesh.faces[3 * f], i1 = mesh.faces[3 * f + 1], i2 = mesh.faces[3 * f + 2];
    const double3 a = vd(i0), b = vd(i1), d = vd(i2);
    V += a.x * (b.y * d.z - b.z * d.y) + a.y * (b.z * d.x - b.x * d.z) +
         a.z * (b.x * d.y - b.y * d.x);
    double3 n;
    const double ln = normal(f, n);
    A += 0.5 * ln;
    const double3 e[3] = {a, b, d};
    for (int k = 0; k < 3; ++k) {
      const double3 s = e[k], q = e[(k + 1) % 3];
      const double l =
          sqrt((q.x - s.x) * (q.x - s.x) + (q.y - s.y) * (q.y - s.y) + (q.z - s.z) * (q.z - s.z));
      const double dl = l / (double)P.l0 - 1.0;
      Ue += 0.5 * dl * dl;  // each edge is seen from both of its faces
      if (P.Kb != 0.0f) {
        const int g = mesh.adj[3 * f + k];
        if (g > f) {  // each edge once; a degenerate face has normal 0
          double3 m;
          const double lm = normal(g, m);
          const double cth =
              ln > 0.0 && lm > 0.0 ? (n.x * m.x + n.y * m.y + n.z * m.z) / (ln * lm) : 0.0;
          Eb += 1.0 - cth;
        }
      }
    }
  }
  V = block_sum_d(V, red);
  A = block_sum_d(A, red);
  Ue = block_sum_d(Ue, red);
  Eb = block_sum_d(Eb, red);
  if (threadIdx.x == 0) {
    V = fabs(V) / 6.0;
    const double dv = V / (double)P.v0 - 1.0;
    o[0] = V;
    o[1] = A;
    o[2] = 0.5 * (double)P.Kv * dv * dv + 0.5 * (double)P.Ka * Ue + (double)P.Kb * Eb;
  }
}

// ---------------------------------------------------------------------------
// Cell list (3D): periodic bins of the centres, sorted keys, neighbour lists
// ---------------------------------------------------------------------------

__device__ __forceinline__ int bin3(float x, float L, float inv, int nb) {
  const float wx = __fsub_rn(x, __fmul_rn(L, floorf(__fdiv_rn(x, L))));
  const int b = (int)floorf(__fmul_rn(wx, inv));
  return max(0, min(b, nb - 1));
}

__global__ void __launch_bounds__(256) k3d_binprep(Rebuild3DArgs a, int local_bits) {
  __shared__ float red[64];
  const int t = blockIdx.x;
  const Tissue3D T = a.tissues[t];
  float dmax = 0.0f;
  for (int c = T.cell_begin + threadIdx.x; c < T.cell_end; c += blockDim.x) {
    const Geom3D g = a.geom[c];
    dmax = fmaxf(dmax, fmaxf(2.0f * winding_reach(g), 2.0f * g.R + T.arange));
  }
  dmax = warp_max(dmax);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dmax;
  __syncthreads();
  float m = 0.0f;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = fmaxf(m, red[i]);
  float wdt = __fadd_rn(__fadd_rn(m, T.skin), __fadd_rn(__fmul_rn(1e-3f, m), __fmul_rn(1e-5f, T.L)));
  int nb = (int)floorf(__fdiv_rn(T.L, wdt));
  nb = max(1, min(nb, T.cap));
  if (threadIdx.x == 0) {
    a.tissues[t].nb = nb;
    a.tissues[t].binw = wdt;
    a.stale[t] = 0;
    // the tissue's share of the rebuild period that follows
    if (a.block_len > 0) {
      const int run = min(T.steps_left, a.block_len);
      a.tissues[t].run_now = run;
      if (T.steps_left < kStepsUnlimited) a.tissues[t].steps_left = T.steps_left - run;
    }
  }
  const float inv = __fdiv_rn((float)nb, T.L);
  for (int c = T.cell_begin + threadIdx.x; c < T.cell_end; c += blockDim.x) {
    const Geom3D g = a.geom[c];
    const int bx = bin3(g.cx, T.L, inv, nb), by = bin3(g.cy, T.L, inv, nb),
              bz = bin3(g.cz, T.L, inv, nb);
    a.keys[c] = ((uint32_t)t << local_bits) | (uint32_t)((bz * nb + by) * nb + bx);
    a.vals[c] = (uint32_t)c;
  }
  // empty slots sort after the tissue's cells
  for (int c = T.cell_end + threadIdx.x; c < T.cell_cap; c += blockDim.x) {
    a.keys[c] = ((uint32_t)t << local_bits) | ((1u << local_bits) - 1u);
    a.vals[c] = (uint32_t)c;
  }
}

constexpr int kNb3Warps = 8;
constexpr int kNb3Buf = 128;

__device__ __forceinline__ int lb_u32(const uint32_t *a, int lo, int hi, uint32_t key) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ bool pair3(const Geom3D &gi, const Geom3D &gj, const Tissue3D &T) {
  float dx = __fsub_rn(gi.cx, gj.cx), dy = __fsub_rn(gi.cy, gj.cy), dz = __fsub_rn(gi.cz, gj.cz);
  if (T.pbc) {
    dx = __fsub_rn(dx, __fmul_rn(T.L, roundf(__fdiv_rn(dx, T.L))));
    dy = __fsub_rn(dy, __fmul_rn(T.L, roundf(__fdiv_rn(dy, T.L))));
    dz = __fsub_rn(dz, __fmul_rn(T.L, roundf(__fdiv_rn(dz, T.L))));
  }
  const float mag = __fadd_rn(__fadd_rn(__fadd_rn(fabsf(gi.cx), fabsf(gi.cy)), fabsf(gi.cz)), T.L);
  // vertices of i (within R_i) that can reach j (within its winding reach),
  // or the other way round; with the attraction, vertex pairs within its
  // range
  const float ri = winding_reach(gi), rj = winding_reach(gj);
  const float span = fmaxf(fmaxf(__fadd_rn(gi.R, rj), __fadd_rn(gj.R, ri)),
                           __fadd_rn(__fadd_rn(gi.R, gj.R), T.arange));
  const float m = __fadd_rn(__fmul_rn(1e-3f, span), __fmul_rn(1e-4f, mag));
  const float r = __fadd_rn(__fadd_rn(span, T.skin), m);
  const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  return d2 <= __fmul_rn(r, r);
}

__global__ void __launch_bounds__(kNb3Warps * 32) k3d_neighbors(Rebuild3DArgs a, int local_bits) {
  __shared__ int buf[kNb3Warps][kNb3Buf];
  __shared__ unsigned char uniq[kNb3Warps][kNb3Buf];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * kNb3Warps + w;
  if (c >= a.ncells) return;
  if (!a.cells[c].active) {  // an empty slot
    if (lane == 0) a.nn[c] = 0;
    return;
  }
  const int t = (int)a.cells[c].tissue;
  const Tissue3D T = a.tissues[t];
  const Geom3D gi = a.geom[c];
  const unsigned lt = (1u << lane) - 1u;
  const int nb = T.nb;
  const float inv = __fdiv_rn((float)nb, T.L);
  const int bx = bin3(gi.cx, T.L, inv, nb), by = bin3(gi.cy, T.L, inv, nb),
            bz = bin3(gi.cz, T.L, inv, nb);
  // lane l finds the sorted range of the l-th neighbouring bin (the
  // searches run side by side), then their cells are tested in bin order,
  // 32 at a time
  const int lo_off = nb >= 3 ? -1 : 0, hi_off = nb >= 3 ? 1 : nb - 1;
  const int nax = hi_off - lo_off + 1, nbins = nax * nax * nax;  // at most 27
  int blo = 0, bhi = 0;
  if (lane < nbins) {
    const int oz = lo_off + lane / (nax * nax), oy = lo_off + (lane / nax) % nax,
              ox = lo_off + lane % nax;
    const int xx = (bx + ox + nb) % nb, yy = (by + oy + nb) % nb, zz = (bz + oz + nb) % nb;
    const uint32_t key = ((uint32_t)t << local_bits) | (uint32_t)((zz * nb + yy) * nb + xx);
    blo = lb_u32(a.sorted_keys, T.cell_begin, T.cell_end, key);
    bhi = lb_u32(a.sorted_keys, blo, T.cell_end, key + 1u);
  }
  int cnt = 0;
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
    const bool ok = j >= 0 && j != c && pair3(gi, a.geom[j], T);
    const unsigned m = __ballot_sync(kFull, ok);
    const int pos = cnt + __popc(m & lt);
    if (ok && pos < kNb3Buf) buf[w][pos] = j;
    cnt += __popc(m);
  }
  __syncwarp();
  int nout;
  if (cnt > kNb3Buf) {
    nout = kNbOverflow;
  } else {
    for (int i = lane; i < cnt; i += 32) {
      const int v = buf[w][i];
      bool first = true;
      for (int k = 0; k < i; ++k) first &= buf[w][k] != v;
      uniq[w][i] = first ? 1 : 0;
    }
    __syncwarp();
    int nu = 0;
    for (int i = 0; i < cnt; ++i) nu += uniq[w][i];
    if (nu > kMaxNB3D) {
      nout = kNbOverflow;
    } else {
      int *out = a.nbr + (size_t)c * kMaxNB3D;
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

} // namespace

size_t step3d_smem_bytes(int nv, int nf, int ne, bool bend, int threads) {
  const size_t warps = (size_t)threads / 32;
  size_t floats = (size_t)6 * nv + (size_t)q_region(nv, nf, ne) + 64 + warps * kNearWords +
                  (bend ? (size_t)7 * nf : 0) + kNumCounters + kMaxPatches3D + 4;
  size_t halves = (size_t)3 * nf + 3 * (size_t)nv + warps * kNearList + kDefer;
  return sizeof(float4) * (2 * kMaxPatches3D + 6) + floats * 4 + halves * 2 + (size_t)nv + 16;
}

int step3d_threads(int nv, int nf, int ne, bool bend, int ncells, int sm_count) {
  // A cell's step is latency-bound: while two 512-thread blocks per SM hold
  // every cell, 16 warps per cell finish soonest; with more cells, 256
  // threads let four cells share an SM when their shared memory fits in its
  // 228 KB (1 KB reserved per block).  Measured on subdivision-2 batches of
  // 1,660-2,048 cells: 256 threads 14-17% faster; on 64-256 cells, or at
  // subdivision 3 (98 KB per block), 512 faster.
  const size_t b256 = step3d_smem_bytes(nv, nf, ne, bend, 256) + 1024;
  const bool four_fit = 4 * b256 <= (size_t)228 * 1024;
  return four_fit && ncells > 2 * sm_count ? 256 : 512;
}

// The kernels' dynamic shared-memory limit is a per-device attribute shared
// by every batch: it is only ever raised, so a batch of a smaller mesh made
// after a larger one does not lower it under the larger one's launches.
cudaError_t prepare_step3d(int nv, int nf, int ne, bool bend) {
  static std::mutex mu;
  static size_t granted[64] = {0};
  // the 512-thread block needs the most; the smaller ones get the same limit
  const size_t bytes = step3d_smem_bytes(nv, nf, ne, bend, 512);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (dev >= 0 && dev < 64 && bytes <= granted[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(k3d_step<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k3d_step<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k3d_step<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes);
  if (e == cudaSuccess && dev >= 0 && dev < 64) granted[dev] = bytes;
  return e;
}

cudaError_t launch_step3d(const Step3DArgs &a, int threads, cudaStream_t s) {
  const size_t bytes = step3d_smem_bytes(a.mesh.nv, a.mesh.nf, a.mesh.ne, a.bend != 0, threads);
  switch (threads) {
    case 128: k3d_step<128><<<a.ncells, 128, bytes, s>>>(a); break;
    case 256: k3d_step<256><<<a.ncells, 256, bytes, s>>>(a); break;
    case 512: k3d_step<512><<<a.ncells, 512, bytes, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_diag3d(const float *x, const float *y, const float *z, const Mesh3D &mesh,
                          const Cell3D *cells, double *out, int ncells, cudaStream_t s) {
  k3d_diag<<<ncells, kThreads, 0, s>>>(x, y, z, mesh, cells, out, mesh.nv);
  return cudaGetLastError();
}

cudaError_t launch_geom3d(const float *x, const float *y, const float *z, const Mesh3D &mesh,
                          const Cell3D *cells, Geom3D *geom, int ncells, cudaStream_t s) {
  k3d_geom<<<ncells, kThreads, 0, s>>>(x, y, z, mesh.faces, mesh.nf, cells, geom, mesh.nv);
  return cudaGetLastError();
}

cudaError_t launch_binprep3d(const Rebuild3DArgs &a, int local_bits, cudaStream_t s) {
  k3d_binprep<<<a.ntissues, 256, 0, s>>>(a, local_bits);
  return cudaGetLastError();
}

cudaError_t launch_neighbors3d(const Rebuild3DArgs &a, int local_bits, cudaStream_t s) {
  k3d_neighbors<<<(a.ncells + kNb3Warps - 1) / kNb3Warps, kNb3Warps * 32, 0, s>>>(a, local_bits);
  return cudaGetLastError();
}

} // namespace dpm
