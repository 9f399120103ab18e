/*
 * CPU oracle for the Deformable Particle Model time step (plain C, OpenMP).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, the smoke check
 * and the CPU baseline of the benchmark.  The product never links it.
 *
 * This restates the reference algorithm function by function.  Each routine
 * cites the reference lines it follows; the arithmetic keeps the reference's
 * evaluation order and precision, including the places where an unsuffixed
 * double literal (0.5, 1.0, 2.0) promotes a float expression to double on an
 * fp64-capable OpenCL device, so that on the same inputs it reproduces the
 * reference bit for bit when both are built with -ffp-contract=off.  Work
 * that the reference repeats per work-item with identical results (the area
 * of a cell, its centre of mass) is computed once per cell here.
 */
#include "dpm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* ------------------------------------------------------------------------ */
/* 2D geometry                                                               */
/* ------------------------------------------------------------------------ */

/* Cell2D::GetArea (src/cell.cpp:35-47): shoelace over (j=i-1, i), |A|. */
float orc_area2d(const float *xy, unsigned nv) {
  float area = 0.0f;
  unsigned j = nv - 1;
  for (unsigned i = 0; i < nv; i++) {
    float s = xy[2 * j] + xy[2 * i];
    float d = xy[2 * j + 1] - xy[2 * i + 1];
    area = (float)((double)area + 0.5 * (double)(s * d));
    j = i;
  }
  if (area < 0.0f) area = -area;
  return area;
}

/* Cell2D::Cell2D (src/cell.cpp:12-33): regular nv-gon of radius r0 centred
 * at (x0, y0), vertex i at angle 2*pi*(i+1)/nv; calA0, a0, l0. */
void orc_cell2d(float x0, float y0, float calA, unsigned nv, float r0,
                float *xy, float *a0, float *l0, float *calA0) {
  float c0 = (float)((double)calA * ((double)nv * tan(M_PI / nv) / M_PI));
  for (unsigned i = 0; i < nv; i++) {
    double ang = 2.0 * M_PI * (i + 1.0) / (double)(float)nv;
    xy[2 * i] = (float)((double)r0 * cos(ang) + (double)x0);
    xy[2 * i + 1] = (float)((double)r0 * sin(ang) + (double)y0);
  }
  float a = orc_area2d(xy, nv);
  *a0 = a;
  *l0 = (float)(2.0 * sqrt(M_PI * (double)c0 * (double)a) / (double)(float)nv);
  *calA0 = c0;
}

/* Tissue2D::Tissue2D (src/Tissue2D.cpp:23-31): L = sqrt(sum of areas)/phi0,
 * the sum in float, the root and quotient in double. */
float orc_box2d(const float *areas, int ncells, float phi0) {
  float total = 0.0f;
  for (int c = 0; c < ncells; c++) total += areas[c];
  return (float)(sqrt((double)total) / (double)phi0);
}

/* ------------------------------------------------------------------------ */
/* 2D step (shaders/Cell2D_kernel.cl)                                        */
/* ------------------------------------------------------------------------ */

/* GetCOM (Cell2D_kernel.cl:3-11): sequential float sum, then / (float)NV. */
static void com2d(const float *p, unsigned nv, float *cx, float *cy) {
  float sx = 0.0f, sy = 0.0f;
  for (unsigned i = 0; i < nv; i++) {
    sx += p[2 * i];
    sy += p[2 * i + 1];
  }
  *cx = sx / (float)nv;
  *cy = sy / (float)nv;
}

static inline void normalize2(float x, float y, float *ox, float *oy) {
  float l2 = x * x + y * y;
  if (l2 == 0.0f) {
    *ox = x;
    *oy = y;
    return;
  }
  float l = sqrtf(l2);
  *ox = x / l;
  *oy = y / l;
}

/* Crossing-number test of vertex (vx, vy) against cell cj's polygon, with the
 * reference's periodic shifts (RepulsionForceUpdate, Cell2D_kernel.cl:166-196):
 * per edge (i, j=i-1) the offsets di = v - P_i and dj = v - P_j are shifted
 * in x by L*floor(d/L) and in y by L*round(d/L), each only when that edge has
 * |d| > L on that axis.  Returns 1 when the crossing count is odd. */
static int inside2d(float vx, float vy, const float *p, unsigned nv, int pbc,
                    float L) {
  int odd = 0;
  unsigned j = nv - 1;
  for (unsigned i = 0; i < nv; j = i++) {
    float dix = vx - p[2 * i], diy = vy - p[2 * i + 1];
    float djx = vx - p[2 * j], djy = vy - p[2 * j + 1];
    if (pbc) {
      if (fabsf(dix) > L || fabsf(djx) > L) {
        dix -= L * floorf(dix / L);
        djx -= L * floorf(djx / L);
      }
      if (fabsf(diy) > L || fabsf(djy) > L) {
        diy -= L * roundf(diy / L);
        djy -= L * roundf(djy / L);
      }
    }
    if ((diy > 0) != (djy > 0) &&
        (0 < (djx - dix) * (0 - diy) / (djy - diy) + dix))
      odd = !odd;
  }
  return odd;
}

static void forces2d(const orc_tissue2d *t, const float *xy, float *F,
                     unsigned char *contained) {
  const int n = t->ncells;
  float *comx = (float *)malloc(sizeof(float) * (size_t)n);
  float *comy = (float *)malloc(sizeof(float) * (size_t)n);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < n; c++) com2d(xy + 2 * t->off[c], t->nv[c], &comx[c], &comy[c]);

#pragma omp parallel for schedule(dynamic, 1)
  for (int ci = 0; ci < n; ci++) {
    const unsigned NV = t->nv[ci];
    const float *p = xy + 2 * t->off[ci];
    float *f = F + 2 * t->off[ci];
    const float Ka = t->Ka[ci], Kl = t->Kl[ci], Kb = t->Kb[ci];
    const float a0 = t->a0[ci], l0 = t->l0[ci], r0 = t->r0[ci];

    /* AreaForceUpdates (Cell2D_kernel.cl:13-42): the area is the same for
     * every vertex of the cell. */
    float area = 0.0f;
    for (unsigned vj = 0; vj < NV; vj++) {
      unsigned jm = vj == 0 ? NV - 1 : vj - 1;
      float s = p[2 * jm] + p[2 * vj];
      float d = p[2 * jm + 1] - p[2 * vj + 1];
      area = (float)((double)area + 0.5 * (double)(s * d));
    }
    if (area < 0.0) area = -area;
    float strain = (float)((double)(area / a0) - 1.0);
    float kA = Ka / sqrtf(a0);
    float kL = Kl * sqrtf(a0 / l0);

    for (unsigned vi = 0; vi < NV; vi++) {
      unsigned im1 = vi == 0 ? NV - 1 : vi - 1;
      unsigned ip1 = vi == NV - 1 ? 0 : vi + 1;
      unsigned im2 = im1 == 0 ? NV - 1 : im1 - 1;
      unsigned ip2 = ip1 == NV - 1 ? 0 : ip1 + 1;
      const float x = p[2 * vi], y = p[2 * vi + 1];
      const float xm = p[2 * im1], ym = p[2 * im1 + 1];
      const float xp = p[2 * ip1], yp = p[2 * ip1 + 1];
      const float xmm = p[2 * im2], ymm = p[2 * im2 + 1];
      const float xpp = p[2 * ip2], ypp = p[2 * ip2 + 1];
      float fx = 0.0f, fy = 0.0f;

      /* area force, Fy with the reference's sign (Cell2D_kernel.cl:38-41) */
      fx = (float)((double)fx + (double)kA * 0.5 * (double)strain * (double)(ym - yp));
      fy = (float)((double)fy + (double)kA * 0.5 * (double)strain * (double)(xm - xp));

      /* PerimeterForceUpdates (Cell2D_kernel.cl:92-119) */
      {
        float lvx = xp - x, lvy = yp - y;
        float lmx = x - xm, lmy = y - ym;
        float len = sqrtf(lvx * lvx + lvy * lvy);
        float lenm = sqrtf(lmx * lmx + lmy * lmy);
        float ux = lvx / len, uy = lvy / len;
        float umx = lmx / lenm, umy = lmy / lenm;
        float dl = (float)((double)(len / l0) - 1.0);
        float dlm = (float)((double)(lenm / l0) - 1.0);
        fx += kL * (dl * ux - dlm * umx);
        fy += kL * (dl * uy - dlm * umy);
      }

      /* BendingForceUpdates (Cell2D_kernel.cl:44-90) */
      {
        float lvx = xp - x, lvy = yp - y;
        float lvxm = x - xm, lvym = y - ym;
        float six = lvx - lvxm, siy = lvy - lvym;
        float sixp = (xpp - xp) - lvx, siyp = (ypp - yp) - lvy;
        float sixm = lvxm - (xm - xmm), siym = lvym - (ym - ymm);
        fx = (float)((double)fx + (double)Kb * (2.0 * six - sixm - sixp));
        fy = (float)((double)fy + (double)Kb * (2.0 * siy - siym - siyp));
      }

      /* AttractionForceUpdate (Cell2D_kernel.cl:222-268): every vertex of
       * every other cell within l0 of this one. */
      if (t->Kat != 0.0f) {
        for (int cj = 0; cj < n; cj++) {
          if (cj == ci) continue;
          const float *q = xy + 2 * t->off[cj];
          for (unsigned vj = 0; vj < t->nv[cj]; vj++) {
            float rx = q[2 * vj] - x, ry = q[2 * vj + 1] - y;
            if (t->pbc) {
              rx -= t->L * roundf(rx / t->L);
              ry -= t->L * roundf(ry / t->L);
            }
            float dist = sqrtf(rx * rx + ry * ry);
            if (dist < l0) {
              float ftmp = t->Kat / (float)NV * dist / l0;
              float nx, ny;
              normalize2(rx, ry, &nx, &ny);
              fx += ftmp * nx;
              fy += ftmp * ny;
            }
          }
        }
      }

      /* RepulsionForceUpdate (Cell2D_kernel.cl:121-220): inside any other
       * cell -> push toward own centre of mass. */
      int overlaps = 0;
      for (int cj = 0; cj < n && !overlaps; cj++) {
        if (cj == ci) continue;
        overlaps = inside2d(x, y, xy + 2 * t->off[cj], t->nv[cj], t->pbc, t->L);
      }
      if (contained) contained[t->off[ci] + vi] = (unsigned char)overlaps;
      if (overlaps) {
        float dx = comx[ci] - x, dy = comy[ci] - y;
        if (t->pbc) {
          dx -= t->L * roundf(dx / t->L);
          dy -= t->L * roundf(dy / t->L);
        }
        float dist = sqrtf(dx * dx + dy * dy);
        float xij = dist / (2 * r0);
        float ftmp = t->Kre * (1 - xij);
        float nx, ny;
        normalize2(dx, dy, &nx, &ny);
        fx += 0.5f * ftmp * nx;
        fy += 0.5f * ftmp * ny;
      }
      f[2 * vi] = fx;
      f[2 * vi + 1] = fy;
    }
  }
  free(comx);
  free(comy);
}

/* Tissue2D::CLEulerUpdate (src/Tissue2D.cpp:215-229): forces, then Euler
 * x += F*dt (EulerUpdate, Cell2D_kernel.cl:270-281); F of the last step is
 * what the caller receives. */
int orc_run2d(const orc_tissue2d *t, float dt, int nsteps, float *xy, float *F,
              unsigned char *contained, int nthreads) {
  if (!t || t->ncells <= 0 || nsteps < 0) return 1;
  set_threads(nthreads);
  size_t total = 0;
  for (int c = 0; c < t->ncells; c++) total += t->nv[c];
  memset(F, 0, sizeof(float) * 2 * total);
  for (int s = 0; s < nsteps; s++) {
    forces2d(t, xy, F, contained);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)(2 * total); k++) xy[k] += F[k] * dt;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* 3D geometry (src/cell.cpp:62-230)                                         */
/* ------------------------------------------------------------------------ */

int orc_icosphere_counts(int level, int *nv, int *nf) {
  if (level < 0 || level > 7) return 1;
  int v = 12, f = 20;
  for (int i = 0; i < level; i++) {
    v = v + (3 * f) / 2;
    f = 4 * f;
  }
  *nv = v;
  *nf = f;
  return 0;
}

/* Midpoint of edge (p1, p2), cached per unordered pair so that each edge is
 * split once (Cell3D::AddMiddlePoint, src/cell.cpp:160-194).  The new point is
 * pushed outward to the unit sphere the way the reference does it: one
 * component at a time, each divided by the norm of the partly updated point. */
typedef struct {
  unsigned *keys_lo, *keys_hi, *vals;
  unsigned cap;
} edge_map;

static unsigned midpoint(edge_map *m, float *xyz, unsigned *count, unsigned p1,
                         unsigned p2) {
  unsigned lo = p1 < p2 ? p1 : p2, hi = p1 < p2 ? p2 : p1;
  unsigned h = (lo * 2654435761u) ^ (hi * 40503u);
  for (unsigned k = h % m->cap;; k = (k + 1) % m->cap) {
    if (m->vals[k] == 0xffffffffu) {
      float mp[3];
      for (int i = 0; i < 3; i++) {
        mp[i] = xyz[3 * p2 + i] + xyz[3 * p1 + i];
        mp[i] = (float)((double)mp[i] * 0.5);
      }
      for (int i = 0; i < 3; i++) {
        float norm = sqrtf(mp[0] * mp[0] + mp[1] * mp[1] + mp[2] * mp[2]);
        mp[i] /= norm;
      }
      unsigned id = (*count)++;
      memcpy(xyz + 3 * id, mp, sizeof(mp));
      m->keys_lo[k] = lo;
      m->keys_hi[k] = hi;
      m->vals[k] = id;
      return id;
    }
    if (m->keys_lo[k] == lo && m->keys_hi[k] == hi) return m->vals[k];
  }
}

/* Unit icosphere with the reference's vertex and face numbering: the 12
 * icosahedron vertices and 20 faces of src/cell.cpp:68-119, then `level`
 * rounds of 4-way subdivision (src/cell.cpp:121-142; the reference fixes
 * level 2).  xyz: [nv*3], faces: [nf*3]. */
int orc_icosphere(int level, float *xyz, unsigned *faces) {
  int nv, nf;
  if (orc_icosphere_counts(level, &nv, &nf)) return 1;
  const float t = (float)((1 + sqrt(5.0)) / 2);
  const float base[12][3] = {{-1, t, 0}, {1, t, 0},  {-1, -t, 0}, {1, -t, 0},
                             {0, -1, t}, {0, 1, t},  {0, -1, -t}, {0, 1, -t},
                             {t, 0, -1}, {t, 0, 1},  {-t, 0, -1}, {-t, 0, 1}};
  static const unsigned base_faces[20][3] = {
      {0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
      {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
      {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
      {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
  for (int i = 0; i < 12; i++) {
    float x = base[i][0], y = base[i][1], z = base[i][2];
    float norm = sqrtf(x * x + y * y + z * z);
    xyz[3 * i] = x / norm;
    xyz[3 * i + 1] = y / norm;
    xyz[3 * i + 2] = z / norm;
  }
  unsigned *cur = (unsigned *)malloc(sizeof(unsigned) * 3 * (size_t)nf);
  unsigned *nxt = (unsigned *)malloc(sizeof(unsigned) * 3 * (size_t)nf);
  memcpy(cur, base_faces, sizeof(base_faces));
  unsigned count = 12, ncur = 20;
  edge_map m;
  m.cap = 4u * (unsigned)nv + 17u;
  m.keys_lo = (unsigned *)malloc(sizeof(unsigned) * m.cap);
  m.keys_hi = (unsigned *)malloc(sizeof(unsigned) * m.cap);
  m.vals = (unsigned *)malloc(sizeof(unsigned) * m.cap);
  memset(m.vals, 0xff, sizeof(unsigned) * m.cap);
  for (int lv = 0; lv < level; lv++) {
    for (unsigned j = 0; j < ncur; j++) {
      unsigned f0 = cur[3 * j], f1 = cur[3 * j + 1], f2 = cur[3 * j + 2];
      unsigned a = midpoint(&m, xyz, &count, f0, f1);
      unsigned b = midpoint(&m, xyz, &count, f1, f2);
      unsigned c = midpoint(&m, xyz, &count, f2, f0);
      unsigned *o = nxt + 12 * j;
      o[0] = f0; o[1] = a; o[2] = c;
      o[3] = f1; o[4] = b; o[5] = a;
      o[6] = f2; o[7] = c; o[8] = b;
      o[9] = a;  o[10] = b; o[11] = c;
    }
    unsigned *tmp = cur;
    cur = nxt;
    nxt = tmp;
    ncur *= 4;
  }
  memcpy(faces, cur, sizeof(unsigned) * 3 * (size_t)nf);
  free(cur);
  free(nxt);
  free(m.keys_lo);
  free(m.keys_hi);
  free(m.vals);
  return (int)count == nv ? 0 : 2;
}

/* Cell3D::GetVolume (src/cell.cpp:196-211): |sum (v1 x v2) . v0| / 6. */
float orc_volume3d(const float *xyz, const unsigned *faces, int nf) {
  float volume = 0.0f;
  for (int f = 0; f < nf; f++) {
    const float *v0 = xyz + 3 * faces[3 * f], *v1 = xyz + 3 * faces[3 * f + 1],
                *v2 = xyz + 3 * faces[3 * f + 2];
    float c0 = v1[1] * v2[2] - v1[2] * v2[1];
    float c1 = v1[2] * v2[0] - v1[0] * v2[2];
    float c2 = v1[0] * v2[1] - v1[1] * v2[0];
    volume += c0 * v0[0] + c1 * v0[1] + c2 * v0[2];
  }
  return (float)((double)fabsf(volume) / 6.0);
}

/* Cell3D::GetSurfaceArea (src/cell.cpp:213-230): sum of |A x B| over faces,
 * which is twice the area (the reference has no factor 1/2). */
float orc_surface3d(const float *xyz, const unsigned *faces, int nf) {
  float sa = 0.0f;
  for (int f = 0; f < nf; f++) {
    const float *v0 = xyz + 3 * faces[3 * f], *v1 = xyz + 3 * faces[3 * f + 1],
                *v2 = xyz + 3 * faces[3 * f + 2];
    float A[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    float B[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
    float c0 = A[1] * B[2] - A[2] * B[1];
    float c1 = A[2] * B[0] - A[0] * B[2];
    float c2 = A[0] * B[1] - A[1] * B[0];
    sa += sqrtf(c0 * c0 + c1 * c1 + c2 * c2);
  }
  return sa;
}

/* Cell3D::Cell3D (src/cell.cpp:62-158) with the subdivision level as a
 * parameter: mesh scaled by r0 and moved to start; v0 = 4/3 pi r0^3,
 * sa0 = (6 sqrt(pi) v0 calA)^(2/3), a0 = sa0 / nf. */
void orc_cell3d(const float *start, float calA, float r0, int level,
                float *xyz, unsigned *faces, float *v0, float *sa0, float *a0) {
  int nv, nf;
  orc_icosphere_counts(level, &nv, &nf);
  orc_icosphere(level, xyz, faces);
  for (int v = 0; v < nv; v++)
    for (int k = 0; k < 3; k++) {
      xyz[3 * v + k] *= r0;
      xyz[3 * v + k] += start[k];
    }
  float vv = (float)((double)(4.0f / 3.0f) * M_PI * pow((double)r0, 3));
  float ss = (float)pow(6 * sqrt(M_PI) * (double)vv * (double)calA,
                        (double)(2.0f / 3.0f));
  *v0 = vv;
  *sa0 = ss;
  *a0 = ss / (float)nf;
}

/* Tissue3D::Tissue3D (src/Tissue3D.cpp:24-28): L = cbrt(sum v0) / phi0. */
float orc_box3d(const float *v0, int ncells, float phi0) {
  float total = 0.0f;
  for (int c = 0; c < ncells; c++) total += v0[c];
  return (float)(cbrt((double)total) / (double)phi0);
}

/* Rest edge length of the 3D surface springs (src/Tissue3D.cpp:177):
 * sqrt(4 a0) / sqrt(3) (not the equilateral edge sqrt(4 a0 / sqrt 3)). */
float orc_l0_3d(float a0) {
  return (float)(sqrt((double)(4.0f * a0)) / sqrt(3.0));
}

/* ------------------------------------------------------------------------ */
/* 3D step (shaders/Cell3D_Kernel.cl)                                        */
/* ------------------------------------------------------------------------ */

typedef struct {
  float x, y, z;
} v3;

static inline v3 mk3(float x, float y, float z) {
  v3 r = {x, y, z};
  return r;
}
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 scl3(float s, v3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
static inline v3 div3(v3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross3(v3 a, v3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 norm3(v3 a) {
  float l2 = dot3(a, a);
  if (l2 == 0.0f) return a;
  return div3(a, sqrtf(l2));
}
static inline v3 ld3(const float *p, size_t i) {
  return mk3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
static inline void acc3(float *F, size_t i, v3 f) {
  F[3 * i] += f.x;
  F[3 * i + 1] += f.y;
  F[3 * i + 2] += f.z;
}

/* GetCOM (Cell3D_Kernel.cl:35-44): sequential sum times 1/NV. */
static v3 com3d(const float *xyz, int nv) {
  v3 s = mk3(0.0f, 0.0f, 0.0f);
  for (int i = 0; i < nv; i++) s = add3(s, ld3(xyz, (size_t)i));
  float inv = 1.0f / (float)nv;
  return scl3(inv, s);
}

/* Winding number of `point` with respect to cell cj's mesh shifted by
 * `shift` (RepellingForces, Cell3D_Kernel.cl:283-302). */
static float winding3d(const float *q, const unsigned *faces, int nf, v3 shift,
                       v3 point) {
  float total = 0.0f;
  for (int f = 0; f < nf; f++) {
    v3 a = sub3(add3(ld3(q, faces[3 * f]), shift), point);
    v3 b = sub3(add3(ld3(q, faces[3 * f + 1]), shift), point);
    v3 c = sub3(add3(ld3(q, faces[3 * f + 2]), shift), point);
    v3 u = norm3(a), v = norm3(b), w = norm3(c);
    float denom = 1.0f + dot3(u, v) + dot3(v, w) + dot3(w, u);
    if (denom < 1e-8f) continue;
    float num = dot3(u, cross3(v, w));
    total += 2.0f * atan2f(num, denom);
  }
  return total / (4.0f * (float)M_PI);
}

/* Triangle-bending force (extension; the reference has no 3D bending):
 * E = kb * sum over interior edges of (1 - n1.n2) with n the unit normals of
 * the two faces sharing the edge.  For face (p0,p1,p2) with n = (p1-p0)x(p2-p0)
 * and G = sum over its three edges of (n_other - (n.n_other) n)/|n|, the
 * force is kb*((p1-p2)xG, (p2-p0)xG, Gx(p1-p0)) on (p0, p1, p2). */
static void bend3d(const float *p, const unsigned *faces, int nf,
                   const int *adj, float kb, float *F) {
  v3 *nh = (v3 *)malloc(sizeof(v3) * (size_t)nf);
  float *nl = (float *)malloc(sizeof(float) * (size_t)nf);
  for (int f = 0; f < nf; f++) {
    v3 p0 = ld3(p, faces[3 * f]), p1 = ld3(p, faces[3 * f + 1]),
       p2 = ld3(p, faces[3 * f + 2]);
    v3 n = cross3(sub3(p1, p0), sub3(p2, p0));
    float l = sqrtf(dot3(n, n));
    nl[f] = l;
    nh[f] = l > 0.0f ? div3(n, l) : mk3(0.0f, 0.0f, 0.0f);
  }
  for (int f = 0; f < nf; f++) {
    if (nl[f] == 0.0f) continue;
    v3 G = mk3(0.0f, 0.0f, 0.0f);
    for (int e = 0; e < 3; e++) {
      int g = adj[3 * f + e];
      if (g < 0) continue;
      float c = dot3(nh[f], nh[g]);
      G = add3(G, div3(sub3(nh[g], scl3(c, nh[f])), nl[f]));
    }
    v3 p0 = ld3(p, faces[3 * f]), p1 = ld3(p, faces[3 * f + 1]),
       p2 = ld3(p, faces[3 * f + 2]);
    acc3(F, faces[3 * f], scl3(kb, cross3(sub3(p1, p2), G)));
    acc3(F, faces[3 * f + 1], scl3(kb, cross3(sub3(p2, p0), G)));
    acc3(F, faces[3 * f + 2], scl3(kb, cross3(G, sub3(p1, p0))));
  }
  free(nh);
  free(nl);
}

/* adj[3*f+e]: the face sharing edge e (vertices e, e+1) of face f, or -1. */
static int *face_adjacency(const unsigned *faces, int nf) {
  int *adj = (int *)malloc(sizeof(int) * 3 * (size_t)nf);
  for (int i = 0; i < 3 * nf; i++) adj[i] = -1;
  for (int f = 0; f < nf; f++)
    for (int e = 0; e < 3; e++) {
      if (adj[3 * f + e] >= 0) continue;
      unsigned a = faces[3 * f + e], b = faces[3 * f + (e + 1) % 3];
      for (int g = f + 1; g < nf && adj[3 * f + e] < 0; g++)
        for (int k = 0; k < 3; k++) {
          unsigned c = faces[3 * g + k], d = faces[3 * g + (k + 1) % 3];
          if ((c == a && d == b) || (c == b && d == a)) {
            adj[3 * f + e] = g;
            adj[3 * g + k] = f;
            break;
          }
        }
    }
  return adj;
}

static void forces3d(const orc_tissue3d *t, const float *xyz, float *F,
                     unsigned char *wnflags, const int *adj) {
  const int n = t->ncells, NV = t->nv, NF = t->nf;
  const unsigned *fc = t->faces;
  v3 *com = (v3 *)malloc(sizeof(v3) * (size_t)n);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < n; c++) com[c] = com3d(xyz + 3 * (size_t)c * NV, NV);

#pragma omp parallel for schedule(dynamic, 1)
  for (int ci = 0; ci < n; ci++) {
    const float *p = xyz + 3 * (size_t)ci * NV;
    float *f = F + 3 * (size_t)ci * NV;
    /* ClearForces (Cell3D_Kernel.cl:366-369) */
    memset(f, 0, sizeof(float) * 3 * (size_t)NV);

    /* VolumeForceUpdate (Cell3D_Kernel.cl:66-112), with the volume
     * computed before any face reads it. */
    if (t->Kv[ci] != 0.0f) {
      float volume = 0.0f;
      for (int fi = 0; fi < NF; fi++) {
        v3 P0 = ld3(p, fc[3 * fi]), P1 = ld3(p, fc[3 * fi + 1]),
           P2 = ld3(p, fc[3 * fi + 2]);
        volume += dot3(cross3(P0, P1), P2) / 6.0f;
      }
      volume = fabsf(volume);
      float strain = volume / t->v0[ci] - 1.0f;
      float k = -t->Kv[ci] * strain;
      for (int fi = 0; fi < NF; fi++) {
        v3 P0 = ld3(p, fc[3 * fi]), P1 = ld3(p, fc[3 * fi + 1]),
           P2 = ld3(p, fc[3 * fi + 2]);
        v3 A = sub3(P1, com[ci]), B = sub3(P2, com[ci]), C = sub3(P0, com[ci]);
        acc3(f, fc[3 * fi], div3(scl3(k, cross3(A, B)), 6.0f));
        acc3(f, fc[3 * fi + 1], div3(scl3(k, cross3(B, C)), 6.0f));
        acc3(f, fc[3 * fi + 2], div3(scl3(k, cross3(C, A)), 6.0f));
      }
    }

    /* SurfaceAreaForceUpdate (Cell3D_Kernel.cl:114-177) */
    if (!(t->Ka[ci] < 1e-8f)) {
      float tl = t->l0[ci];
      float scale = t->Ka[ci] * sqrtf(t->a0[ci]) / tl * 0.3f;
      for (int fi = 0; fi < NF; fi++) {
        v3 P0 = ld3(p, fc[3 * fi]), P1 = ld3(p, fc[3 * fi + 1]),
           P2 = ld3(p, fc[3 * fi + 2]);
        v3 lv0 = sub3(P1, P0), lv1 = sub3(P2, P1), lv2 = sub3(P0, P2);
        float l0 = sqrtf(dot3(lv0, lv0)), l1 = sqrtf(dot3(lv1, lv1)),
              l2 = sqrtf(dot3(lv2, lv2));
        if (l0 < 1e-12f || l1 < 1e-12f || l2 < 1e-12f) continue;
        v3 n0 = div3(lv0, l0), n1 = div3(lv1, l1), n2 = div3(lv2, l2);
        float d0 = l0 / tl - 1.0f, d1 = l1 / tl - 1.0f, d2 = l2 / tl - 1.0f;
        v3 f0 = sub3(scl3(d0, n0), scl3(d2, n2));
        v3 f1 = sub3(scl3(d1, n1), scl3(d0, n0));
        v3 f2 = sub3(scl3(d2, n2), scl3(d1, n1));
        acc3(f, fc[3 * fi], scl3(scale, f0));
        acc3(f, fc[3 * fi + 1], scl3(scale, f1));
        acc3(f, fc[3 * fi + 2], scl3(scale, f2));
      }
    }

    /* StickToSurface (Cell3D_Kernel.cl:180-247); the adhesion range is
     * 2*l0 unless the extension sets it. */
    if (!(t->Ks[ci] < 1e-12f)) {
      float ks = t->Ks[ci], tl = t->l0[ci];
      float range = t->adh ? t->adh[ci] : tl * 2.0f;
      for (int fi = 0; fi < NF; fi++) {
        v3 P0 = ld3(p, fc[3 * fi]), P1 = ld3(p, fc[3 * fi + 1]),
           P2 = ld3(p, fc[3 * fi + 2]);
        v3 un = norm3(cross3(sub3(P1, P0), sub3(P2, P0)));
        if (!(un.z < -0.1f)) continue;
        v3 pos[3] = {P0, P1, P2};
        for (int k = 0; k < 3; k++) {
          unsigned idx = fc[3 * fi + k];
          if (pos[k].z < 0.0f) f[3 * idx + 2] += ks * fabsf(pos[k].z);
          v3 sp = mk3(pos[k].x, pos[k].y, 0.0f);
          float h = fabsf(pos[k].z);
          if (h < range) {
            v3 c2v = sub3(sp, com[ci]);
            float dd = sqrtf(dot3(sub3(pos[k], sp), sub3(pos[k], sp)));
            float ftmp = (float)((double)ks * (1.0 - (double)(dd / tl)));
            acc3(f, idx, scl3(ftmp, norm3(c2v)));
          }
        }
      }
    }

    /* Triangle bending (extension). */
    if (t->Kb && t->Kb[ci] != 0.0f) bend3d(p, fc, NF, adj, t->Kb[ci], f);
  }

  /* RepellingForces (Cell3D_Kernel.cl:251-310): for every vertex and every
   * other cell, the winding number of the vertex in that cell's mesh
   * (shifted by the periodic image of the centres); if |wn| >= 1e-6 push
   * toward the own centre by |wn| * 0.5 * Kc. */
  if (t->Kre != 0.0f) {
#pragma omp parallel for schedule(dynamic, 16)
    for (long gv = 0; gv < (long)n * NV; gv++) {
      int ci = (int)(gv / NV);
      v3 point = ld3(xyz, (size_t)gv);
      v3 comi = com[ci];
      int hits = 0;
      for (int cj = 0; cj < n; cj++) {
        if (cj == ci) continue;
        v3 comj = com[cj];
        v3 shift = mk3(0.0f, 0.0f, 0.0f);
        if (t->pbc) {
          v3 r = div3(sub3(comi, comj), t->L);
          shift = scl3(t->L, mk3(roundf(r.x), roundf(r.y), roundf(r.z)));
        }
        float wn = winding3d(xyz + 3 * (size_t)cj * NV, fc, NF, shift, point);
        if (fabsf(wn) < 1e-6f) continue;
        hits++;
        v3 dir = norm3(sub3(comi, point));
        acc3(F, (size_t)gv, scl3(fabsf(wn) * 0.5f * t->Kre, dir));
      }
      if (wnflags) wnflags[gv] = (unsigned char)(hits > 255 ? 255 : hits);
    }
  } else if (wnflags) {
    memset(wnflags, 0, (size_t)n * NV);
  }
  free(com);
  /* AllVertAttraction, after the repulsion, when switched on */
  if (t->Kat != 0.0f) orc_attraction3d(n, NV, xyz, t->l0, t->L, t->pbc, t->Kat, F);
}

/* AllVertAttraction (Cell3D_Kernel.cl:313-364).  The reference visits every
 * ordered pair (vertex p1 of cell ci, vertex p2 of cell cj != ci): delta =
 * p2 - p1, wrapped per axis by L*round(delta/L); dist = |delta|; with L0 =
 * l0[ci] (at least 1e-12), if 1e-12 < dist < 2 L0 then tmp = Kat * 0.5 *
 * (dist/L0 - 1) * (delta/dist) is subtracted from p1 and added to p2.  The
 * visit from cj sees exactly -delta and the same dist, so vertex p1 gathers
 * -tmp(L0 = l0[ci]) and +tmp'(L0 = l0[cj]) with tmp' built on -delta. */
void orc_attraction3d(int ncells, int nv, const float *xyz, const float *l0, float L,
                      int pbc, float Kat, float *F) {
  if (Kat == 0.0f) return;
#pragma omp parallel for schedule(dynamic, 16)
  for (long gv = 0; gv < (long)ncells * nv; gv++) {
    const int ci = (int)(gv / nv);
    const float p1x = xyz[3 * gv], p1y = xyz[3 * gv + 1], p1z = xyz[3 * gv + 2];
    float L0i = l0[ci];
    if (L0i < 1e-12f) L0i = 1e-12f;
    float fx = F[3 * gv], fy = F[3 * gv + 1], fz = F[3 * gv + 2];
    for (int cj = 0; cj < ncells; cj++) {
      if (cj == ci) continue;
      float L0j = l0[cj];
      if (L0j < 1e-12f) L0j = 1e-12f;
      for (int vj = 0; vj < nv; vj++) {
        const size_t k = (size_t)cj * nv + vj;
        float dx = xyz[3 * k] - p1x, dy = xyz[3 * k + 1] - p1y, dz = xyz[3 * k + 2] - p1z;
        if (pbc) {
          const float rx = roundf(dx / L), ry = roundf(dy / L), rz = roundf(dz / L);
          dx = dx - L * rx;
          dy = dy - L * ry;
          dz = dz - L * rz;
        }
        const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
        if (dist < L0i * 2.0f && dist > 1e-12f) {
          const float a = Kat * 0.5f * (dist / L0i - 1.0f);
          fx = fx + -(a * (dx / dist));
          fy = fy + -(a * (dy / dist));
          fz = fz + -(a * (dz / dist));
        }
        if (dist < L0j * 2.0f && dist > 1e-12f) {
          const float b = Kat * 0.5f * (dist / L0j - 1.0f);
          fx = fx + b * (-dx / dist);
          fy = fy + b * (-dy / dist);
          fz = fz + b * (-dz / dist);
        }
      }
    }
    F[3 * gv] = fx;
    F[3 * gv + 1] = fy;
    F[3 * gv + 2] = fz;
  }
}

/* Tissue3D::CLEulerUpdate (src/Tissue3D.cpp:372-445): per step clear,
 * accumulate all forces, then EulerPosition x += F*dt (Cell3D_Kernel.cl:
 * 371-381); F is read back after the last Euler update. */
int orc_run3d(const orc_tissue3d *t, float dt, int nsteps, float *xyz, float *F,
              unsigned char *wn, int nthreads) {
  if (!t || t->ncells <= 0 || nsteps < 0) return 1;
  set_threads(nthreads);
  int *adj = face_adjacency(t->faces, t->nf);
  size_t total = (size_t)t->ncells * t->nv;
  memset(F, 0, sizeof(float) * 3 * total);
  for (int s = 0; s < nsteps; s++) {
    forces3d(t, xyz, F, wn, adj);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)(3 * total); k++) xyz[k] += F[k] * dt;
  }
  free(adj);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Dispersion (host relaxation of centres with drand48)                       */
/* ------------------------------------------------------------------------ */

/* Soft-disk relaxation of cell centres (src/Tissue2D.cpp:42-105 and
 * src/Tissue3D.cpp:40-106): centres drawn with drand48()*L after
 * srand48(seed), overlap force (1 - d/(ri+rj))/(ri+rj), step 0.01, until the
 * energy change is <= 1e-6 or after 1e5 iterations.  `scale` multiplies the
 * radii (1 in 2D, 2 in 3D). */
static void relax_centres(int n, const float *r0, float scale, float L,
                          long seed, float *X, float *Y) {
  float *Fx = (float *)calloc((size_t)n, sizeof(float));
  float *Fy = (float *)calloc((size_t)n, sizeof(float));
  srand48(seed);
  for (int i = 0; i < n; i++) {
    X[i] = (float)(drand48() * L);
    Y[i] = (float)(drand48() * L);
  }
  float oldU = 100, dU = 100;
  int count = 0;
  while (dU > 1e-6) {
    float U = 0;
    for (int i = 0; i < n; i++) {
      Fx[i] = 0.0f;
      Fy[i] = 0.0f;
    }
    for (int i = 0; i < n; i++) {
      float xi = X[i], yi = Y[i], ri = r0[i] * scale;
      for (int j = 0; j < n; j++) {
        if (j == i) continue;
        float rj = r0[j] * scale;
        float dx = X[j] - xi;
        dx = (float)((double)dx - (double)L * round((double)(dx / L)));
        float dy = Y[j] - yi;
        dy = (float)((double)dy - (double)L * round((double)(dy / L)));
        float dist = (float)sqrt((double)(dx * dx + dy * dy));
        if (dist < 0.0) dist *= -1;
        if (dist <= (ri + rj)) {
          float ux = dx / dist, uy = dy / dist;
          float ftmp = (float)((1.0 - (double)(dist / (ri + rj))) / (double)(ri + rj));
          float fx = ftmp * ux, fy = ftmp * uy;
          Fx[i] -= fx;
          Fy[i] -= fy;
          Fy[j] += fy;
          Fx[j] += fx;
          float q = dist / (ri + rj);
          float inner = 1 - q * (1 - q);
          U = (float)((double)U + 0.5 * (double)inner);
        }
      }
    }
    for (int i = 0; i < n; i++) {
      X[i] = (float)((double)X[i] + 0.01 * (double)Fx[i]);
      Y[i] = (float)((double)Y[i] + 0.01 * (double)Fy[i]);
    }
    dU = U - oldU;
    if (dU < 0.0) dU *= -1;
    oldU = U;
    count++;
    if (count > 1e5) break;
  }
  free(Fx);
  free(Fy);
}

/* Tissue2D::Disperse: relax centres, then rebuild every cell as a regular
 * polygon of radius r0 around its centre (src/Tissue2D.cpp:106-113). */
void orc_disperse2d(int ncells, const unsigned *nv, const unsigned *off,
                    const float *r0, float L, long seed, float *xy) {
  float *X = (float *)malloc(sizeof(float) * (size_t)ncells);
  float *Y = (float *)malloc(sizeof(float) * (size_t)ncells);
  relax_centres(ncells, r0, 1.0f, L, seed, X, Y);
  for (int i = 0; i < ncells; i++)
    for (unsigned j = 0; j < nv[i]; j++) {
      double ang = 2.0 * M_PI * (j + 1) / nv[i];
      xy[2 * (off[i] + j)] = (float)((double)r0[i] * cos(ang) + (double)X[i]);
      xy[2 * (off[i] + j) + 1] = (float)((double)r0[i] * sin(ang) + (double)Y[i]);
    }
  free(X);
  free(Y);
}

/* Tissue3D::Disperse2D: relax centres with doubled radii, then move each
 * cell by -(COM) - (X, Y) in x and y (src/Tissue3D.cpp:107-114; the
 * reference subtracts the target centre). */
void orc_disperse3d(int ncells, int nv, const float *r0, float L, long seed,
                    float *xyz) {
  float *X = (float *)malloc(sizeof(float) * (size_t)ncells);
  float *Y = (float *)malloc(sizeof(float) * (size_t)ncells);
  relax_centres(ncells, r0, 2.0f, L, seed, X, Y);
  for (int i = 0; i < ncells; i++) {
    float *p = xyz + 3 * (size_t)i * nv;
    float cx = 0.0f, cy = 0.0f;
    for (int v = 0; v < nv; v++) {
      cx += p[3 * v];
      cy += p[3 * v + 1];
    }
    cx /= (float)nv;
    cy /= (float)nv;
    for (int v = 0; v < nv; v++) {
      p[3 * v] -= cx;
      p[3 * v + 1] -= cy;
      p[3 * v] -= X[i];
      p[3 * v + 1] -= Y[i];
    }
  }
  free(X);
  free(Y);
}

/* ------------------------------------------------------------------------ */
/* FP64 diagnostics                                                          */
/* ------------------------------------------------------------------------ */

/* Per cell: area, perimeter and the energy
 * U = Ka/2 (A/a0-1)^2 + Kl/2 sum (l/l0-1)^2 + Kb/2 sum |s_i|^2,
 * all in double (project-defined; the reference defines no energy). */
void orc_diag2d(const orc_tissue2d *t, const float *xy, double *area,
                double *perim, double *energy) {
  for (int c = 0; c < t->ncells; c++) {
    const unsigned NV = t->nv[c];
    const float *p = xy + 2 * t->off[c];
    double A = 0.0, P = 0.0, Ul = 0.0, Ub = 0.0;
    for (unsigned i = 0; i < NV; i++) {
      unsigned j = (i + 1) % NV, k = (i + NV - 1) % NV;
      double xi = p[2 * i], yi = p[2 * i + 1], xj = p[2 * j], yj = p[2 * j + 1];
      A += xi * yj - xj * yi;
      double l = sqrt((xj - xi) * (xj - xi) + (yj - yi) * (yj - yi));
      P += l;
      double dl = l / t->l0[c] - 1.0;
      Ul += dl * dl;
      double sx = (xj - xi) - (xi - p[2 * k]), sy = (yj - yi) - (yi - p[2 * k + 1]);
      Ub += sx * sx + sy * sy;
    }
    A = fabs(0.5 * A);
    double da = A / t->a0[c] - 1.0;
    if (area) area[c] = A;
    if (perim) perim[c] = P;
    if (energy)
      energy[c] = 0.5 * t->Ka[c] * da * da + 0.5 * t->Kl[c] * Ul + 0.5 * t->Kb[c] * Ub;
  }
}

/* Per cell: enclosed volume, true surface area, and the energy
 * U = Kv/2 (V/v0-1)^2 + Ka/2 sum_edges (l/l0-1)^2 (+ bending), in double. */
void orc_diag3d(const orc_tissue3d *t, const float *xyz, double *volume,
                double *area, double *energy) {
  const int NV = t->nv, NF = t->nf;
  double *dp = (double *)malloc(sizeof(double) * 3 * (size_t)NV);
  for (int c = 0; c < t->ncells; c++) {
    const float *p = xyz + 3 * (size_t)c * NV;
    for (int i = 0; i < 3 * NV; i++) dp[i] = p[i];
    double V = 0.0, A = 0.0, Ue = 0.0;
    for (int f = 0; f < NF; f++) {
      const double *a = dp + 3 * t->faces[3 * f], *b = dp + 3 * t->faces[3 * f + 1],
                   *d = dp + 3 * t->faces[3 * f + 2];
      V += a[0] * (b[1] * d[2] - b[2] * d[1]) + a[1] * (b[2] * d[0] - b[0] * d[2]) +
           a[2] * (b[0] * d[1] - b[1] * d[0]);
      double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
      double w[3] = {d[0] - a[0], d[1] - a[1], d[2] - a[2]};
      double cx = u[1] * w[2] - u[2] * w[1], cy = u[2] * w[0] - u[0] * w[2],
             cz = u[0] * w[1] - u[1] * w[0];
      A += 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
      const double *e[3] = {a, b, d};
      for (int k = 0; k < 3; k++) {
        const double *s = e[k], *q = e[(k + 1) % 3];
        double l = sqrt((q[0] - s[0]) * (q[0] - s[0]) + (q[1] - s[1]) * (q[1] - s[1]) +
                        (q[2] - s[2]) * (q[2] - s[2]));
        double dl = l / t->l0[c] - 1.0;
        Ue += 0.5 * dl * dl; /* each edge is seen from both faces */
      }
    }
    V = fabs(V) / 6.0;
    double dv = V / t->v0[c] - 1.0;
    double U = 0.5 * t->Kv[c] * dv * dv + 0.5 * t->Ka[c] * Ue;
    if (t->Kb && t->Kb[c] != 0.0f) U += orc_bend_energy3d(NV, NF, t->faces, t->Kb[c], dp);
    if (volume) volume[c] = V;
    if (area) area[c] = A;
    if (energy) energy[c] = U;
  }
  free(dp);
}

/* E = kb * sum over edges shared by two faces of (1 - n1.n2), in double. */
double orc_bend_energy3d(int nv, int nf, const unsigned *faces, double kb,
                         const double *xyz) {
  (void)nv;
  int *adj = face_adjacency(faces, nf);
  double E = 0.0;
  double *nh = (double *)malloc(sizeof(double) * 3 * (size_t)nf);
  for (int f = 0; f < nf; f++) {
    const double *a = xyz + 3 * faces[3 * f], *b = xyz + 3 * faces[3 * f + 1],
                 *c = xyz + 3 * faces[3 * f + 2];
    double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    double w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2],
                   u[0] * w[1] - u[1] * w[0]};
    double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; k++) nh[3 * f + k] = l > 0 ? n[k] / l : 0.0;
  }
  for (int f = 0; f < nf; f++)
    for (int e = 0; e < 3; e++) {
      int g = adj[3 * f + e];
      if (g <= f) continue; /* each edge once */
      double c = nh[3 * f] * nh[3 * g] + nh[3 * f + 1] * nh[3 * g + 1] +
                 nh[3 * f + 2] * nh[3 * g + 2];
      E += kb * (1.0 - c);
    }
  free(nh);
  free(adj);
  return E;
}
