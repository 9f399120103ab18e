// Cell geometry of the clDPM API.  The arithmetic keeps the reference's
// precision choices (double where its expressions promote, float where they
// do not), so a cell built here has exactly the reference's vertices and
// rest values (src/cell.cpp).
#include "dpm_host.hpp"

#include <cmath>
#include <stdexcept>
#include <unordered_map>

namespace DPM {

namespace {

float shoelace(const std::vector<std::array<float, 2>> &v) {
  float area = 0.0f;
  size_t j = v.size() - 1;
  for (size_t i = 0; i < v.size(); i++) {
    float s = v[j][0] + v[i][0];
    float d = v[j][1] - v[i][1];
    area = (float)((double)area + 0.5 * (double)(s * d));
    j = i;
  }
  return area < 0.0f ? -area : area;
}

} // namespace

// src/cell.cpp:12-33
Cell2D::Cell2D(float x0, float y0, float calA, unsigned int numVerts, float radius) {
  if (numVerts < 3) throw std::invalid_argument("a Cell2D needs at least 3 vertices");
  NV = numVerts;
  r0 = radius;
  calA0 = (float)((double)calA * ((double)NV * std::tan(M_PI / NV) / M_PI));
  Verticies.resize(NV);
  Forces.assign(NV, {0.0f, 0.0f});
  for (unsigned int i = 0; i < NV; i++) {
    const double ang = 2.0 * M_PI * (i + 1.0) / (double)(float)NV;
    Verticies[i][0] = (float)((double)r0 * std::cos(ang) + (double)x0);
    Verticies[i][1] = (float)((double)r0 * std::sin(ang) + (double)y0);
  }
  a0 = GetArea();
  l0 = (float)(2.0 * std::sqrt(M_PI * (double)calA0 * (double)a0) / (double)(float)NV);
}

// src/cell.cpp:35-47
float Cell2D::GetArea() const { return shoelace(Verticies); }

float Cell2D::GetPerim() const {
  float p = 0.0f;
  for (size_t i = 0; i < Verticies.size(); i++) {
    const auto &a = Verticies[i];
    const auto &b = Verticies[(i + 1) % Verticies.size()];
    const float dx = b[0] - a[0], dy = b[1] - a[1];
    p += std::sqrt(dx * dx + dy * dy);
  }
  return p;
}

namespace {

// Icosphere with the reference's numbering: 12 icosahedron vertices and 20
// faces (src/cell.cpp:68-119), then 4-way subdivision (src/cell.cpp:121-142)
// with each edge midpoint created once, pushed to the unit sphere one
// component at a time as the reference does (src/cell.cpp:160-194).
void icosphere(int level, std::vector<std::array<float, 3>> &V,
               std::vector<std::array<unsigned, 3>> &F) {
  const float t = (float)((1 + std::sqrt(5.0)) / 2);
  V = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
       {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
  for (auto &p : V) {
    const float norm = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    p[0] /= norm;
    p[1] /= norm;
    p[2] /= norm;
  }
  F = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
       {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
       {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
       {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
  std::unordered_map<uint64_t, unsigned> cache;
  auto mid = [&](unsigned p1, unsigned p2) -> unsigned {
    const uint64_t key = ((uint64_t)std::min(p1, p2) << 32) | std::max(p1, p2);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    std::array<float, 3> m;
    for (int i = 0; i < 3; i++) {
      m[i] = V[p2][i] + V[p1][i];
      m[i] = (float)((double)m[i] * 0.5);
    }
    for (int i = 0; i < 3; i++) {
      const float norm = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
      m[i] /= norm;
    }
    V.push_back(m);
    const unsigned id = (unsigned)V.size() - 1;
    cache.emplace(key, id);
    return id;
  };
  for (int lv = 0; lv < level; lv++) {
    std::vector<std::array<unsigned, 3>> nf;
    nf.reserve(F.size() * 4);
    for (const auto &f : F) {
      const unsigned a = mid(f[0], f[1]), b = mid(f[1], f[2]), c = mid(f[2], f[0]);
      nf.push_back({f[0], a, c});
      nf.push_back({f[1], b, a});
      nf.push_back({f[2], c, b});
      nf.push_back({a, b, c});
    }
    F.swap(nf);
  }
}

} // namespace

// src/cell.cpp:62-158
Cell3D::Cell3D(std::array<float, 3> start, float calA, float radius, int lvl) {
  if (lvl < 0 || lvl > 4) throw std::invalid_argument("subdivision level must be 0..4");
  level = lvl;
  calA0 = calA;
  r0 = radius;
  icosphere(level, Verts, Faces);
  NV = (unsigned)Verts.size();
  NF = (unsigned)Faces.size();
  Forces.assign(NV, {0.0f, 0.0f, 0.0f});
  for (auto &p : Verts)
    for (int k = 0; k < 3; k++) {
      p[k] *= r0;
      p[k] += start[k];
    }
  v0 = (float)((double)(4.0f / 3.0f) * M_PI * std::pow((double)r0, 3));
  sa0 = (float)std::pow(6 * std::sqrt(M_PI) * (double)v0 * (double)calA,
                        (double)(2.0f / 3.0f));
  a0 = sa0 / (float)NF;
  Volume = GetVolume();
  SurfaceArea = GetSurfaceArea();
}

// src/cell.cpp:196-211
float Cell3D::GetVolume() const {
  float volume = 0.0f;
  for (const auto &f : Faces) {
    const auto &v0 = Verts[f[0]], &v1 = Verts[f[1]], &v2 = Verts[f[2]];
    const float c0 = v1[1] * v2[2] - v1[2] * v2[1];
    const float c1 = v1[2] * v2[0] - v1[0] * v2[2];
    const float c2 = v1[0] * v2[1] - v1[1] * v2[0];
    volume += c0 * v0[0] + c1 * v0[1] + c2 * v0[2];
  }
  return (float)((double)std::fabs(volume) / 6.0);
}

// src/cell.cpp:213-230 (sum of |A x B|: twice the area, as in the reference)
float Cell3D::GetSurfaceArea() const {
  float sa = 0.0f;
  for (const auto &f : Faces) {
    const auto &v0 = Verts[f[0]], &v1 = Verts[f[1]], &v2 = Verts[f[2]];
    const float A[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    const float B[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
    const float c0 = A[1] * B[2] - A[2] * B[1];
    const float c1 = A[2] * B[0] - A[0] * B[2];
    const float c2 = A[0] * B[1] - A[1] * B[0];
    sa += std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  }
  return sa;
}

std::vector<std::vector<float>> Cell3D::GetPositions() const {
  std::vector<std::vector<float>> p(3, std::vector<float>(NV));
  for (unsigned i = 0; i < NV; i++)
    for (int k = 0; k < 3; k++) p[k][i] = Verts[i][k];
  return p;
}

// src/cell.cpp:242-253: x wrapped onto a cylinder of circumference L.
std::vector<std::vector<float>> Cell3D::GetVesselPositions(float L) const {
  std::vector<std::vector<float>> p(3, std::vector<float>(NV));
  const float scale = (float)((2.0 * M_PI) / L);
  const float radius = (float)(L / (2 * M_PI));
  for (unsigned i = 0; i < NV; i++) {
    const float theta = Verts[i][0] * scale;
    p[0][i] = (float)((radius - Verts[i][2]) * std::cos(theta));
    p[2][i] = (float)((radius - Verts[i][2]) * std::sin(theta));
    p[1][i] = Verts[i][1];
  }
  return p;
}

std::vector<std::vector<float>> Cell3D::GetForces() const {
  std::vector<std::vector<float>> p(3, std::vector<float>(NV));
  for (unsigned i = 0; i < NV; i++)
    for (int k = 0; k < 3; k++) p[k][i] = Forces[i][k];
  return p;
}

std::vector<std::array<int, 3>> Cell3D::GetFaces() const {
  std::vector<std::array<int, 3>> f(NF);
  for (unsigned i = 0; i < NF; i++)
    for (int k = 0; k < 3; k++) f[i][k] = (int)Faces[i][k];
  return f;
}

// src/cell.cpp:276-288
std::array<float, 3> Cell3D::GetCOM() const {
  std::array<float, 3> c = {0.0f, 0.0f, 0.0f};
  for (const auto &p : Verts)
    for (int k = 0; k < 3; k++) c[k] += p[k];
  for (int k = 0; k < 3; k++) c[k] /= (float)NV;
  return c;
}

} // namespace DPM
