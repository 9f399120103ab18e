// Tissue classes of the clDPM API: construction, dispersion and the
// CLEulerUpdate step loops, which go through the C ABI to the GPU.
#include "dpm_host.hpp"

#include <cmath>
#include <cstdlib>
#include <iostream>
#include <mutex>
#include <stdexcept>

#include "dpm_gb300.h"

namespace DPM {

// ---------------------------------------------------------------------------
// drand48-compatible generator and the library context
// ---------------------------------------------------------------------------

namespace {
// glibc's state before any srand48 call (as if srand48(0x1234ABCD))
uint64_t g_x48 = 0x1234ABCD330Eull;
std::mutex g_rng_mu;
std::mutex g_ctx_mu;
dpm_ctx *g_ctx = nullptr;

void check(int rc, const char *what) {
  if (rc == DPM_OK) return;
  std::string msg = std::string(what) + ": " + dpm_last_error();
  if (rc == DPM_EINVAL) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}
} // namespace

void seed48(long seed) {
  std::lock_guard<std::mutex> g(g_rng_mu);
  g_x48 = (((uint64_t)(uint32_t)seed) << 16) | 0x330Eull;
}

double rand48() {
  std::lock_guard<std::mutex> g(g_rng_mu);
  g_x48 = (0x5DEECE66Dull * g_x48 + 0xBull) & ((1ull << 48) - 1);
  return std::ldexp((double)g_x48, -48);
}

dpm_ctx *default_context() {
  std::lock_guard<std::mutex> g(g_ctx_mu);
  if (!g_ctx) {
    const char *d = std::getenv("DPM_DEVICE");
    check(dpm_ctx_create(d ? std::atoi(d) : 0, &g_ctx), "dpm_ctx_create");
  }
  return g_ctx;
}

namespace {

// Soft-disk relaxation of centres (src/Tissue2D.cpp:42-105,
// src/Tissue3D.cpp:40-106): drand48 centres in [0, L), overlap force
// (1 - d/(ri+rj))/(ri+rj), step 0.01, until |dU| <= 1e-6 or 1e5 iterations.
int relax(const std::vector<float> &radius, float L, std::vector<float> &X,
          std::vector<float> &Y, bool warn, bool device) {
  const int n = (int)radius.size();
  X.resize(n);
  Y.resize(n);
  std::vector<float> Fx(n), Fy(n);
  for (int i = 0; i < n; i++) {
    X[i] = (float)(rand48() * L);
    Y[i] = (float)(rand48() * L);
  }
  if (device) {
    // the same loop on the GPU, bit for bit
    int count = 0;
    check(dpm_disperse(default_context(), 1, &n, radius.data(), &L, X.data(), Y.data(), &count),
          "dpm_disperse");
    if (warn && count > 100000)
      std::cerr << "Warning: Max timesteps for dispersion reached" << std::endl;
    return count;
  }
  float oldU = 100, dU = 100;
  int count = 0;
  while (dU > 1e-6) {
    float U = 0;
    for (int i = 0; i < n; i++) Fx[i] = Fy[i] = 0.0f;
    for (int i = 0; i < n; i++) {
      const float xi = X[i], yi = Y[i], ri = radius[i];
      for (int j = 0; j < n; j++) {
        if (j == i) continue;
        const float rj = radius[j];
        float dx = X[j] - xi;
        dx = (float)((double)dx - (double)L * std::round((double)(dx / L)));
        float dy = Y[j] - yi;
        dy = (float)((double)dy - (double)L * std::round((double)(dy / L)));
        float dist = (float)std::sqrt((double)(dx * dx + dy * dy));
        if (dist < 0.0) dist *= -1;
        if (dist <= (ri + rj)) {
          const float ux = dx / dist, uy = dy / dist;
          const float ftmp = (float)((1.0 - (double)(dist / (ri + rj))) / (double)(ri + rj));
          const float fx = ftmp * ux, fy = ftmp * uy;
          Fx[i] -= fx;
          Fy[i] -= fy;
          Fy[j] += fy;
          Fx[j] += fx;
          const float q = dist / (ri + rj);
          const float inner = 1 - q * (1 - q);
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
    if (count > 1e5) {
      if (warn) std::cerr << "Warning: Max timesteps for dispersion reached" << std::endl;
      break;
    }
  }
  return count;
}

} // namespace

void draw_centres(long seed, int n, float L, std::vector<float> &X, std::vector<float> &Y) {
  seed48(seed);
  X.resize(n);
  Y.resize(n);
  for (int i = 0; i < n; i++) {
    X[i] = (float)(rand48() * L);
    Y[i] = (float)(rand48() * L);
  }
}

int relax_centres(const std::vector<float> &radius, float L, long seed, bool device,
                  std::vector<float> &X, std::vector<float> &Y) {
  seed48(seed);
  return relax(radius, L, X, Y, false, device);
}

// ---------------------------------------------------------------------------
// Tissue2D
// ---------------------------------------------------------------------------

// src/Tissue2D.cpp:15-40
Tissue2D::Tissue2D(std::vector<Cell2D> inputCells, float packingFraction) {
  if (inputCells.empty()) throw std::invalid_argument("a tissue needs at least one cell");
  cells = std::move(inputCells);
  NCELLS = (int)cells.size();
  PBC = true;
  Kre = 1.0f;
  Kat = 0.0f;
  phi0 = packingFraction;
  float total = 0.0f;
  for (const auto &c : cells) total += c.GetArea();
  L = (float)(std::sqrt((double)total) / (double)phi0);
}

Tissue2D::~Tissue2D() { release(); }
Tissue2D::Tissue2D(const Tissue2D &o)
    : cells(o.cells), NCELLS(o.NCELLS), PBC(o.PBC), Kre(o.Kre), Kat(o.Kat), phi0(o.phi0),
      L(o.L) {}
Tissue2D &Tissue2D::operator=(const Tissue2D &o) {
  if (this != &o) {
    release();
    cells = o.cells;
    NCELLS = o.NCELLS;
    PBC = o.PBC;
    Kre = o.Kre;
    Kat = o.Kat;
    phi0 = o.phi0;
    L = o.L;
  }
  return *this;
}

void Tissue2D::release() {
  if (batch_) dpm2d_destroy(batch_);
  batch_ = nullptr;
  batch_nv_.clear();
}

// src/Tissue2D.cpp:42-114: relax centres, then regular polygons around them.
void Tissue2D::Disperse(bool device) {
  std::vector<float> r(NCELLS), X, Y;
  for (int i = 0; i < NCELLS; i++) r[i] = cells[i].r0;
  relax(r, L, X, Y, false, device);
  for (int i = 0; i < NCELLS; i++)
    for (unsigned j = 0; j < cells[i].NV; j++) {
      const double ang = 2.0 * M_PI * (j + 1) / cells[i].NV;
      cells[i].Verticies[j][0] = (float)((double)cells[i].r0 * std::cos(ang) + (double)X[i]);
      cells[i].Verticies[j][1] = (float)((double)cells[i].r0 * std::sin(ang) + (double)Y[i]);
    }
}

// src/Tissue2D.cpp:116-241: pack, step on the GPU, unpack positions and the
// forces of the last step.
void Tissue2D::CLEulerUpdate(int nsteps, float dt) {
  if ((int)cells.size() != NCELLS) throw std::invalid_argument("Cells changed size");
  std::vector<unsigned> nv(NCELLS);
  size_t total = 0;
  for (int c = 0; c < NCELLS; c++) {
    nv[c] = cells[c].NV;
    if (cells[c].Verticies.size() != cells[c].NV)
      throw std::invalid_argument("Verts must hold NV vertices");
    total += nv[c];
  }
  dpm_ctx *ctx = default_context();
  if (!batch_ || batch_nv_ != nv) {
    release();
    int n = NCELLS;
    check(dpm2d_create(ctx, 1, &n, nv.data(), &batch_), "dpm2d_create");
    batch_nv_ = nv;
  }
  std::vector<float> Ka(NCELLS), Kl(NCELLS), Kb(NCELLS), a0(NCELLS), l0(NCELLS), r0(NCELLS);
  std::vector<float> xy(2 * total), F(2 * total);
  size_t off = 0;
  for (int c = 0; c < NCELLS; c++) {
    const Cell2D &C = cells[c];
    Ka[c] = C.Ka;
    Kl[c] = C.Kl;
    Kb[c] = C.Kb;
    a0[c] = C.a0;
    l0[c] = C.l0;
    r0[c] = C.r0;
    for (unsigned v = 0; v < C.NV; v++) {
      xy[2 * (off + v)] = C.Verticies[v][0];
      xy[2 * (off + v) + 1] = C.Verticies[v][1];
    }
    off += C.NV;
  }
  const int pbc = PBC ? 1 : 0;
  check(dpm2d_set_cells(batch_, Ka.data(), Kl.data(), Kb.data(), a0.data(), l0.data(),
                        r0.data()),
        "dpm2d_set_cells");
  check(dpm2d_set_tissues(batch_, &L, &Kre, &Kat, &pbc), "dpm2d_set_tissues");
  check(dpm2d_upload(batch_, xy.data()), "dpm2d_upload");
  check(dpm2d_step(batch_, nsteps, dt), "dpm2d_step");
  const int rc = dpm2d_download(batch_, xy.data(), F.data());
  if (rc != DPM_OK && rc != DPM_ENONFINITE) check(rc, "dpm2d_download");
  off = 0;
  for (int c = 0; c < NCELLS; c++) {
    Cell2D &C = cells[c];
    for (unsigned v = 0; v < C.NV; v++) {
      C.Verticies[v] = {xy[2 * (off + v)], xy[2 * (off + v) + 1]};
      C.Forces[v] = {F[2 * (off + v)], F[2 * (off + v) + 1]};
    }
    off += C.NV;
  }
}

// Extension: rescale the box to true packing fraction phi (sum of areas /
// L^2), moving every cell rigidly with its centroid (shapes unchanged).
void Tissue2D::SetPackingFraction(float phi) {
  if (!(phi > 0.0f)) throw std::invalid_argument("phi must be positive");
  double area = 0.0;
  for (const auto &c : cells) area += c.GetArea();
  const double Lnew = std::sqrt(area / phi);
  const double s = Lnew / L;
  for (auto &c : cells) {
    double cx = 0.0, cy = 0.0;
    for (const auto &v : c.Verticies) {
      cx += v[0];
      cy += v[1];
    }
    cx /= c.NV;
    cy /= c.NV;
    const double dx = cx * (s - 1.0), dy = cy * (s - 1.0);
    for (auto &v : c.Verticies) {
      v[0] = (float)(v[0] + dx);
      v[1] = (float)(v[1] + dy);
    }
  }
  L = (float)Lnew;
}

float Tissue2D::GetPackingFraction() const {
  double area = 0.0;
  for (const auto &c : cells) area += c.GetArea();
  return (float)(area / ((double)L * L));
}

std::vector<float> Tissue2D::GetShapeIndices() const {
  std::vector<float> s;
  s.reserve(cells.size());
  for (const auto &c : cells)
    s.push_back((float)(c.GetPerim() / std::sqrt(4.0 * M_PI * c.GetArea())));
  return s;
}

// ---------------------------------------------------------------------------
// Tissue3D
// ---------------------------------------------------------------------------

// src/Tissue3D.cpp:16-38
Tissue3D::Tissue3D(std::vector<Cell3D> cells, float phi0) {
  if (cells.empty()) throw std::invalid_argument("a tissue needs at least one cell");
  Cells = std::move(cells);
  NCELLS = (int)Cells.size();
  float volume = 0.0f;
  for (const auto &c : Cells) volume += c.v0;
  L = (float)(std::cbrt((double)volume) / (double)phi0);
  PBC = 1;
  attractionMethod = "General";
}

Tissue3D::~Tissue3D() { release(); }
Tissue3D::Tissue3D(const Tissue3D &o)
    : NCELLS(o.NCELLS), PBC(o.PBC), L(o.L), Kre(o.Kre), Kat(o.Kat),
      AllVertAttraction(o.AllVertAttraction), attractionMethod(o.attractionMethod),
      Cells(o.Cells) {}
Tissue3D &Tissue3D::operator=(const Tissue3D &o) {
  if (this != &o) {
    release();
    NCELLS = o.NCELLS;
    PBC = o.PBC;
    L = o.L;
    Kre = o.Kre;
    Kat = o.Kat;
    AllVertAttraction = o.AllVertAttraction;
    attractionMethod = o.attractionMethod;
    Cells = o.Cells;
  }
  return *this;
}

void Tissue3D::release() {
  if (batch_) dpm3d_destroy(batch_);
  batch_ = nullptr;
  batch_ncells_ = batch_nv_ = 0;
}

// src/Tissue3D.cpp:40-116 (cells move to -(X, Y), as in the reference)
void Tissue3D::Disperse2D(bool device) {
  std::vector<float> r(NCELLS), X, Y;
  for (int i = 0; i < NCELLS; i++) r[i] = Cells[i].r0 * 2;
  relax(r, L, X, Y, true, device);
  for (int i = 0; i < NCELLS; i++) {
    const std::array<float, 3> com = Cells[i].GetCOM();
    for (auto &v : Cells[i].Verts) {
      v[0] -= com[0];
      v[1] -= com[1];
      v[0] -= X[i];
      v[1] -= Y[i];
    }
  }
}

// src/Tissue3D.cpp:118-522: validate, pack, step on the GPU, unpack, then the
// host-side volume and surface area with the reference's warnings.
void Tissue3D::CLEulerUpdate(int nsteps, float dt) {
  if (nsteps <= 0) {
    std::cerr << "[ERROR] Invalid nsteps: " << nsteps << std::endl;
    throw std::invalid_argument("nsteps must be positive");
  }
  if (dt <= 0.0f || dt > 0.1f) {
    std::cerr << "[ERROR] Invalid dt: " << dt << " (should be in range (0, 0.1])" << std::endl;
    throw std::invalid_argument("dt must be positive and reasonable");
  }
  if (NCELLS <= 0 || (int)Cells.size() != NCELLS) {
    std::cerr << "[ERROR] Invalid NCELLS: " << NCELLS << std::endl;
    throw std::invalid_argument("NCELLS must be positive");
  }
  const Cell3D &c0 = Cells[0];
  const int NV = (int)c0.NV, NF = (int)c0.NF;
  std::vector<unsigned> faces(3 * (size_t)NF);
  for (int f = 0; f < NF; f++) {
    for (int k = 0; k < 3; k++) {
      if (c0.Faces[f][k] >= (unsigned)NV) {
        std::cerr << "[ERROR] Invalid face index at face " << f << std::endl;
        throw std::runtime_error("Invalid face indices");
      }
      faces[3 * f + k] = c0.Faces[f][k];
    }
  }
  std::vector<float> Kv(NCELLS), Ka(NCELLS), Ks(NCELLS), v0(NCELLS), a0(NCELLS), l0(NCELLS),
      Kb(NCELLS), adh(NCELLS);
  std::vector<float> xyz(3 * (size_t)NCELLS * NV), F(3 * (size_t)NCELLS * NV);
  bool any_kb = false, any_adh = false;
  for (int ci = 0; ci < NCELLS; ci++) {
    const Cell3D &C = Cells[ci];
    if ((int)C.NV != NV || C.Verts.size() != (size_t)NV)
      throw std::invalid_argument("all cells must share one mesh");
    if (C.Kv <= 0 || C.Ka <= 0 || C.Ks <= 0) {
      std::cerr << "[ERROR] Invalid spring constants for cell " << ci << ": Kv=" << C.Kv
                << ", Ka=" << C.Ka << ", Ks=" << C.Ks << std::endl;
      throw std::runtime_error("Invalid spring constants");
    }
    if (C.v0 <= 0 || C.a0 <= 0) {
      std::cerr << "[ERROR] Invalid reference values for cell " << ci << ": v0=" << C.v0
                << ", a0=" << C.a0 << std::endl;
      throw std::runtime_error("Invalid reference values");
    }
    Kv[ci] = C.Kv;
    Ka[ci] = C.Ka;
    Ks[ci] = C.Ks;
    v0[ci] = C.v0;
    a0[ci] = C.a0;
    l0[ci] = (float)(std::sqrt((double)(4.0f * C.a0)) / std::sqrt(3.0));
    Kb[ci] = C.Kb;
    adh[ci] = C.adh >= 0.0f ? C.adh : 2.0f * l0[ci];
    any_kb |= C.Kb != 0.0f;
    any_adh |= C.adh >= 0.0f;
    for (int v = 0; v < NV; v++)
      for (int k = 0; k < 3; k++) {
        const float x = C.Verts[v][k];
        if (!std::isfinite(x)) {
          std::cerr << "[ERROR] Non-finite vertex coordinate at cell " << ci << ", vertex " << v
                    << ", coord " << k << ": " << x << std::endl;
          throw std::runtime_error("Non-finite vertex coordinates");
        }
        xyz[3 * ((size_t)ci * NV + v) + k] = x;
      }
  }
  dpm_ctx *ctx = default_context();
  if (!batch_ || batch_ncells_ != NCELLS || batch_nv_ != NV) {
    release();
    int n = NCELLS;
    check(dpm3d_create(ctx, 1, &n, NV, NF, faces.data(), &batch_), "dpm3d_create");
    batch_ncells_ = NCELLS;
    batch_nv_ = NV;
  }
  check(dpm3d_set_cells(batch_, Kv.data(), Ka.data(), Ks.data(), v0.data(), a0.data(),
                        l0.data(), any_kb ? Kb.data() : nullptr, any_adh ? adh.data() : nullptr),
        "dpm3d_set_cells");
  check(dpm3d_set_tissues(batch_, &L, &Kre, &PBC), "dpm3d_set_tissues");
  const float kat = AllVertAttraction ? Kat : 0.0f;
  check(dpm3d_set_attraction(batch_, &kat), "dpm3d_set_attraction");
  check(dpm3d_upload(batch_, xyz.data()), "dpm3d_upload");
  check(dpm3d_step(batch_, nsteps, dt), "dpm3d_step");
  const int rc = dpm3d_download(batch_, xyz.data(), F.data());
  if (rc != DPM_OK && rc != DPM_ENONFINITE) check(rc, "dpm3d_download");
  for (int ci = 0; ci < NCELLS; ci++) {
    Cell3D &C = Cells[ci];
    for (int v = 0; v < NV; v++) {
      const size_t i = 3 * ((size_t)ci * NV + v);
      for (int k = 0; k < 3; k++) {
        if (!std::isfinite(xyz[i + k])) {
          std::cerr << "[ERROR] Non-finite result vertex at cell " << ci << ", vertex " << v
                    << ", coord " << k << ": " << xyz[i + k] << std::endl;
          throw std::runtime_error("Non-finite simulation results");
        }
        if (!std::isfinite(F[i + k]))
          std::cerr << "[WARNING] Non-finite force at cell " << ci << ", vertex " << v
                    << ", coord " << k << ": " << F[i + k] << std::endl;
      }
      C.Verts[v] = {xyz[i], xyz[i + 1], xyz[i + 2]};
      C.Forces[v] = {F[i], F[i + 1], F[i + 2]};
    }
    C.Volume = C.GetVolume();
    C.SurfaceArea = C.GetSurfaceArea();
    if (!std::isfinite(C.Volume) || C.Volume <= 0)
      std::cerr << "[WARNING] Invalid volume for cell " << ci << ": " << C.Volume << std::endl;
    if (!std::isfinite(C.SurfaceArea) || C.SurfaceArea <= 0)
      std::cerr << "[WARNING] Invalid surface area for cell " << ci << ": " << C.SurfaceArea
                << std::endl;
  }
}

} // namespace DPM
