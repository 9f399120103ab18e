// Host model classes of the clDPM API, above the C ABI.
//
// These mirror the reference's public C++ types (include/cell.hpp,
// include/Tissue.hpp): the same class names, fields, constructors and
// methods, with the same value semantics.  Stepping goes through the C ABI
// (include/dpm_gb300.h) to the sm_103a kernels; there is no OpenCL and no
// CPU fallback.  Additions beyond the reference are marked "extension".
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

struct dpm_ctx;
struct dpm2d_batch;
struct dpm3d_batch;

namespace DPM {

// Process-wide drand48-compatible generator (X' = a X + c mod 2^48), used by
// Disperse/Disperse2D like the reference's unseeded drand48() calls.
void seed48(long seed);
double rand48();
// The starting centres of a dispersion after seed48(seed): X[i], Y[i] drawn
// in turn as (float)(drand48() * L).
void draw_centres(long seed, int n, float L, std::vector<float> &X, std::vector<float> &Y);
// seed48(seed), then the dispersion loop (host or device); returns the
// iteration count.
int relax_centres(const std::vector<float> &radius, float L, long seed, bool device,
                  std::vector<float> &X, std::vector<float> &Y);

// Process-wide library context on the device named by $DPM_DEVICE (default 0).
dpm_ctx *default_context();

// 2D deformable polygon (include/cell.hpp:12-27, src/cell.cpp:12-60).
struct Cell2D {
  unsigned int NV;
  float calA0;
  float a0;
  float l0;
  float r0;
  float Ka = 0.0f;
  float Kb = 0.0f;
  float Kl = 0.0f;
  float Ks = 0.0f;
  std::vector<std::array<float, 2>> Verticies;
  std::vector<std::array<float, 2>> Forces;
  // Regular NV-gon of radius r0 around (x0, y0); the fifth argument is the
  // radius (the reference header calls it a0).
  Cell2D(float x0, float y0, float calA, unsigned int NV, float r0);
  float GetArea() const;
  // Perimeter of the closed polygon (the reference's version reads one
  // vertex past the end, src/cell.cpp:56; this one closes the ring).
  float GetPerim() const;
};

// 3D deformable icosphere mesh (include/cell.hpp:28-58, src/cell.cpp:62-288).
// The subdivision level is a constructor argument (extension; the reference
// fixes it at 2: 162 vertices, 320 faces).
class Cell3D {
public:
  unsigned int NV;
  unsigned int NF;
  int level;
  float calA0;
  float r0;
  float v0;
  float sa0;
  float a0;
  float Kv = 0.0f;
  float Ka = 0.0f;
  float Ks = 0.0f;
  float Kb = 0.0f;   // extension: triangle bending
  float adh = -1.0f; // extension: adhesion range (< 0: the reference's 2*l0)
  float Volume;
  float SurfaceArea;
  std::vector<std::array<float, 3>> Verts;
  std::vector<std::array<float, 3>> Forces;
  std::vector<std::array<unsigned int, 3>> Faces;

  Cell3D(std::array<float, 3> starting_point, float CalA0, float r0, int level = 2);
  float GetVolume() const;
  float GetSurfaceArea() const;
  std::vector<std::vector<float>> GetPositions() const;
  std::vector<std::vector<float>> GetVesselPositions(float L) const;
  std::vector<std::vector<float>> GetForces() const;
  std::vector<std::array<int, 3>> GetFaces() const;
  std::array<float, 3> GetCOM() const;
};

class Tissue2D {
public:
  std::vector<Cell2D> cells;
  int NCELLS;
  bool PBC;
  float Kre;
  float Kat;
  float phi0;
  float L;
  Tissue2D(std::vector<Cell2D> cells, float phi0);
  ~Tissue2D();
  Tissue2D(const Tissue2D &o);
  Tissue2D &operator=(const Tissue2D &o);
  // device: relax on the GPU (dpm_disperse, same bits); false: on the host
  void Disperse(bool device = true);
  void CLEulerUpdate(int nsteps, float dt);
  // extensions
  void SetPackingFraction(float phi);
  float GetPackingFraction() const;
  std::vector<float> GetShapeIndices() const;

private:
  dpm2d_batch *batch_ = nullptr;
  std::vector<unsigned> batch_nv_;
  void release();
};

class Tissue3D {
public:
  int NCELLS;
  int PBC;
  float L;
  float Kre = 0.0f;
  float Kat = 0.0f;
  // extension: also run the reference's AllVertAttraction kernel with Kat
  // (its own step loop never enqueues it, so Kat alone has no effect)
  bool AllVertAttraction = false;
  std::string attractionMethod;
  std::vector<Cell3D> Cells;
  Tissue3D(std::vector<Cell3D> cells, float phi0);
  ~Tissue3D();
  Tissue3D(const Tissue3D &o);
  Tissue3D &operator=(const Tissue3D &o);
  void CLEulerUpdate(int nsteps, float dt);
  void Disperse2D(bool device = true);

private:
  dpm3d_batch *batch_ = nullptr;
  int batch_ncells_ = 0, batch_nv_ = 0;
  void release();
};

} // namespace DPM
