// 3D DPM kernels: launch interface.
#pragma once

#include "dpm_common.cuh"

namespace dpm {

// Mesh topology shared by every cell of a 3D batch.
struct Mesh3D {
  int nv, nf;
  const uint16_t *faces;    // [nf*3] vertex ids
  const int *inc_off;       // [nv+1] CSR offsets: faces around each vertex
  const uint16_t *inc_face; // [3*nf] face ids, ascending per vertex
  const uint8_t *inc_corner;// [3*nf] corner (0..2) of the vertex in that face
  const int16_t *adj;       // [nf*3] face across edge e (vertices e, e+1), -1 none
  // Patches: groups of at most 32 vertices that are close on the surface
  // (vertex ids pvert[poff[p] .. poff[p+1]), np <= kMaxPatches3D).
  int np;
  const int *poff;          // [np+1]
  const uint16_t *pvert;    // [nv]
  // Edges: endpoints (lower id first) and, per face corner k, the edge from
  // corner k to corner k+1 (bit 15 set when it runs from the higher id).
  int ne;
  const uint16_t *eva;      // [2*ne]
  const uint16_t *fedge;    // [3*nf]
};

constexpr int kMaxPatches3D = 32;
constexpr int kPatchSize3D = 32;

struct Step3DArgs {
  Mesh3D mesh;
  const Cell3D *cells;
  const Tissue3D *tissues;
  const float *xin, *yin, *zin;  // positions (SoA, cell-major)
  float *xout, *yout, *zout;
  float *fx, *fy, *fz;           // forces of this step, or nullptr
  unsigned char *wn_out;         // winding hits of this step, or nullptr
  const Geom3D *geom_in;
  Geom3D *geom_out;
  const Geom3D *geom0;
  const int *nn, *nbr;
  int *stale, *err;
  int ncells;
  float dt;
  int bend; // any cell with Kb != 0
  int step_index; // index of this step within its rebuild period
  int all_forces; // 1: outputs for every cell; 0: only at each tissue's last step
};

struct Rebuild3DArgs {
  const Cell3D *cells;
  Tissue3D *tissues;
  const Geom3D *geom;
  Geom3D *geom0;
  uint32_t *keys, *vals;
  const uint32_t *sorted_keys, *sorted_vals;
  int *nn, *nbr, *stale;
  int ncells, ntissues;
  int block_len; // steps in the rebuild period that follows (0: leave budgets)
};

cudaError_t launch_geom3d(const float *x, const float *y, const float *z, const Mesh3D &mesh,
                          const Cell3D *cells, Geom3D *geom, int ncells, cudaStream_t s);
// Per cell, in double: (volume, surface area, energy) into out[3*c .. 3*c+2].
cudaError_t launch_diag3d(const float *x, const float *y, const float *z, const Mesh3D &mesh,
                          const Cell3D *cells, double *out, int ncells, cudaStream_t s);
cudaError_t launch_binprep3d(const Rebuild3DArgs &a, int local_bits, cudaStream_t s);
cudaError_t launch_neighbors3d(const Rebuild3DArgs &a, int local_bits, cudaStream_t s);
// Dynamic shared memory of one k3d_step block of `threads` threads.
size_t step3d_smem_bytes(int nv, int nf, int ne, bool bend, int threads);
// Threads per cell the runtime picks: 256 when a launch has more cells than
// two 512-thread blocks per SM hold and four 256-thread blocks' shared memory
// fits on an SM, else 512.
int step3d_threads(int nv, int nf, int ne, bool bend, int ncells, int sm_count);
cudaError_t prepare_step3d(int nv, int nf, int ne, bool bend);
// One fused 3D step, one block of `threads` (128, 256 or 512) per cell; every
// block size gives the same bits.
cudaError_t launch_step3d(const Step3DArgs &a, int threads, cudaStream_t s);

} // namespace dpm
