// 2D DPM kernels: launch interface.
#pragma once

#include "dpm_common.cuh"

namespace dpm {

struct Step2DArgs {
  const Cell2D *cells;
  const Tissue2D *tissues;
  const float2 *pos_in;
  float2 *pos_out;
  float2 *force_out;        // forces of this step, or nullptr
  unsigned char *flags_out; // containment flags of this step, or nullptr
  const Geom2D *geom_in;    // geometry of pos_in
  Geom2D *geom_out;         // geometry of pos_out (written)
  const Geom2D *geom0;      // geometry at the last neighbour-list rebuild (nullptr:
                            // no lists, no staleness check)
  const int *nn;            // neighbour counts (kNbOverflow = scan tissue; nullptr:
                            // every cell scans its tissue)
  const int *nbr;           // neighbour lists, kMaxNB2D per cell
  int *stale;               // per tissue: list no longer covers all pairs
  int *err;                 // bit 0: non-finite positions
  int ncells;
  float dt;
  int step_index;  // index of this step within its rebuild period
  int all_forces;  // 1: force_out/flags_out take every cell's values; 0: only
                   // those of tissues whose step budget ends at this step
  int *sched;      // two zeroed counters for the dynamic schedule, or nullptr
  const int *order; // the launch's cells: order[0..ncells), or nullptr for
                    // cells 0..ncells-1 (a batch of mixed ring sizes launches
                    // one kernel per vertex-slot class over its own cells)
};

struct Rebuild2DArgs {
  const Cell2D *cells;
  Tissue2D *tissues;
  const Geom2D *geom;
  Geom2D *geom0;
  uint32_t *keys;
  uint32_t *vals;
  const uint32_t *sorted_keys;
  const uint32_t *sorted_vals;
  int *nn;
  int *nbr;
  int *stale;
  int ncells;
  int ntissues;
  int block_len;  // steps in the rebuild period that follows (0: leave budgets)
};

// Geometry of every cell (circle, area, box) from positions.
cudaError_t launch_geom2d(const Cell2D *cells, const float2 *pos, Geom2D *geom,
                          int ncells, int maxnv, cudaStream_t s);
// Per-cell diagnostics in double: (|area|, perimeter, sum (l/l0-1)^2,
// sum |s_i|^2) of the ring at pos.
struct Diag2D {
  double area, perim, ul, ub;
};
cudaError_t launch_diag2d(const Cell2D *cells, const float2 *pos, Diag2D *out, int ncells,
                          cudaStream_t s);
// Rescales each tissue t with phi[t] > 0 to true packing fraction phi[t]:
// new L, centroids moved affinely, shapes kept (one block per tissue).
cudaError_t launch_rescale2d(const Cell2D *cells, Tissue2D *tissues, const float *phi,
                             float2 *pos, int *stale, int ntissues, cudaStream_t s);
// Per-tissue bin sizes and per-cell bin keys (one block per tissue).
cudaError_t launch_binprep2d(const Rebuild2DArgs &a, int local_bits, cudaStream_t s);
// Neighbour lists from the sorted cell list (one warp per cell).
cudaError_t launch_neighbors2d(const Rebuild2DArgs &a, int local_bits, cudaStream_t s);
// One fused time step.  warps: 4, 8 or 16 per block; variant bit 0 caps
// registers for 32 resident warps per SM (else the compiler chooses), bit 1
// selects the dynamic schedule (needs a.sched), bit 2 compiles the
// attraction in (needed when any tissue has Kat != 0; without it the kernel
// is smaller and faster).
cudaError_t launch_step2d(const Step2DArgs &a, int maxnv, int warps, int variant,
                          cudaStream_t s);
// Resident run of small tissues (k2d_run_resident): one block per tissue
// keeps the tissue in shared memory for `nsteps` steps.  `a` carries the
// cells, tissues, outputs (forces and flags of the last step), geom0, nn, err,
// dt and all_forces of an ordinary step; pos and geom are the batch's current
// positions and their geometry, read at the start and written at the end.
struct Resident2DArgs {
  Step2DArgs a;
  float2 *pos;
  Geom2D *geom;
  int nsteps;
  int ncmax;  // largest tissue: cells and vertices (sizes the shared memory)
  int nvmax;
};
constexpr int kResidentWarps = 16;
// Tissues that take the resident run: at most this many cells and vertices.
constexpr int kResidentMaxCells = 64;
constexpr int kResidentMaxVerts = 2048;
// Dynamic shared memory of one block of the resident run.
size_t resident2d_smem_bytes(int ncmax, int nvmax);
// Launches the resident run over tissues [0, ntissues) (variant bit 2: the
// attraction compiled in); maxnv <= 64.
cudaError_t launch_resident2d(const Resident2DArgs &r, int ntissues, int maxnv, int variant,
                              cudaStream_t s);
cudaError_t launch_resident2d_s1(const Resident2DArgs &r, int ntissues, int variant,
                                 cudaStream_t s);
cudaError_t launch_resident2d_s2(const Resident2DArgs &r, int ntissues, int variant,
                                 cudaStream_t s);
// One step with a team of 4 warps per cell (no attraction; maxnv <= 64;
// variant bit 0: register cap).
cudaError_t launch_team2d_s1(const Step2DArgs &a, int variant, cudaStream_t s);
cudaError_t launch_team2d_s2(const Step2DArgs &a, int variant, cudaStream_t s);
constexpr int kStepVariantTeam = 32;
// The same for 32*S vertex slots per warp (dpm2d_step_s<S>.cu).
cudaError_t launch_step2d_s1(const Step2DArgs &a, int warps, int variant, cudaStream_t s);
cudaError_t launch_step2d_s2(const Step2DArgs &a, int warps, int variant, cudaStream_t s);
cudaError_t launch_step2d_s4(const Step2DArgs &a, int warps, int variant, cudaStream_t s);
cudaError_t launch_step2d_s8(const Step2DArgs &a, int warps, int variant, cudaStream_t s);
cudaError_t launch_step2d_s8_att(const Step2DArgs &a, int warps, int variant, cudaStream_t s);
constexpr int kStepVariantAttraction = 4;

// Host mirror of the bin arithmetic (for the host rebuild check).
int bin_axis_count(float L, float w, int cap);

} // namespace dpm
