// dpm2d_step_noalloc: the 2D step for one tissue without any device
// allocation.
//
// Who needs this: callers that cannot allocate device memory themselves or
// through this library -- a host program whose device memory is handed out
// by another framework's pool (a stray cudaMalloc there fails or fragments
// the pool), code that must not synchronize the device (cudaMalloc and
// cudaFree may), and embedded uses that reserve all memory at start-up.
// They pass their own device buffers for positions and forces; everything
// else the step needs (cell constants, geometry, the cell list and its sort,
// neighbour lists, the second position buffer) lives in one file-scope
// device array of fixed size, `g_dpm_noalloc_scratch` below, which every GPU
// that loads the library holds until the process exits.
//
// Limits: at most DPM_NOALLOC_MAX_CELLS cells and DPM_NOALLOC_MAX_VERTICES
// vertices (3..256 per cell), one tissue.  All calls share the array and
// its contents are not valid between calls; a process-wide lock serializes
// the calls (on every device) and each returns after its stream drains, so
// calls never overlap inside the library.  The first call on a device looks
// up the array's device address (cudaGetSymbolAddress) once for that device
// and keeps it for the life of the process (the primary context must not be
// reset between calls).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "dpm2d_kernels.cuh"
#include "dpm_common.cuh"
#include "radix_sort.cuh"

namespace dpm {
namespace {

constexpr int kMaxCells = DPM_NOALLOC_MAX_CELLS;
constexpr int kMaxVerts = DPM_NOALLOC_MAX_VERTICES;
constexpr int kPeriod = 16; // neighbour-list rebuild period (the batch default)

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte offsets of the regions of the scratch array.
constexpr size_t kOffCells = 0;
constexpr size_t kOffTissue = align256(kOffCells + sizeof(Cell2D) * kMaxCells);
constexpr size_t kOffGeom0 = align256(kOffTissue + sizeof(Tissue2D));
constexpr size_t kOffGeom1 = align256(kOffGeom0 + sizeof(Geom2D) * kMaxCells);
constexpr size_t kOffGeomR = align256(kOffGeom1 + sizeof(Geom2D) * kMaxCells);
constexpr size_t kOffNn = align256(kOffGeomR + sizeof(Geom2D) * kMaxCells);
constexpr size_t kOffNbr = align256(kOffNn + sizeof(int) * kMaxCells);
constexpr size_t kOffFlags = align256(kOffNbr + sizeof(int) * kMaxCells * kMaxNB2D);
constexpr size_t kOffKeys = align256(kOffFlags + 2 * sizeof(int));
constexpr size_t kOffSort = align256(kOffKeys + 4 * sizeof(uint32_t) * kMaxCells);
constexpr size_t kSortBytes = sizeof(uint32_t) * 256 * ((kMaxCells + 1023) / 1024) + 256;
constexpr size_t kOffPos = align256(kOffSort + kSortBytes);
constexpr size_t kScratchBytes = align256(kOffPos + sizeof(float2) * kMaxVerts);

// The scratch array (about 1.7 MB).  In host code its name is only a
// stand-in for the symbol: kernels get the address from
// cudaGetSymbolAddress, looked up once per device.
static __device__ __align__(256) unsigned char g_dpm_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
constexpr int kMaxDevices = 64;
unsigned char *g_addr[kMaxDevices] = {};
// Host staging of the per-cell constants (guarded by g_mu).
Cell2D g_host_cells[kMaxCells];

int scratch_address(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return fail(DPM_ECAPACITY, "device id too large");
  if (!g_addr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_dpm_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_dpm_noalloc_scratch)");
    g_addr[device] = static_cast<unsigned char *>(p);
  }
  *out = g_addr[device];
  return DPM_OK;
}

int ceil_log2i(long v) {
  int b = 0;
  while ((1L << b) < v) ++b;
  return b;
}

} // namespace
} // namespace dpm

using namespace dpm;

extern "C" int dpm2d_step_noalloc(int ncells, const unsigned *nv, const float *Ka,
                                  const float *Kl, const float *Kb, const float *a0,
                                  const float *l0, const float *r0, float L, float Kre,
                                  float Kat, int pbc, float *xy_dev, float *F_dev, int nsteps,
                                  float dt, void *stream_ptr) {
  if (!nv || !Ka || !Kl || !Kb || !a0 || !l0 || !r0 || !xy_dev)
    return fail(DPM_EINVAL, "null argument");
  if (ncells <= 0) return fail(DPM_EINVAL, "ncells must be positive");
  if (ncells > kMaxCells)
    return fail(DPM_ECAPACITY, "dpm2d_step_noalloc: more than DPM_NOALLOC_MAX_CELLS (2048) cells");
  if (nsteps < 0) return fail(DPM_EINVAL, "nsteps must be non-negative");
  if (!std::isfinite(dt)) return fail(DPM_EINVAL, "dt must be finite");
  if (!(L > 0.0f) || !std::isfinite(L)) return fail(DPM_EINVAL, "L must be positive");
  long total = 0;
  float l0max = 0.0f, a0max = 0.0f;
  double rsum = 0.0;
  for (int c = 0; c < ncells; ++c) {
    if (nv[c] < 3 || nv[c] > (unsigned)kMaxNV2D)
      return fail(DPM_EINVAL, "every cell needs 3..256 vertices");
    if (!(a0[c] > 0.0f) || !(l0[c] > 0.0f) || !(r0[c] > 0.0f))
      return fail(DPM_EINVAL, "a0, l0 and r0 must be positive");
    total += nv[c];
    l0max = std::fmax(l0max, l0[c]);
    a0max = std::fmax(a0max, a0[c]);
    rsum += r0[c];
  }
  if (total > kMaxVerts)
    return fail(DPM_ECAPACITY,
                "dpm2d_step_noalloc: more than DPM_NOALLOC_MAX_VERTICES (65536) vertices");
  if (nsteps == 0) return DPM_OK;  // nothing to step: no device work

  std::lock_guard<std::mutex> lock(g_mu);
  int device = 0;
  DPM_CUDA_TRY(cudaGetDevice(&device));
  unsigned char *base = nullptr;
  if (int r = scratch_address(device, &base)) return r;
  cudaStream_t s = static_cast<cudaStream_t>(stream_ptr);

  Cell2D *cells = reinterpret_cast<Cell2D *>(base + kOffCells);
  Tissue2D *tissue = reinterpret_cast<Tissue2D *>(base + kOffTissue);
  Geom2D *geom[2] = {reinterpret_cast<Geom2D *>(base + kOffGeom0),
                     reinterpret_cast<Geom2D *>(base + kOffGeom1)};
  Geom2D *geom0 = reinterpret_cast<Geom2D *>(base + kOffGeomR);
  int *nn = reinterpret_cast<int *>(base + kOffNn);
  int *nbr = reinterpret_cast<int *>(base + kOffNbr);
  int *stale = reinterpret_cast<int *>(base + kOffFlags);
  int *err = stale + 1;
  uint32_t *keys = reinterpret_cast<uint32_t *>(base + kOffKeys);
  uint32_t *vals = keys + kMaxCells, *keys_alt = vals + kMaxCells, *vals_alt = keys_alt + kMaxCells;
  uint32_t *sort_scratch = reinterpret_cast<uint32_t *>(base + kOffSort);
  float2 *pos[2] = {reinterpret_cast<float2 *>(xy_dev), reinterpret_cast<float2 *>(base + kOffPos)};

  // per-cell and per-tissue constants, formed as dpm2d_set_cells/_tissues do
  uint32_t off = 0;
  for (int c = 0; c < ncells; ++c) {
    Cell2D &C = g_host_cells[c];
    std::memset(&C, 0, sizeof(C));
    C.voff = off;
    C.nv = nv[c];
    C.tissue = 0;
    C.a0 = a0[c];
    C.l0 = l0[c];
    C.kA = Ka[c] / std::sqrt(a0[c]);
    C.kL = Kl[c] * std::sqrt(a0[c] / l0[c]);
    C.Kb = Kb[c];
    C.r0 = r0[c];
    C.inv_l0 = 1.0f / l0[c];
    C.inv_2r0 = 1.0f / (2.0f * r0[c]);
    off += nv[c];
  }
  Tissue2D T;
  std::memset(&T, 0, sizeof(T));
  T.L = L;
  T.Kre = Kre;
  T.Kat = Kat;
  T.l0max = l0max;
  T.pbc = pbc ? 1 : 0;
  T.cell_begin = 0;
  T.cell_end = ncells;
  T.skin = (float)(0.15 * 2.0 * rsum / ncells);
  const double rad = std::sqrt(a0max / M_PI);
  long cap = (long)std::floor(L / std::max(rad, 1e-6));
  cap = std::max(1L, std::min(cap, (long)kMaxBinsAxis));
  T.cap = (int)cap;
  T.nbx = T.nby = 1;
  T.cell_cap = ncells;
  T.steps_left = kStepsUnlimited;
  T.run_now = kStepsUnlimited;
  const int local_bits = std::max(1, ceil_log2i(cap * cap));

  // everything that must start at zero: neighbour counts, stale and error flags
  DPM_CUDA_TRY(cudaMemcpyAsync(cells, g_host_cells, sizeof(Cell2D) * ncells,
                               cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(tissue, &T, sizeof(T), cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemsetAsync(nn, 0, sizeof(int) * ncells, s));
  DPM_CUDA_TRY(cudaMemsetAsync(stale, 0, 2 * sizeof(int), s));
  if (F_dev) DPM_CUDA_TRY(cudaMemsetAsync(F_dev, 0, sizeof(float2) * total, s));
  DPM_CUDA_TRY(launch_geom2d(cells, pos[0], geom[0], ncells, 0, s));

  Rebuild2DArgs rb{};
  rb.cells = cells;
  rb.tissues = tissue;
  rb.geom0 = geom0;
  rb.keys = keys;
  rb.vals = vals;
  rb.nn = nn;
  rb.nbr = nbr;
  rb.stale = stale;
  rb.ncells = ncells;
  rb.ntissues = 1;
  int maxnv = 0;
  for (int c = 0; c < ncells; ++c) maxnv = std::max(maxnv, (int)nv[c]);

  int cur = 0;
  for (int done = 0; done < nsteps;) {
    const int len = std::min(kPeriod, nsteps - done);
    rb.geom = geom[cur];
    rb.block_len = len;
    DPM_CUDA_TRY(launch_binprep2d(rb, local_bits, s));
    bool alt = false;
    DPM_CUDA_TRY(radix_sort_pairs(keys, vals, keys_alt, vals_alt, ncells, local_bits,
                                  sort_scratch, s, &alt));
    rb.sorted_keys = alt ? keys_alt : keys;
    rb.sorted_vals = alt ? vals_alt : vals;
    DPM_CUDA_TRY(launch_neighbors2d(rb, local_bits, s));
    for (int i = 0; i < len; ++i) {
      Step2DArgs a{};
      a.cells = cells;
      a.tissues = tissue;
      a.pos_in = pos[cur];
      a.pos_out = pos[1 - cur];
      a.force_out = (done + i == nsteps - 1) ? reinterpret_cast<float2 *>(F_dev) : nullptr;
      a.flags_out = nullptr;
      a.geom_in = geom[cur];
      a.geom_out = geom[1 - cur];
      a.geom0 = geom0;
      a.nn = nn;
      a.nbr = nbr;
      a.stale = stale;
      a.err = err;
      a.ncells = ncells;
      a.dt = dt;
      a.step_index = i;
      a.all_forces = 1;
      DPM_CUDA_TRY(launch_step2d(a, maxnv, 8, Kat != 0.0f ? 1 | kStepVariantAttraction : 1, s));
      cur = 1 - cur;
    }
    done += len;
  }
  if (cur == 1)
    DPM_CUDA_TRY(cudaMemcpyAsync(xy_dev, pos[1], sizeof(float2) * total,
                                 cudaMemcpyDeviceToDevice, s));
  int herr = 0;
  DPM_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  if (herr & 1) return fail(DPM_ENONFINITE, "non-finite vertex positions");
  return DPM_OK;
}
