// Runtime of the 2D path: context, batch objects, captured step graphs and
// the C ABI declared in include/dpm_gb300.h.
//
// A call dpm2d_step(b, n, dt) runs n steps as blocks of `rebuild_period`
// steps.  Each block is one CUDA graph: the cell-list rebuild (per-tissue
// bins and keys, a stable device radix sort of the keys, neighbour lists)
// followed by `rebuild_period` launches of the fused step kernel, the last
// of which also stores the forces and containment flags when it ends the
// call.  Graphs are instantiated once per (block length, parity, dt, last)
// and replayed.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "ckpt_io.hpp"
#include "dpm2d_kernels.cuh"
#include "dpm_common.cuh"
#include "dpm_runtime.hpp"
#include "radix_sort.cuh"

namespace dpm {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char *what) {
  g_last_error = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
  return DPM_ECUDA;
}
const char *last_error() { return g_last_error.c_str(); }

void ctx_retain(dpm_ctx *ctx) { ctx->refs.fetch_add(1); }

void ctx_release(dpm_ctx *ctx) {
  if (ctx->refs.fetch_sub(1) != 1) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

static int ceil_log2(long v) {
  int b = 0;
  while ((1L << b) < v) ++b;
  return b;
}

} // namespace dpm

using namespace dpm;

struct dpm2d_batch {
  dpm_ctx *ctx = nullptr;
  cudaStream_t stream = nullptr; // the context's, or the pool's own
  bool own_stream = false;
  int ntissues = 0, ncells = 0, maxnv = 0;
  long nverts = 0;
  std::vector<int> tissue_ncells;
  std::vector<unsigned> nv;
  std::vector<uint32_t> voff;
  std::vector<Cell2D> h_cells;
  std::vector<float> h_Ka, h_Kl;  // spring constants as given (for the energy)
  std::vector<Tissue2D> h_tissues;
  bool cells_set = false, tissues_set = false, uploaded = false;

  DeviceArena arena;
  Cell2D *d_cells = nullptr;
  Tissue2D *d_tissues = nullptr;
  float2 *d_pos[2] = {nullptr, nullptr};
  float2 *d_force = nullptr;
  unsigned char *d_flags = nullptr;
  Geom2D *d_geom[2] = {nullptr, nullptr};
  Geom2D *d_geom0 = nullptr;
  int *d_nn = nullptr, *d_nbr = nullptr, *d_stale = nullptr, *d_err = nullptr;
  int *d_sched = nullptr; // dynamic-schedule counters of the step kernel (per class)
  float *d_phi = nullptr; // per-tissue packing fractions of a rescale

  // Vertex-slot classes (rings of at most 32, 64, 128, 256 vertices, one
  // warp lane holding 1, 2, 4, 8 of them).  A cell's class is that of its
  // tissue's largest ring.  A batch whose tissues fall into more than one
  // class launches one step kernel per class over its own cells
  // (d_order[class_begin[k] .. class_begin[k+1])), side by side on two
  // streams (a fork and join inside the captured graph), so that every
  // tissue runs the code compiled for its ring sizes.
  int nclass = 1;
  int class_begin[5] = {0, 0, 0, 0, 0};

  // Resident run (k2d_run_resident): batches whose tissues are all small
  // (at most kResidentMaxCells cells and kResidentMaxVerts vertices, rings of
  // at most 64) step with one block per tissue holding it in shared memory
  // for a whole call, unless switched off (variant bit 3).
  bool resident_fits = false, no_resident = false;
  int res_ncmax = 0, res_nvmax = 0;
  int *d_order = nullptr;
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  uint32_t *d_keys = nullptr, *d_vals = nullptr, *d_keys_alt = nullptr, *d_vals_alt = nullptr;
  uint32_t *d_sort_scratch = nullptr;
  int cur = 0;
  int local_bits = 1, key_bits = 1;
  bool sorted_in_alt = false;

  int rebuild_period = 16;
  float skin_rel = 0.15f;
  int warps = 8;
  int occ = 1;
  bool att = false;     // some tissue has Kat != 0: launch the step with attraction
  bool team = false;    // variant bit 5: four warps per cell (no attraction, rings <= 64)
  bool serving = false; // slot pool of a server: per-tissue step budgets
  long rebuilds = 0;

  // slot pools: launches cover the tissues [0, run_tissues) and their cells
  // [0, run_cells) only (0: all); the server keeps occupied slots low
  int run_tissues = 0, run_cells = 0;
  int nc() const { return run_cells ? run_cells : ncells; }
  int nt() const { return run_tissues ? run_tissues : ntissues; }

  std::map<std::tuple<int, int, uint32_t, int, int>, cudaGraphExec_t> graphs;

  ~dpm2d_batch() {
    clear_graphs();
    if (own_stream && stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
    if (aux) {
      cudaStreamSynchronize(aux);
      cudaStreamDestroy(aux);
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
  }
  void clear_graphs() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
  }
  // the step kernel's variant: the tuned occupancy/schedule bits, and the
  // attraction compiled in only when a tissue uses it
  int variant() const { return occ | (att ? kStepVariantAttraction : 0); }

  Rebuild2DArgs rebuild_args() const {
    Rebuild2DArgs a{};
    a.cells = d_cells;
    a.tissues = d_tissues;
    a.geom = d_geom[cur];
    a.geom0 = d_geom0;
    a.keys = d_keys;
    a.vals = d_vals;
    a.sorted_keys = sorted_in_alt ? d_keys_alt : d_keys;
    a.sorted_vals = sorted_in_alt ? d_vals_alt : d_vals;
    a.nn = d_nn;
    a.nbr = d_nbr;
    a.stale = d_stale;
    a.ncells = nc();
    a.ntissues = nt();
    return a;
  }

  // Enqueue one neighbour-list rebuild on geometry buffer `g`, for a rebuild
  // period of block_len steps (0: leave the step budgets untouched).
  cudaError_t enqueue_rebuild(int g, int block_len, cudaStream_t s) {
    Rebuild2DArgs a = rebuild_args();
    a.geom = d_geom[g];
    a.block_len = block_len;
    cudaError_t e = launch_binprep2d(a, local_bits, s);
    if (e != cudaSuccess) return e;
    bool alt = false;
    e = radix_sort_pairs(d_keys, d_vals, d_keys_alt, d_vals_alt, nc(), key_bits,
                         d_sort_scratch, s, &alt);
    if (e != cudaSuccess) return e;
    sorted_in_alt = alt;
    a.sorted_keys = alt ? d_keys_alt : d_keys;
    a.sorted_vals = alt ? d_vals_alt : d_vals;
    return launch_neighbors2d(a, local_bits, s);
  }

  Step2DArgs step_args(int from, float dt, bool last, int index) const {
    Step2DArgs a{};
    a.cells = d_cells;
    a.tissues = d_tissues;
    a.pos_in = d_pos[from];
    a.pos_out = d_pos[1 - from];
    if (serving) {
      // each tissue stores its outputs at the last step of its own budget
      a.force_out = d_force;
      a.flags_out = d_flags;
      a.all_forces = 0;
    } else {
      a.force_out = last ? d_force : nullptr;
      a.flags_out = last ? d_flags : nullptr;
      a.all_forces = 1;
    }
    a.step_index = index;
    a.geom_in = d_geom[from];
    a.geom_out = d_geom[1 - from];
    a.geom0 = d_geom0;
    a.nn = d_nn;
    a.nbr = d_nbr;
    a.stale = d_stale;
    a.err = d_err;
    a.sched = d_sched;
    a.ncells = nc();
    a.dt = dt;
    return a;
  }

  // One launch of the step over a's cells, whose rings have at most maxnv_k
  // vertices: the team kernel when it is chosen and applies, else one warp
  // per cell.
  cudaError_t launch_one(const Step2DArgs &a, int maxnv_k, cudaStream_t s) const {
    if (team && !att && maxnv_k <= 64)
      return maxnv_k <= 32 ? launch_team2d_s1(a, occ, s) : launch_team2d_s2(a, occ, s);
    return launch_step2d(a, maxnv_k, warps, variant(), s);
  }

  // One step of every cell: a single launch, or one launch per vertex-slot
  // class (by the tissue's largest ring), the largest rings first on the
  // auxiliary stream and the smallest on `s`, joined back into `s`.  The
  // classes write disjoint cells and read only the step's inputs, so their
  // order does not matter.
  cudaError_t launch_step(const Step2DArgs &a0, cudaStream_t s) {
    if (serving) return launch_step2d(a0, maxnv, warps, variant(), s);
    if (nclass <= 1) return launch_one(a0, maxnv, s);
    cudaError_t e = cudaEventRecord(ev_fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, ev_fork, 0);
    int first = 0;
    while (class_begin[first + 1] == class_begin[first]) ++first;
    for (int k = 3; k >= first && e == cudaSuccess; --k) {
      const int n = class_begin[k + 1] - class_begin[k];
      if (n == 0) continue;
      Step2DArgs a = a0;
      a.order = d_order + class_begin[k];
      a.ncells = n;
      a.sched = d_sched + 2 * k;
      e = launch_one(a, 32 << k, k == first ? s : aux);
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev_join, aux);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev_join, 0);
    return e;
  }

  // Enqueue a block: rebuild, then `len` steps starting from buffer `from`.
  cudaError_t enqueue_block(int len, int from, float dt, bool last, cudaStream_t s) {
    cudaError_t e = enqueue_rebuild(from, len, s);
    if (e != cudaSuccess) return e;
    int f = from;
    for (int i = 0; i < len; ++i) {
      e = launch_step(step_args(f, dt, last && i == len - 1, i), s);
      if (e != cudaSuccess) return e;
      f = 1 - f;
    }
    return cudaSuccess;
  }

  bool resident() const { return resident_fits && !no_resident && !serving; }

  // A call of nsteps on the resident run: launches of up to 4096 steps each;
  // the positions and geometry stay in buffer `cur`.
  int run_resident(int nsteps, float dt) {
    constexpr int kChunk = 4096;
    for (int done = 0; done < nsteps;) {
      const int len = std::min(kChunk, nsteps - done);
      Resident2DArgs r{};
      r.a = step_args(cur, dt, done + len == nsteps, 0);
      r.pos = d_pos[cur];
      r.geom = d_geom[cur];
      r.nsteps = len;
      r.ncmax = res_ncmax;
      r.nvmax = res_nvmax;
      DPM_CUDA_TRY(launch_resident2d(r, ntissues, maxnv, variant(), stream));
      done += len;
    }
    return DPM_OK;
  }

  int run_block(int len, float dt, bool last) {
    cudaStream_t s = stream;
    uint32_t dtbits;
    std::memcpy(&dtbits, &dt, 4);
    auto key = std::make_tuple(len, cur, dtbits, last ? 1 : 0, nc());
    auto it = graphs.find(key);
    if (it == graphs.end()) {
      cudaGraph_t g = nullptr;
      DPM_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = enqueue_block(len, cur, dt, last, s);
      cudaError_t e2 = cudaStreamEndCapture(s, &g);
      if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(e, "enqueue_block");
      }
      if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
      cudaGraphExec_t ex = nullptr;
      e = cudaGraphInstantiate(&ex, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
      it = graphs.emplace(key, ex).first;
    }
    DPM_CUDA_TRY(cudaGraphLaunch(it->second, s));
    if (len % 2) cur = 1 - cur;
    ++rebuilds;
    return DPM_OK;
  }
};

namespace {

int check_batch(dpm2d_batch *b) {
  if (!b) return fail(DPM_EINVAL, "null batch");
  return DPM_OK;
}

} // namespace

extern "C" {

const char *dpm_last_error(void) { return dpm::last_error(); }
const char *dpm_version(void) { return "dpm_gb300 0.1 (sm_103a)"; }

int dpm_ctx_create(int device, dpm_ctx **out) {
  if (!out) return fail(DPM_EINVAL, "null output pointer");
  *out = nullptr;
  int n = 0;
  DPM_CUDA_TRY(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(DPM_EINVAL, "no such CUDA device");
  DPM_CUDA_TRY(cudaSetDevice(device));
  auto *c = new (std::nothrow) dpm_ctx();
  if (!c) return fail(DPM_ECAPACITY, "out of host memory");
  c->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaStreamCreate");
  }
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  *out = c;
  return DPM_OK;
}

int dpm_ctx_destroy(dpm_ctx *ctx) {
  if (!ctx) return DPM_OK;
  dpm::ctx_release(ctx);
  return DPM_OK;
}

int dpm_ctx_synchronize(dpm_ctx *ctx) {
  if (!ctx) return fail(DPM_EINVAL, "null context");
  DPM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return DPM_OK;
}

int dpm_ctx_sm_count(dpm_ctx *ctx, int *out) {
  if (!ctx || !out) return fail(DPM_EINVAL, "null argument");
  *out = ctx->sm_count;
  return DPM_OK;
}

int dpm_ctx_stream(dpm_ctx *ctx, void **stream) {
  if (!ctx || !stream) return fail(DPM_EINVAL, "null argument");
  *stream = (void *)ctx->stream;
  return DPM_OK;
}

int dpm2d_create(dpm_ctx *ctx, int ntissues, const int *ncells, const unsigned *nv,
                 dpm2d_batch **out) {
  if (!ctx || !ncells || !nv || !out) return fail(DPM_EINVAL, "null argument");
  *out = nullptr;
  if (ntissues <= 0) return fail(DPM_EINVAL, "ntissues must be positive");
  if (ntissues > 4096) return fail(DPM_ECAPACITY, "at most 4096 tissues per batch");
  try {
    auto b = std::make_unique<dpm2d_batch>();
    b->ctx = ctx;
    b->stream = ctx->stream;
    b->ntissues = ntissues;
    long total_cells = 0;
    for (int t = 0; t < ntissues; ++t) {
      if (ncells[t] <= 0) return fail(DPM_EINVAL, "every tissue needs at least one cell");
      total_cells += ncells[t];
    }
    if (total_cells > (1L << 26)) return fail(DPM_ECAPACITY, "too many cells");
    b->ncells = (int)total_cells;
    b->tissue_ncells.assign(ncells, ncells + ntissues);
    b->nv.assign(nv, nv + total_cells);
    b->voff.resize(total_cells);
    long off = 0;
    for (long c = 0; c < total_cells; ++c) {
      if (nv[c] < 3 || nv[c] > (unsigned)kMaxNV2D)
        return fail(DPM_EINVAL, "every cell needs 3..256 vertices");
      b->voff[c] = (uint32_t)off;
      off += nv[c];
      b->maxnv = std::max(b->maxnv, (int)nv[c]);
    }
    if (off > (1L << 31) - 1) return fail(DPM_ECAPACITY, "too many vertices");
    b->nverts = off;
    // vertex-slot classes and the cells of each, in cell order.  A cell's
    // class is that of the largest ring of its TISSUE: the step holds the
    // neighbours' rings (cells of the same tissue) in the same slots as its
    // own, so every cell of a tissue runs the code of the tissue's largest
    // ring.
    auto slot_class = [](unsigned v) { return v <= 32 ? 0 : v <= 64 ? 1 : v <= 128 ? 2 : 3; };
    std::vector<unsigned char> cls(total_cells);
    {
      long c0 = 0;
      for (int t = 0; t < ntissues; ++t) {
        unsigned m = 0;
        for (long c = c0; c < c0 + ncells[t]; ++c) m = std::max(m, nv[c]);
        for (long c = c0; c < c0 + ncells[t]; ++c) cls[c] = (unsigned char)slot_class(m);
        c0 += ncells[t];
      }
    }
    {
      long c0 = 0;
      bool fits = b->maxnv <= 64;
      for (int t = 0; t < ntissues; ++t) {
        long v = 0;
        for (long c = c0; c < c0 + ncells[t]; ++c) v += nv[c];
        fits = fits && ncells[t] <= kResidentMaxCells && v <= kResidentMaxVerts;
        b->res_ncmax = std::max(b->res_ncmax, ncells[t]);
        b->res_nvmax = std::max(b->res_nvmax, (int)v);
        c0 += ncells[t];
      }
      b->resident_fits = fits;
    }
    int cnt[4] = {0, 0, 0, 0};
    for (long c = 0; c < total_cells; ++c) ++cnt[cls[c]];
    b->nclass = (cnt[0] > 0) + (cnt[1] > 0) + (cnt[2] > 0) + (cnt[3] > 0);
    std::vector<int> order;
    if (b->nclass > 1) {
      for (int k = 0; k < 4; ++k) b->class_begin[k + 1] = b->class_begin[k] + cnt[k];
      order.resize(total_cells);
      int fill[4] = {b->class_begin[0], b->class_begin[1], b->class_begin[2], b->class_begin[3]};
      for (long c = 0; c < total_cells; ++c) order[fill[cls[c]]++] = (int)c;
    }
    b->h_cells.resize(total_cells);
    b->h_Ka.assign(total_cells, 0.0f);
    b->h_Kl.assign(total_cells, 0.0f);
    b->h_tissues.resize(ntissues);
    int cb = 0;
    for (int t = 0; t < ntissues; ++t) {
      Tissue2D &T = b->h_tissues[t];
      std::memset(&T, 0, sizeof(T));
      T.cell_begin = cb;
      T.cell_end = cb + ncells[t];
      T.cap = 1;
      T.nbx = T.nby = 1;
      T.cell_cap = T.cell_end;
      T.steps_left = kStepsUnlimited;
      T.run_now = kStepsUnlimited;
      for (int c = cb; c < cb + ncells[t]; ++c) {
        Cell2D &C = b->h_cells[c];
        std::memset(&C, 0, sizeof(C));
        C.voff = b->voff[c];
        C.nv = b->nv[c];
        C.tissue = (uint32_t)t;
      }
      cb += ncells[t];
    }
    const long V = b->nverts, N = b->ncells;
    DeviceArena &A = b->arena;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    e = A.reserve(sizeof(Cell2D) * N + sizeof(Tissue2D) * ntissues + 3 * sizeof(float2) * V +
                  V + 3 * sizeof(Geom2D) * N + sizeof(int) * (N + N * kMaxNB2D) +
                  sizeof(int) * (ntissues + 1) + sizeof(float) * ntissues + sizeof(int) * 8 +
                  (b->nclass > 1 ? sizeof(int) * N : 0) +
                  4 * sizeof(uint32_t) * N +
                  radix_sort_scratch_bytes((int)N) + 64 * 256);
    if (e != cudaSuccess) return cuda_fail(e, "device allocation");
    b->d_cells = A.take<Cell2D>(N);
    b->d_tissues = A.take<Tissue2D>(ntissues);
    b->d_pos[0] = A.take<float2>(V);
    b->d_pos[1] = A.take<float2>(V);
    b->d_force = A.take<float2>(V);
    b->d_flags = A.take<unsigned char>(V);
    b->d_geom[0] = A.take<Geom2D>(N);
    b->d_geom[1] = A.take<Geom2D>(N);
    b->d_geom0 = A.take<Geom2D>(N);
    b->d_nn = A.take<int>(N);
    b->d_nbr = A.take<int>(N * kMaxNB2D);
    b->d_stale = A.take<int>(ntissues);
    b->d_err = A.take<int>(1);
    b->d_sched = A.take<int>(8);
    b->d_phi = A.take<float>(ntissues);
    if (b->nclass > 1) b->d_order = A.take<int>(N);
    b->d_keys = A.take<uint32_t>(N);
    b->d_vals = A.take<uint32_t>(N);
    b->d_keys_alt = A.take<uint32_t>(N);
    b->d_vals_alt = A.take<uint32_t>(N);
    b->d_sort_scratch = A.take<uint32_t>(radix_sort_scratch_bytes((int)N) / 4 + 1);
    if (!A.ok()) return fail(DPM_ECAPACITY, "device arena exhausted");
    e = cudaMemsetAsync(A.base(), 0, A.used(), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemset");
    if (b->nclass > 1) {
      e = cudaMemcpyAsync(b->d_order, order.data(), sizeof(int) * N, cudaMemcpyHostToDevice,
                          ctx->stream);
      if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->aux, cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) return cuda_fail(e, "vertex-slot classes");
    }
    *out = b.release();
    ctx_retain(ctx);
    return DPM_OK;
  } catch (const std::bad_alloc &) {
    return fail(DPM_ECAPACITY, "out of host memory");
  }
}

int dpm2d_destroy(dpm2d_batch *b) {
  if (!b) return DPM_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->stream);
  dpm_ctx *c = b->ctx;
  delete b;
  ctx_release(c);
  return DPM_OK;
}

int dpm2d_sizes(dpm2d_batch *b, int *ncells, long *nvertices) {
  if (int r = check_batch(b)) return r;
  if (ncells) *ncells = b->ncells;
  if (nvertices) *nvertices = b->nverts;
  return DPM_OK;
}

int dpm2d_set_cells(dpm2d_batch *b, const float *Ka, const float *Kl, const float *Kb,
                    const float *a0, const float *l0, const float *r0) {
  if (int r = check_batch(b)) return r;
  if (!Ka || !Kl || !Kb || !a0 || !l0 || !r0) return fail(DPM_EINVAL, "null parameter array");
  b->h_Ka.assign(Ka, Ka + b->ncells);
  b->h_Kl.assign(Kl, Kl + b->ncells);
  for (int c = 0; c < b->ncells; ++c) {
    if (!(a0[c] > 0.0f) || !(l0[c] > 0.0f) || !(r0[c] > 0.0f))
      return fail(DPM_EINVAL, "a0, l0 and r0 must be positive");
    Cell2D &C = b->h_cells[c];
    C.a0 = a0[c];
    C.l0 = l0[c];
    // the reference forms these in float (Cell2D_kernel.cl:38, :118)
    C.kA = Ka[c] / std::sqrt(a0[c]);
    C.kL = Kl[c] * std::sqrt(a0[c] / l0[c]);
    C.Kb = Kb[c];
    C.r0 = r0[c];
    C.inv_l0 = 1.0f / l0[c];
    C.inv_2r0 = 1.0f / (2.0f * r0[c]);
  }
  // attraction range, skin and bin cap depend on the cells of each tissue
  for (int t = 0; t < b->ntissues; ++t) {
    Tissue2D &T = b->h_tissues[t];
    float l0max = 0.0f, a0max = 0.0f;
    double rsum = 0.0;
    for (int c = T.cell_begin; c < T.cell_end; ++c) {
      l0max = std::max(l0max, b->h_cells[c].l0);
      a0max = std::max(a0max, b->h_cells[c].a0);
      rsum += b->h_cells[c].r0;
    }
    T.l0max = l0max;
    T.skin = (float)(b->skin_rel * 2.0 * rsum / (T.cell_end - T.cell_begin));
  }
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_cells, b->h_cells.data(), sizeof(Cell2D) * b->ncells,
                               cudaMemcpyHostToDevice, b->stream));
  b->cells_set = true;
  if (b->tissues_set) {
    DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(),
                                 sizeof(Tissue2D) * b->ntissues, cudaMemcpyHostToDevice,
                                 b->stream));
  }
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DPM_OK;
}

int dpm2d_set_tissues(dpm2d_batch *b, const float *L, const float *Kre, const float *Kat,
                      const int *pbc) {
  if (int r = check_batch(b)) return r;
  if (!L || !Kre || !Kat || !pbc) return fail(DPM_EINVAL, "null parameter array");
  int max_local = 1;
  bool att = false;
  for (int t = 0; t < b->ntissues; ++t) {
    if (!(L[t] > 0.0f) || !std::isfinite(L[t])) return fail(DPM_EINVAL, "L must be positive");
    Tissue2D &T = b->h_tissues[t];
    T.L = L[t];
    T.Kre = Kre[t];
    T.Kat = Kat[t];
    T.pbc = pbc[t] ? 1 : 0;
    att |= Kat[t] != 0.0f;
    // bins per axis never need to be narrower than a cell radius
    float a0max = 0.0f;
    for (int c = T.cell_begin; c < T.cell_end; ++c) a0max = std::max(a0max, b->h_cells[c].a0);
    const double rad = a0max > 0.0f ? std::sqrt(a0max / M_PI) : 0.5;
    long cap = (long)std::floor(L[t] / std::max(rad, 1e-6));
    cap = std::max(1L, std::min(cap, (long)kMaxBinsAxis));
    T.cap = (int)cap;
    max_local = std::max(max_local, ceil_log2(cap * cap));
  }
  b->local_bits = std::max(1, max_local);
  b->key_bits = b->local_bits + ceil_log2(b->ntissues);
  if (b->key_bits > 32) return fail(DPM_ECAPACITY, "cell-list keys exceed 32 bits");
  b->att = att;
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(), sizeof(Tissue2D) * b->ntissues,
                               cudaMemcpyHostToDevice, b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->tissues_set = true;
  b->clear_graphs();
  return DPM_OK;
}

int dpm2d_set_tuning(dpm2d_batch *b, int rebuild_period, float skin_rel, int warps_per_block) {
  if (int r = check_batch(b)) return r;
  if (rebuild_period > 0) {
    if (rebuild_period % 2) return fail(DPM_EINVAL, "rebuild period must be even");
    b->rebuild_period = rebuild_period;
  }
  if (skin_rel > 0.0f) b->skin_rel = skin_rel;
  if (warps_per_block > 0) {
    if (warps_per_block != 4 && warps_per_block != 8 && warps_per_block != 16)
      return fail(DPM_EINVAL, "warps per block must be 4, 8 or 16");
    b->warps = warps_per_block;
  }
  b->clear_graphs();
  if (b->cells_set && skin_rel > 0.0f) {
    for (int t = 0; t < b->ntissues; ++t) {
      Tissue2D &T = b->h_tissues[t];
      double rsum = 0.0;
      for (int c = T.cell_begin; c < T.cell_end; ++c) rsum += b->h_cells[c].r0;
      T.skin = (float)(b->skin_rel * 2.0 * rsum / (T.cell_end - T.cell_begin));
    }
    if (b->tissues_set) {
      cudaSetDevice(b->ctx->device);
      DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(),
                                   sizeof(Tissue2D) * b->ntissues, cudaMemcpyHostToDevice,
                                   b->stream));
      DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
    }
  }
  return DPM_OK;
}

int dpm2d_set_kernel_variant(dpm2d_batch *b, int variant) {
  if (int r = check_batch(b)) return r;
  if (variant < 0 || (variant & ~(3 | 8 | kStepVariantTeam)) != 0)
    return fail(DPM_EINVAL, "step-kernel variant must be 0..3, plus 8 to switch off the resident "
                            "run and 32 for four warps per cell");
  b->occ = variant & 3;
  b->team = (variant & kStepVariantTeam) != 0;
  b->no_resident = (variant & 8) != 0;
  b->clear_graphs();
  return DPM_OK;
}

int dpm2d_upload(dpm2d_batch *b, const float *xy) {
  if (int r = check_batch(b)) return r;
  if (!xy) return fail(DPM_EINVAL, "null positions");
  if (!b->cells_set) return fail(DPM_ESTATE, "set the cell constants before uploading");
  cudaSetDevice(b->ctx->device);
  cudaStream_t s = b->stream;
  b->cur = 0;
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_pos[0], xy, sizeof(float2) * b->nverts,
                               cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemsetAsync(b->d_force, 0, sizeof(float2) * b->nverts, s));
  DPM_CUDA_TRY(cudaMemsetAsync(b->d_flags, 0, b->nverts, s));
  DPM_CUDA_TRY(cudaMemsetAsync(b->d_err, 0, sizeof(int), s));
  DPM_CUDA_TRY(launch_geom2d(b->d_cells, b->d_pos[0], b->d_geom[0], b->ncells, b->maxnv, s));
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  b->uploaded = true;
  return DPM_OK;
}

int dpm2d_step_kernel(dpm2d_batch *b, float dt) {
  if (int r = check_batch(b)) return r;
  if (!b->uploaded || !b->tissues_set) return fail(DPM_ESTATE, "upload before stepping");
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(b->launch_step(b->step_args(b->cur, dt, true, 0), b->stream));
  b->cur = 1 - b->cur;
  return DPM_OK;
}

int dpm2d_step(dpm2d_batch *b, int nsteps, float dt) {
  if (int r = check_batch(b)) return r;
  if (nsteps < 0) return fail(DPM_EINVAL, "nsteps must be non-negative");
  if (!b->uploaded || !b->cells_set || !b->tissues_set)
    return fail(DPM_ESTATE, "set cells and tissues and upload positions before stepping");
  if (!std::isfinite(dt)) return fail(DPM_EINVAL, "dt must be finite");
  if (nsteps == 0) return DPM_OK;
  cudaSetDevice(b->ctx->device);
  if (b->resident()) return b->run_resident(nsteps, dt);
  const int R = b->rebuild_period;
  const int full = nsteps / R, rem = nsteps % R;
  for (int i = 0; i < full; ++i)
    if (int r = b->run_block(R, dt, rem == 0 && i == full - 1)) return r;
  if (rem)
    if (int r = b->run_block(rem, dt, true)) return r;
  return DPM_OK;
}

int dpm2d_download(dpm2d_batch *b, float *xy, float *F) {
  if (int r = check_batch(b)) return r;
  if (!b->uploaded) return fail(DPM_ESTATE, "nothing uploaded");
  cudaSetDevice(b->ctx->device);
  cudaStream_t s = b->stream;
  if (xy)
    DPM_CUDA_TRY(cudaMemcpyAsync(xy, b->d_pos[b->cur], sizeof(float2) * b->nverts,
                                 cudaMemcpyDeviceToHost, s));
  if (F)
    DPM_CUDA_TRY(cudaMemcpyAsync(F, b->d_force, sizeof(float2) * b->nverts,
                                 cudaMemcpyDeviceToHost, s));
  int err = 0;
  DPM_CUDA_TRY(cudaMemcpyAsync(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  if (err & 1) return fail(DPM_ENONFINITE, "non-finite vertex positions");
  return DPM_OK;
}

int dpm2d_device_state(dpm2d_batch *b, void **positions, void **forces) {
  if (int r = check_batch(b)) return r;
  if (positions) *positions = b->d_pos[b->cur];
  if (forces) *forces = b->d_force;
  return DPM_OK;
}

int dpm2d_save(dpm2d_batch *b, const char *path) {
  if (int r = check_batch(b)) return r;
  if (!b->uploaded || !b->cells_set || !b->tissues_set)
    return fail(DPM_ESTATE, "set cells and tissues and upload before saving");
  if (b->serving) return fail(DPM_ESTATE, "slot pools are not saved");
  std::vector<float> xy(2 * (size_t)b->nverts), F(2 * (size_t)b->nverts);
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(xy.data(), b->d_pos[b->cur], sizeof(float2) * b->nverts,
                               cudaMemcpyDeviceToHost, b->stream));
  DPM_CUDA_TRY(cudaMemcpyAsync(F.data(), b->d_force, sizeof(float2) * b->nverts,
                               cudaMemcpyDeviceToHost, b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  const int N = b->ncells, T = b->ntissues;
  std::vector<float> col(N);
  CkptFile f(path, "wb");
  if (!f.open()) return fail(DPM_EINVAL, std::string("cannot write ") + (path ? path : "(null)"));
  f.put_header(2);
  f.put1(T);
  f.put1(N);
  f.put1((int64_t)b->nverts);
  f.put(b->tissue_ncells.data(), T);
  f.put(b->nv.data(), N);
  f.put(b->h_Ka.data(), N);
  f.put(b->h_Kl.data(), N);
  for (int k = 0; k < 4; ++k) {
    for (int c = 0; c < N; ++c) {
      const Cell2D &C = b->h_cells[c];
      col[c] = k == 0 ? C.Kb : k == 1 ? C.a0 : k == 2 ? C.l0 : C.r0;
    }
    f.put(col.data(), N);
  }
  for (int k = 0; k < 4; ++k)
    for (int t = 0; t < T; ++t) {
      const Tissue2D &U = b->h_tissues[t];
      if (k < 3) f.put1(k == 0 ? U.L : k == 1 ? U.Kre : U.Kat);
      else f.put1(U.pbc);
    }
  f.put(xy.data(), xy.size());
  f.put(F.data(), F.size());
  if (!f.ok() || f.close() != 0) return fail(DPM_EINVAL, std::string("write failed: ") + path);
  return DPM_OK;
}

int dpm2d_open(dpm_ctx *ctx, const char *path, dpm2d_batch **out) {
  if (!ctx || !out) return fail(DPM_EINVAL, "null argument");
  CkptFile f(path, "rb");
  if (!f.open()) return fail(DPM_EINVAL, std::string("cannot read ") + (path ? path : "(null)"));
  if (!f.get_header(2)) return fail(DPM_EINVAL, "not a 2D checkpoint");
  const int T = f.get1<int>(), N = f.get1<int>();
  const int64_t V = f.get1<int64_t>();
  if (!f.ok() || T <= 0 || N <= 0 || V <= 0 || V > (int64_t)N * kMaxNV2D)
    return fail(DPM_EINVAL, "corrupt checkpoint header");
  try {
    std::vector<int> nc(T), pbc(T);
    std::vector<unsigned> nv(N);
    std::vector<float> Ka(N), Kl(N), Kb(N), a0(N), l0(N), r0(N), L(T), Kre(T), Kat(T);
    std::vector<float> xy(2 * (size_t)V), F(2 * (size_t)V);
    f.get(nc.data(), T);
    f.get(nv.data(), N);
    for (auto *v : {&Ka, &Kl, &Kb, &a0, &l0, &r0}) f.get(v->data(), N);
    for (auto *v : {&L, &Kre, &Kat}) f.get(v->data(), T);
    f.get(pbc.data(), T);
    f.get(xy.data(), xy.size());
    f.get(F.data(), F.size());
    if (!f.ok()) return fail(DPM_EINVAL, "truncated checkpoint");
    long sum_nv = 0, sum_nc = 0;
    for (unsigned v : nv) sum_nv += v;
    for (int c : nc) sum_nc += c;
    if (sum_nv != V || sum_nc != N) return fail(DPM_EINVAL, "inconsistent checkpoint sizes");
    dpm2d_batch *b = nullptr;
    if (int r = dpm2d_create(ctx, T, nc.data(), nv.data(), &b)) return r;
    int r = dpm2d_set_cells(b, Ka.data(), Kl.data(), Kb.data(), a0.data(), l0.data(), r0.data());
    if (!r) r = dpm2d_set_tissues(b, L.data(), Kre.data(), Kat.data(), pbc.data());
    if (!r) r = dpm2d_upload(b, xy.data());
    if (!r) {
      const cudaError_t e = cudaMemcpyAsync(b->d_force, F.data(), sizeof(float2) * V,
                                            cudaMemcpyHostToDevice, b->stream);
      const cudaError_t e2 = cudaStreamSynchronize(b->stream);
      if (e != cudaSuccess || e2 != cudaSuccess) r = cuda_fail(e ? e : e2, "checkpoint forces");
    }
    if (r) {
      dpm2d_destroy(b);
      return r;
    }
    *out = b;
    return DPM_OK;
  } catch (const std::bad_alloc &) {
    return fail(DPM_ECAPACITY, "out of host memory");
  }
}

int dpm2d_last_contained(dpm2d_batch *b, unsigned char *flags) {
  if (int r = check_batch(b)) return r;
  if (!flags) return fail(DPM_EINVAL, "null output");
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(flags, b->d_flags, b->nverts, cudaMemcpyDeviceToHost,
                               b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DPM_OK;
}

int dpm2d_cell_areas(dpm2d_batch *b, float *area) {
  if (int r = check_batch(b)) return r;
  if (!area) return fail(DPM_EINVAL, "null output");
  std::vector<Geom2D> g(b->ncells);
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(g.data(), b->d_geom[b->cur], sizeof(Geom2D) * b->ncells,
                               cudaMemcpyDeviceToHost, b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (int c = 0; c < b->ncells; ++c) area[c] = g[c].area;
  return DPM_OK;
}

int dpm2d_set_packing_fraction(dpm2d_batch *b, const float *phi) {
  if (int r = check_batch(b)) return r;
  if (!phi) return fail(DPM_EINVAL, "null packing fractions");
  if (!b->uploaded || !b->cells_set || !b->tissues_set)
    return fail(DPM_ESTATE, "set cells and tissues and upload positions before rescaling");
  bool any = false;
  for (int t = 0; t < b->ntissues; ++t) {
    if (!(phi[t] >= 0.0f) || !std::isfinite(phi[t]))
      return fail(DPM_EINVAL, "packing fractions must be finite and non-negative (0: unchanged)");
    any |= phi[t] > 0.0f;
  }
  if (!any) return DPM_OK;
  cudaSetDevice(b->ctx->device);
  cudaStream_t s = b->stream;
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_phi, phi, sizeof(float) * b->ntissues,
                               cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(launch_rescale2d(b->d_cells, b->d_tissues, b->d_phi, b->d_pos[b->cur],
                                b->d_stale, b->ntissues, s));
  DPM_CUDA_TRY(launch_geom2d(b->d_cells, b->d_pos[b->cur], b->d_geom[b->cur], b->ncells,
                             b->maxnv, s));
  // the host copy of each box side follows the device's
  std::vector<Tissue2D> dev(b->ntissues);
  DPM_CUDA_TRY(cudaMemcpyAsync(dev.data(), b->d_tissues, sizeof(Tissue2D) * b->ntissues,
                               cudaMemcpyDeviceToHost, s));
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  for (int t = 0; t < b->ntissues; ++t) {
    if (!(phi[t] > 0.0f)) continue;
    if (!(dev[t].L > 0.0f) || !std::isfinite(dev[t].L))
      return fail(DPM_ENONFINITE, "rescaled box side is not finite");
    b->h_tissues[t].L = dev[t].L;
  }
  return DPM_OK;
}

int dpm2d_diagnostics(dpm2d_batch *b, double *area, double *perimeter, double *energy,
                      double *packing_fraction, double *shape_index) {
  if (int r = check_batch(b)) return r;
  if (!b->uploaded || !b->cells_set) return fail(DPM_ESTATE, "set cells and upload first");
  cudaSetDevice(b->ctx->device);
  DeviceArena A;
  DPM_CUDA_TRY(A.reserve(sizeof(Diag2D) * b->ncells));
  Diag2D *d = A.take<Diag2D>(b->ncells);
  DPM_CUDA_TRY(launch_diag2d(b->d_cells, b->d_pos[b->cur], d, b->ncells, b->stream));
  std::vector<Diag2D> h(b->ncells);
  DPM_CUDA_TRY(cudaMemcpyAsync(h.data(), d, sizeof(Diag2D) * b->ncells, cudaMemcpyDeviceToHost,
                               b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (int c = 0; c < b->ncells; ++c) {
    const Cell2D &C = b->h_cells[c];
    const double Ac = h[c].area, Pc = h[c].perim;
    if (area) area[c] = Ac;
    if (perimeter) perimeter[c] = Pc;
    if (energy) {
      const double da = Ac / C.a0 - 1.0;
      energy[c] = C.nv ? 0.5 * b->h_Ka[c] * da * da + 0.5 * b->h_Kl[c] * h[c].ul +
                             0.5 * C.Kb * h[c].ub
                       : 0.0;
    }
  }
  for (int t = 0; t < b->ntissues; ++t) {
    const Tissue2D &T = b->h_tissues[t];
    double asum = 0.0, ssum = 0.0;
    int n = 0;
    for (int c = T.cell_begin; c < T.cell_end; ++c) {
      if (!b->h_cells[c].nv) continue;
      asum += h[c].area;
      ssum += h[c].perim / std::sqrt(4.0 * M_PI * h[c].area);
      ++n;
    }
    if (packing_fraction) packing_fraction[t] = asum / ((double)T.L * (double)T.L);
    if (shape_index) shape_index[t] = n ? ssum / n : 0.0;
  }
  return DPM_OK;
}

int dpm2d_stats(dpm2d_batch *b, long *rebuilds, long *fallback_steps) {
  if (int r = check_batch(b)) return r;
  if (rebuilds) *rebuilds = b->rebuilds;
  if (fallback_steps) {
    std::vector<int> st(b->ntissues);
    cudaSetDevice(b->ctx->device);
    DPM_CUDA_TRY(cudaMemcpyAsync(st.data(), b->d_stale, sizeof(int) * b->ntissues,
                                 cudaMemcpyDeviceToHost, b->stream));
    DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
    long n = 0;
    for (int v : st) n += v ? 1 : 0;
    *fallback_steps = n;
  }
  return DPM_OK;
}

int dpm2d_rebuild_now(dpm2d_batch *b) {
  if (int r = check_batch(b)) return r;
  if (!b->uploaded || !b->tissues_set) return fail(DPM_ESTATE, "upload before rebuilding");
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(b->enqueue_rebuild(b->cur, 0, b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DPM_OK;
}

int dpm2d_cell_list(dpm2d_batch *b, unsigned *keys, unsigned *ids, int *nn, int *nbr,
                    int *maxnb, float *geom) {
  if (int r = check_batch(b)) return r;
  cudaSetDevice(b->ctx->device);
  cudaStream_t s = b->stream;
  const size_t N = b->ncells;
  if (keys)
    DPM_CUDA_TRY(cudaMemcpyAsync(keys, b->sorted_in_alt ? b->d_keys_alt : b->d_keys,
                                 4 * N, cudaMemcpyDeviceToHost, s));
  if (ids)
    DPM_CUDA_TRY(cudaMemcpyAsync(ids, b->sorted_in_alt ? b->d_vals_alt : b->d_vals, 4 * N,
                                 cudaMemcpyDeviceToHost, s));
  if (nn) DPM_CUDA_TRY(cudaMemcpyAsync(nn, b->d_nn, 4 * N, cudaMemcpyDeviceToHost, s));
  if (nbr)
    DPM_CUDA_TRY(cudaMemcpyAsync(nbr, b->d_nbr, 4 * N * kMaxNB2D, cudaMemcpyDeviceToHost, s));
  if (geom)
    DPM_CUDA_TRY(cudaMemcpyAsync(geom, b->d_geom[b->cur], sizeof(Geom2D) * N,
                                 cudaMemcpyDeviceToHost, s));
  if (maxnb) *maxnb = kMaxNB2D;
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  return DPM_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: warps per block x occupancy variant x (rebuild period, skin)
// ---------------------------------------------------------------------------

namespace {

std::string tune_cache_path() {
  if (const char *p = std::getenv("DPM_TUNE_CACHE")) return p;
  const char *home = std::getenv("HOME");
  return std::string(home ? home : ".") + "/.cache/dpm_gb300_tune2d.jsonl";
}

std::string tune_key(const dpm2d_batch *b, int sm_count) {
  // shape buckets: the choice depends on work per launch, not on exact sizes
  auto bucket = [](long v) {
    int k = 0;
    while ((1L << k) < v) ++k;
    return k;
  };
  char buf[160];
  // "k2": step-kernel variants 0..3 (register cap x dynamic schedule)
  std::snprintf(buf, sizeof(buf), "2d k3 sm%d t%d c%d v%d nv%d", sm_count, bucket(b->ntissues),
                bucket(b->ncells), bucket(b->nverts), b->maxnv);
  return buf;
}

bool tune_lookup(const std::string &key, int *warps, int *occ, int *period, float *skin) {
  FILE *f = std::fopen(tune_cache_path().c_str(), "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof(line), f)) {
    char k[200];
    int w, o, p;
    float sk;
    if (std::sscanf(line, "{\"key\": \"%199[^\"]\", \"warps\": %d, \"occ\": %d, \"period\": %d, "
                          "\"skin_rel\": %f",
                    k, &w, &o, &p, &sk) == 5 &&
        key == k) {
      *warps = w;
      *occ = o;
      *period = p;
      *skin = sk;
      found = true;  // the last entry for a key wins
    }
  }
  std::fclose(f);
  return found;
}

void tune_store(const std::string &key, int warps, int occ, int period, float skin, float ms) {
  const std::string path = tune_cache_path();
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) {
    const std::string dir = path.substr(0, slash);
    for (size_t i = 1; i <= dir.size(); ++i)
      if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
  }
  FILE *f = std::fopen(path.c_str(), "a");
  if (!f) return;
  std::fprintf(f,
               "{\"key\": \"%s\", \"warps\": %d, \"occ\": %d, \"period\": %d, \"skin_rel\": %.4f, "
               "\"ms_per_step\": %.5f}\n",
               key.c_str(), warps, occ, period, skin, ms);
  std::fclose(f);
}

} // namespace

int dpm2d_autotune(dpm2d_batch *b, float dt, int trial_blocks, int use_cache, int *warps_out,
                   int *occ_out, int *period_out, float *skin_out, float *ms_out) {
  if (int r = check_batch(b)) return r;
  if (!b->uploaded || !b->cells_set || !b->tissues_set)
    return fail(DPM_ESTATE, "set cells and tissues and upload before tuning");
  if (trial_blocks <= 0) trial_blocks = 2;
  cudaSetDevice(b->ctx->device);
  cudaStream_t s = b->stream;
  const std::string key = tune_key(b, b->ctx->sm_count);
  int w = 0, o = 0, p = 0;
  float sk = 0.0f, best_ms = -1.0f;
  auto apply = [&](int ww, int oo, int pp, float ss) -> int {
    b->warps = ww;
    b->occ = oo & 3;
    b->team = (oo & kStepVariantTeam) != 0;
    b->rebuild_period = pp;
    b->skin_rel = ss;
    b->clear_graphs();
    for (int t = 0; t < b->ntissues; ++t) {
      Tissue2D &T = b->h_tissues[t];
      double rsum = 0.0;
      for (int c = T.cell_begin; c < T.cell_end; ++c) rsum += b->h_cells[c].r0;
      T.skin = (float)(ss * 2.0 * rsum / (T.cell_end - T.cell_begin));
    }
    DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(),
                                 sizeof(Tissue2D) * b->ntissues, cudaMemcpyHostToDevice, s));
    return DPM_OK;
  };
  if (use_cache && tune_lookup(key, &w, &o, &p, &sk)) {
    if (int r = apply(w, o, p, sk)) return r;
  } else {
    // save the state: the trials advance the simulation
    const size_t pos_bytes = sizeof(float2) * b->nverts, geom_bytes = sizeof(Geom2D) * b->ncells;
    void *save = nullptr;
    DPM_CUDA_TRY(cudaMalloc(&save, pos_bytes + geom_bytes));
    const int cur0 = b->cur;
    DPM_CUDA_TRY(cudaMemcpyAsync(save, b->d_pos[cur0], pos_bytes, cudaMemcpyDeviceToDevice, s));
    DPM_CUDA_TRY(cudaMemcpyAsync((char *)save + pos_bytes, b->d_geom[cur0], geom_bytes,
                                 cudaMemcpyDeviceToDevice, s));
    auto restore = [&]() -> cudaError_t {
      b->cur = cur0;
      cudaError_t e = cudaMemcpyAsync(b->d_pos[cur0], save, pos_bytes, cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_geom[cur0], (char *)save + pos_bytes, geom_bytes,
                            cudaMemcpyDeviceToDevice, s);
      return e;
    };
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int warps_set[3] = {4, 8, 16};
    const int periods[3] = {8, 16, 32};
    const float skins[3] = {0.08f, 0.15f, 0.3f};
    // step-kernel variants: register cap x schedule, and (no attraction,
    // rings of at most 64) four warps per cell with or without the cap
    const int vars[6] = {0, 1, 2, 3, kStepVariantTeam, kStepVariantTeam | 1};
    const int nvar = (!b->att && b->maxnv <= 64) ? 6 : 4;
    int rc = DPM_OK;
    for (int wi = 0; wi < 3 && rc == DPM_OK; ++wi)
      for (int oi = 0; oi < nvar && rc == DPM_OK; ++oi)
        for (int pi = 0; pi < 3 && rc == DPM_OK; ++pi) {
          if (warps_set[wi] == 16 && b->maxnv > 128) continue;
          if ((vars[oi] & kStepVariantTeam) && warps_set[wi] != 8) continue;
          if ((rc = apply(warps_set[wi], vars[oi], periods[pi], skins[pi]))) break;
          cudaError_t e = restore();
          if (e != cudaSuccess) {
            rc = cuda_fail(e, "tuner restore");
            break;
          }
          if ((rc = b->run_block(periods[pi], dt, false))) break;  // warm: capture
          cudaEventRecord(e0, s);
          for (int k = 0; k < trial_blocks && rc == DPM_OK; ++k)
            rc = b->run_block(periods[pi], dt, false);
          cudaEventRecord(e1, s);
          e = cudaEventSynchronize(e1);
          if (e != cudaSuccess) {
            rc = cuda_fail(e, "tuner timing");
            break;
          }
          float ms = 0.0f;
          cudaEventElapsedTime(&ms, e0, e1);
          ms /= (float)(trial_blocks * periods[pi]);
          if (best_ms < 0.0f || ms < best_ms) {
            best_ms = ms;
            w = warps_set[wi];
            o = vars[oi];
            p = periods[pi];
            sk = skins[pi];
          }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t e = restore();
    cudaStreamSynchronize(s);
    cudaFree(save);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "tuner restore");
    if (int r = apply(w, o, p, sk)) return r;
    tune_store(key, w, o, p, sk, best_ms);
  }
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  if (warps_out) *warps_out = w;
  if (occ_out) *occ_out = o;
  if (period_out) *period_out = p;
  if (skin_out) *skin_out = sk;
  if (ms_out) *ms_out = best_ms;
  return DPM_OK;
}

int dpm2d_bins(dpm2d_batch *b, int *local_bits, int *nbins, float *binw, float *skin) {
  if (int r = check_batch(b)) return r;
  std::vector<Tissue2D> T(b->ntissues);
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(T.data(), b->d_tissues, sizeof(Tissue2D) * b->ntissues,
                               cudaMemcpyDeviceToHost, b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (local_bits) *local_bits = b->local_bits;
  for (int t = 0; t < b->ntissues; ++t) {
    if (nbins) nbins[t] = T[t].nbx;
    if (binw) binw[t] = T[t].binw;
    if (skin) skin[t] = T[t].skin;
  }
  return DPM_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Slot pools for the server
// ---------------------------------------------------------------------------

namespace dpm {

int pool2d_create(dpm_ctx *ctx, int nslots, int cells_per_slot, int nv_max, dpm2d_batch **out) {
  if (nslots <= 0 || cells_per_slot <= 0) return fail(DPM_EINVAL, "empty pool");
  if (nv_max < 3 || nv_max > kMaxNV2D) return fail(DPM_EINVAL, "pool nv_max must be 3..256");
  std::vector<int> nc(nslots, cells_per_slot);
  std::vector<unsigned> nv((size_t)nslots * cells_per_slot, (unsigned)nv_max);
  dpm2d_batch *b = nullptr;
  if (int r = dpm2d_create(ctx, nslots, nc.data(), nv.data(), &b)) return r;
  b->serving = true;
  b->occ = 3;  // dynamic schedule: empty and frozen slots cost one fetch each
  // every cell starts as an empty slot; vertex storage stays strided by nv_max
  for (auto &C : b->h_cells) C.nv = 0;
  for (auto &T : b->h_tissues) {
    T.cell_cap = T.cell_end;
    T.cell_end = T.cell_begin;
    T.L = 1.0f;
    T.cap = 1;
    T.steps_left = 0;
    T.run_now = 0;
  }
  // bins per axis are capped at 1024, so local bin indices fit 20 bits
  b->local_bits = 20;
  b->key_bits = 20 + ceil_log2(nslots);
  if (b->key_bits > 32) {
    dpm2d_destroy(b);
    return fail(DPM_ECAPACITY, "too many slots for 32-bit cell-list keys");
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    b->stream = ctx->stream;
    dpm2d_destroy(b);
    return cuda_fail(e, "pool stream");
  }
  b->own_stream = true;
  e = cudaMemcpyAsync(b->d_cells, b->h_cells.data(), sizeof(Cell2D) * b->ncells,
                      cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(), sizeof(Tissue2D) * b->ntissues,
                        cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    dpm2d_destroy(b);
    return cuda_fail(e, "pool upload");
  }
  b->cells_set = b->tissues_set = b->uploaded = true;
  *out = b;
  return DPM_OK;
}

size_t pool2d_bytes(const dpm2d_batch *b) { return b->arena.capacity(); }
cudaStream_t pool2d_stream(const dpm2d_batch *b) { return b->stream; }

void pool2d_set_active(dpm2d_batch *b, int nslots) {
  nslots = std::max(1, std::min(nslots, b->ntissues));
  b->run_tissues = nslots;
  b->run_cells = b->h_tissues[nslots - 1].cell_cap;
}

int pool2d_assign(dpm2d_batch *b, int slot, int ncells, const unsigned *nv, const float *Ka,
                  const float *Kl, const float *Kb, const float *a0, const float *l0,
                  const float *r0, const float *xy, float L, float Kre, float Kat, int pbc,
                  int nsteps) {
  if (slot < 0 || slot >= b->ntissues) return fail(DPM_EINVAL, "no such slot");
  Tissue2D &T = b->h_tissues[slot];
  const int cap_cells = T.cell_cap - T.cell_begin;
  const unsigned nv_max = b->nv[T.cell_begin];
  if (ncells <= 0 || ncells > cap_cells) return fail(DPM_ECAPACITY, "request exceeds slot cells");
  if (!(L > 0.0f) || nsteps <= 0) return fail(DPM_EINVAL, "bad tissue parameters");
  float l0max = 0.0f, a0max = 0.0f;
  double rsum = 0.0;
  for (int i = 0; i < ncells; ++i) {
    if (nv[i] < 3 || nv[i] > nv_max) return fail(DPM_ECAPACITY, "request exceeds slot vertices");
    if (!(a0[i] > 0.0f) || !(l0[i] > 0.0f) || !(r0[i] > 0.0f))
      return fail(DPM_EINVAL, "a0, l0 and r0 must be positive");
  }
  // cell constants of the slot (active cells, then empty ones)
  for (int i = 0; i < cap_cells; ++i) {
    Cell2D &C = b->h_cells[T.cell_begin + i];
    if (i < ncells) {
      C.nv = nv[i];
      C.a0 = a0[i];
      C.l0 = l0[i];
      C.kA = Ka[i] / std::sqrt(a0[i]);
      C.kL = Kl[i] * std::sqrt(a0[i] / l0[i]);
      C.Kb = Kb[i];
      C.r0 = r0[i];
      C.inv_l0 = 1.0f / l0[i];
      C.inv_2r0 = 1.0f / (2.0f * r0[i]);
      b->h_Ka[T.cell_begin + i] = Ka[i];
      b->h_Kl[T.cell_begin + i] = Kl[i];
      l0max = std::max(l0max, l0[i]);
      a0max = std::max(a0max, a0[i]);
      rsum += r0[i];
    } else {
      C.nv = 0;
    }
  }
  T.L = L;
  T.Kre = Kre;
  T.Kat = Kat;
  T.pbc = pbc ? 1 : 0;
  T.l0max = l0max;
  if (Kat != 0.0f && !b->att) {
    // a slot pool keeps the attraction variant once a run has needed it
    b->att = true;
    b->clear_graphs();
  }
  T.skin = (float)(b->skin_rel * 2.0 * rsum / ncells);
  const double rad = std::sqrt(a0max / M_PI);
  long cap = (long)std::floor(L / std::max(rad, 1e-6));
  T.cap = (int)std::max(1L, std::min(cap, (long)kMaxBinsAxis));
  T.cell_end = T.cell_begin + ncells;
  T.steps_left = nsteps;
  T.run_now = 0;
  // positions into the slot's strided storage
  std::vector<float2> stage((size_t)ncells * nv_max, make_float2(0.0f, 0.0f));
  size_t off = 0;
  for (int i = 0; i < ncells; ++i) {
    for (unsigned v = 0; v < nv[i]; ++v)
      stage[(size_t)i * nv_max + v] = make_float2(xy[2 * (off + v)], xy[2 * (off + v) + 1]);
    off += nv[i];
  }
  cudaStream_t s = b->stream;
  const uint32_t v0 = b->voff[T.cell_begin];
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_cells + T.cell_begin, b->h_cells.data() + T.cell_begin,
                               sizeof(Cell2D) * cap_cells, cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues + slot, &T, sizeof(Tissue2D), cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_pos[b->cur] + v0, stage.data(), sizeof(float2) * stage.size(),
                               cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemsetAsync(b->d_force + v0, 0, sizeof(float2) * stage.size(), s));
  DPM_CUDA_TRY(launch_geom2d(b->d_cells + T.cell_begin, b->d_pos[b->cur],
                             b->d_geom[b->cur] + T.cell_begin, cap_cells, b->maxnv, s));
  // the copies above read host memory that goes out of scope
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  return DPM_OK;
}

int pool2d_run(dpm2d_batch *b, int nsteps, float dt) {
  const int R = b->rebuild_period;
  if (nsteps % R) return fail(DPM_EINVAL, "pool chunks must be whole rebuild periods");
  for (int i = 0; i < nsteps / R; ++i)
    if (int r = b->run_block(R, dt, false)) return r;
  return DPM_OK;
}

int pool2d_sync(dpm2d_batch *b) {
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DPM_OK;
}

int pool2d_fetch(dpm2d_batch *b, int slot, int ncells, const unsigned *nv, float *xy, float *F) {
  const Tissue2D &T = b->h_tissues[slot];
  const unsigned nv_max = b->nv[T.cell_begin];
  const uint32_t v0 = b->voff[T.cell_begin];
  std::vector<float2> px((size_t)ncells * nv_max), pf((size_t)ncells * nv_max);
  DPM_CUDA_TRY(cudaMemcpyAsync(px.data(), b->d_pos[b->cur] + v0, sizeof(float2) * px.size(),
                               cudaMemcpyDeviceToHost, b->stream));
  DPM_CUDA_TRY(cudaMemcpyAsync(pf.data(), b->d_force + v0, sizeof(float2) * pf.size(),
                               cudaMemcpyDeviceToHost, b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  size_t off = 0;
  for (int i = 0; i < ncells; ++i) {
    for (unsigned v = 0; v < nv[i]; ++v) {
      const float2 p = px[(size_t)i * nv_max + v], f = pf[(size_t)i * nv_max + v];
      xy[2 * (off + v)] = p.x;
      xy[2 * (off + v) + 1] = p.y;
      if (F) {
        F[2 * (off + v)] = f.x;
        F[2 * (off + v) + 1] = f.y;
      }
    }
    off += nv[i];
  }
  return DPM_OK;
}

int pool2d_release(dpm2d_batch *b, int slot) {
  Tissue2D &T = b->h_tissues[slot];
  for (int c = T.cell_begin; c < T.cell_cap; ++c) b->h_cells[c].nv = 0;
  T.cell_end = T.cell_begin;
  T.steps_left = 0;
  T.run_now = 0;
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_cells + T.cell_begin, b->h_cells.data() + T.cell_begin,
                               sizeof(Cell2D) * (T.cell_cap - T.cell_begin),
                               cudaMemcpyHostToDevice, b->stream));
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues + slot, &T, sizeof(Tissue2D), cudaMemcpyHostToDevice,
                               b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DPM_OK;
}

} // namespace dpm
