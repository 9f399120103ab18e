// Runtime of the 3D path: batch objects, mesh tables, captured step graphs
// and the dpm3d_* entry points of include/dpm_gb300.h.
//
// The mesh topology is shared by every cell (the reference uploads cell 0's
// face table for all cells, src/Tissue3D.cpp:144-146).  At creation the
// host derives from it the vertex -> (face, corner) incidence lists sorted
// by face id, which let each vertex gather its face terms in the order the
// reference's atomics deliver them, and the face adjacency used by the
// bending extension.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "ckpt_io.hpp"
#include "dpm3d_kernels.cuh"
#include "dpm_common.cuh"
#include "dpm_runtime.hpp"
#include "radix_sort.cuh"

using namespace dpm;

namespace {
int ceil_log2l(long v) {
  int b = 0;
  while ((1L << b) < v) ++b;
  return b;
}

// Groups the mesh vertices into patches of at most kPatchSize3D vertices
// that lie close together on the surface: seeds by farthest-point sampling
// in edge hops, then every vertex, nearest first, joins the nearest seed
// with room.  The step kernel bounds each patch by a sphere at the current
// positions, so any grouping is correct; compact patches make the bounds
// tight.  Writes offsets off[0..np] and the vertex ids grouped by patch.
void build_patches(int nv, int nf, const unsigned *faces, std::vector<int> &off,
                   std::vector<uint16_t> &vert) {
  std::vector<std::vector<int>> nb(nv);
  for (int f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) {
      const int a = (int)faces[3 * f + k], c = (int)faces[3 * f + (k + 1) % 3];
      nb[a].push_back(c);
      nb[c].push_back(a);
    }
  const int unreached = 1 << 29;
  auto hops = [&](int src) {
    std::vector<int> d(nv, unreached);
    std::vector<int> queue{src};
    d[src] = 0;
    for (size_t q = 0; q < queue.size(); ++q)
      for (int w : nb[queue[q]])
        if (d[w] == unreached) {
          d[w] = d[queue[q]] + 1;
          queue.push_back(w);
        }
    return d;
  };
  const int fill = kPatchSize3D - 2; // room left for the greedy assignment
  const int np = std::min(kMaxPatches3D, (nv + fill - 1) / fill);
  std::vector<std::vector<int>> dist{hops(0)};
  std::vector<int> dmin = dist[0];
  while ((int)dist.size() < np) {
    const int s = (int)(std::max_element(dmin.begin(), dmin.end()) - dmin.begin());
    dist.push_back(hops(s));
    for (int v = 0; v < nv; ++v) dmin[v] = std::min(dmin[v], dist.back()[v]);
  }
  std::vector<int> order(nv), count(np, 0), patch(nv, 0), seeds(np);
  for (int v = 0; v < nv; ++v) order[v] = v;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return dmin[x] < dmin[y]; });
  for (int v : order) {
    for (int k = 0; k < np; ++k) seeds[k] = k;
    std::stable_sort(seeds.begin(), seeds.end(),
                     [&](int x, int y) { return dist[x][v] < dist[y][v]; });
    for (int k : seeds)
      if (count[k] < kPatchSize3D) {
        patch[v] = k;
        ++count[k];
        break;
      }
  }
  off.assign(1, 0);
  vert.clear();
  for (int k = 0; k < np; ++k) {
    if (count[k] == 0) continue;
    for (int v = 0; v < nv; ++v)
      if (patch[v] == k) vert.push_back((uint16_t)v);
    off.push_back((int)vert.size());
  }
}
} // namespace

struct dpm3d_batch {
  dpm_ctx *ctx = nullptr;
  cudaStream_t stream = nullptr; // the context's, or the pool's own
  bool own_stream = false;
  int ntissues = 0, ncells = 0, nv = 0, nf = 0;
  long nverts = 0;
  std::vector<Cell3D> h_cells;
  std::vector<Tissue3D> h_tissues;
  std::vector<unsigned> h_faces;  // the mesh as given
  bool cells_set = false, tissues_set = false, uploaded = false, bend = false;
  bool serving = false; // slot pool of a server: per-tissue step budgets
  DeviceArena arena;
  Mesh3D mesh{};
  Cell3D *d_cells = nullptr;
  Tissue3D *d_tissues = nullptr;
  float *d_pos[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  float *d_f[3] = {nullptr, nullptr, nullptr};
  unsigned char *d_wn = nullptr;
  Geom3D *d_geom[2] = {nullptr, nullptr};
  Geom3D *d_geom0 = nullptr;
  int *d_nn = nullptr, *d_nbr = nullptr, *d_stale = nullptr, *d_err = nullptr;
  uint32_t *d_keys = nullptr, *d_vals = nullptr, *d_keys_alt = nullptr, *d_vals_alt = nullptr;
  uint32_t *d_scratch = nullptr;
  int cur = 0;
  int local_bits = 1, key_bits = 1;
  // rebuild every 16 steps with a skin of 0.2 diameters: 1.5% faster than
  // (8, 0.1) on a 256-cell monolayer (the list only prunes: the same bits)
  int rebuild_period = 16;
  float skin_rel = 0.2f;
  int threads = 0;  // threads per cell of the step (0: step3d_threads's choice)
  // slot pools: launches cover the tissues [0, run_tissues) and their cells
  // [0, run_cells) only (0: all)
  int run_tissues = 0, run_cells = 0;
  int nc() const { return run_cells ? run_cells : ncells; }
  int nt() const { return run_tissues ? run_tissues : ntissues; }
  std::map<std::tuple<int, int, uint32_t, int, int>, cudaGraphExec_t> graphs;

  ~dpm3d_batch() {
    clear_graphs();
    if (own_stream && stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
  }

  // skin = skin_rel * mean cell diameter of each tissue; the attraction's
  // pair range, 2 * largest l0 (at least 1e-12) when Kat != 0
  void update_skin() {
    for (int t = 0; t < ntissues; ++t) {
      Tissue3D &T = h_tissues[t];
      double vs = 0.0;
      float l0max = 1e-12f;
      for (int c = T.cell_begin; c < T.cell_end; ++c) {
        vs += std::cbrt(h_cells[c].v0);
        l0max = std::max(l0max, h_cells[c].l0);
      }
      T.skin = (float)(skin_rel * 2.0 * std::cbrt(3.0 / (4.0 * M_PI)) * vs /
                       (T.cell_end - T.cell_begin));
      T.arange = T.Kat != 0.0f ? 2.0f * l0max * (1.0f + 1e-4f) : 0.0f;
    }
  }

  void clear_graphs() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
  }

  cudaError_t enqueue_rebuild(int g, int block_len, cudaStream_t s) {
    Rebuild3DArgs a{};
    a.cells = d_cells;
    a.tissues = d_tissues;
    a.geom = d_geom[g];
    a.geom0 = d_geom0;
    a.keys = d_keys;
    a.vals = d_vals;
    a.nn = d_nn;
    a.nbr = d_nbr;
    a.stale = d_stale;
    a.ncells = nc();
    a.ntissues = nt();
    a.block_len = block_len;
    cudaError_t e = launch_binprep3d(a, local_bits, s);
    if (e != cudaSuccess) return e;
    bool alt = false;
    e = radix_sort_pairs(d_keys, d_vals, d_keys_alt, d_vals_alt, nc(), key_bits, d_scratch, s,
                         &alt);
    if (e != cudaSuccess) return e;
    a.sorted_keys = alt ? d_keys_alt : d_keys;
    a.sorted_vals = alt ? d_vals_alt : d_vals;
    return launch_neighbors3d(a, local_bits, s);
  }

  Step3DArgs step_args(int from, float dt, bool last, int index) const {
    Step3DArgs a{};
    a.mesh = mesh;
    a.cells = d_cells;
    a.tissues = d_tissues;
    a.xin = d_pos[from][0];
    a.yin = d_pos[from][1];
    a.zin = d_pos[from][2];
    a.xout = d_pos[1 - from][0];
    a.yout = d_pos[1 - from][1];
    a.zout = d_pos[1 - from][2];
    const bool out = serving || last;
    a.fx = out ? d_f[0] : nullptr;
    a.fy = out ? d_f[1] : nullptr;
    a.fz = out ? d_f[2] : nullptr;
    a.wn_out = out ? d_wn : nullptr;
    a.all_forces = serving ? 0 : 1;
    a.step_index = index;
    a.geom_in = d_geom[from];
    a.geom_out = d_geom[1 - from];
    a.geom0 = d_geom0;
    a.nn = d_nn;
    a.nbr = d_nbr;
    a.stale = d_stale;
    a.err = d_err;
    a.ncells = nc();
    a.dt = dt;
    a.bend = bend ? 1 : 0;
    return a;
  }

  cudaError_t enqueue_block(int len, int from, float dt, bool last, cudaStream_t s) {
    cudaError_t e = enqueue_rebuild(from, len, s);
    if (e != cudaSuccess) return e;
    const int nt =
        threads ? threads : step3d_threads(nv, nf, mesh.ne, bend, nc(), ctx->sm_count);
    int f = from;
    for (int i = 0; i < len; ++i) {
      e = launch_step3d(step_args(f, dt, last && i == len - 1, i), nt, s);
      if (e != cudaSuccess) return e;
      f = 1 - f;
    }
    return cudaSuccess;
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
        return cuda_fail(e, "enqueue_block (3D)");
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
    return DPM_OK;
  }
};

namespace {
int check3(dpm3d_batch *b) {
  if (!b) return fail(DPM_EINVAL, "null batch");
  return DPM_OK;
}
} // namespace

extern "C" {

int dpm3d_create(dpm_ctx *ctx, int ntissues, const int *ncells, int nv, int nf,
                 const unsigned *faces, dpm3d_batch **out) {
  if (!ctx || !ncells || !faces || !out) return fail(DPM_EINVAL, "null argument");
  *out = nullptr;
  if (ntissues <= 0) return fail(DPM_EINVAL, "ntissues must be positive");
  if (ntissues > 4096) return fail(DPM_ECAPACITY, "at most 4096 tissues per batch");
  if (nv < 4 || nf < 4) return fail(DPM_EINVAL, "a mesh needs at least 4 vertices and faces");
  if (nv > kMaxNV3D)
    return fail(DPM_ECAPACITY, "at most 642 vertices per 3D cell (icosphere level 3)");
  try {
    auto b = std::make_unique<dpm3d_batch>();
    b->ctx = ctx;
    b->stream = ctx->stream;
    b->ntissues = ntissues;
    b->nv = nv;
    b->nf = nf;
    long total = 0;
    for (int t = 0; t < ntissues; ++t) {
      if (ncells[t] <= 0) return fail(DPM_EINVAL, "every tissue needs at least one cell");
      total += ncells[t];
    }
    if (total * nv > (1L << 31) - 1) return fail(DPM_ECAPACITY, "too many vertices");
    b->ncells = (int)total;
    b->nverts = total * nv;
    b->h_faces.assign(faces, faces + 3 * (size_t)nf);
    // mesh tables
    std::vector<uint16_t> f16(3 * (size_t)nf);
    std::vector<std::vector<std::pair<int, int>>> inc(nv);
    for (int f = 0; f < nf; ++f)
      for (int k = 0; k < 3; ++k) {
        const unsigned v = faces[3 * f + k];
        if (v >= (unsigned)nv) return fail(DPM_EINVAL, "face index out of range");
        f16[3 * f + k] = (uint16_t)v;
        inc[v].push_back({f, k});
      }
    std::vector<int> off(nv + 1, 0);
    std::vector<uint16_t> incf;
    std::vector<uint8_t> incc;
    for (int v = 0; v < nv; ++v) {
      std::sort(inc[v].begin(), inc[v].end());
      off[v + 1] = off[v] + (int)inc[v].size();
      for (auto &p : inc[v]) {
        incf.push_back((uint16_t)p.first);
        incc.push_back((uint8_t)p.second);
      }
    }
    std::vector<int> poff;
    std::vector<uint16_t> pvert;
    build_patches(nv, nf, faces, poff, pvert);
    std::vector<int16_t> adj(3 * (size_t)nf, -1);
    // edges: endpoints (lower id first) and the edge of each face corner
    std::vector<uint16_t> eva, fedge(3 * (size_t)nf);
    {
      std::map<std::pair<unsigned, unsigned>, std::pair<int, int>> edges;
      std::map<std::pair<unsigned, unsigned>, int> edge_id;
      for (int f = 0; f < nf; ++f)
        for (int e = 0; e < 3; ++e) {
          const unsigned a = faces[3 * f + e], c = faces[3 * f + (e + 1) % 3];
          auto key = std::make_pair(std::min(a, c), std::max(a, c));
          auto id = edge_id.find(key);
          if (id == edge_id.end()) {
            id = edge_id.emplace(key, (int)eva.size() / 2).first;
            eva.push_back((uint16_t)key.first);
            eva.push_back((uint16_t)key.second);
          }
          fedge[3 * f + e] = (uint16_t)(id->second | (a > c ? 0x8000 : 0));
          auto it = edges.find(key);
          if (it == edges.end()) {
            edges.emplace(key, std::make_pair(f, e));
          } else {
            adj[3 * f + e] = (int16_t)it->second.first;
            adj[3 * it->second.first + it->second.second] = (int16_t)f;
          }
        }
    }
    const int ne = (int)eva.size() / 2;
    b->h_cells.resize(total);
    b->h_tissues.resize(ntissues);
    int cb = 0;
    for (int t = 0; t < ntissues; ++t) {
      Tissue3D &T = b->h_tissues[t];
      std::memset(&T, 0, sizeof(T));
      T.cell_begin = cb;
      T.cell_end = cb + ncells[t];
      T.cap = 1;
      T.nb = 1;
      T.cell_cap = T.cell_end;
      T.steps_left = kStepsUnlimited;
      T.run_now = kStepsUnlimited;
      for (int c = cb; c < cb + ncells[t]; ++c) {
        std::memset(&b->h_cells[c], 0, sizeof(Cell3D));
        b->h_cells[c].tissue = (uint32_t)t;
        b->h_cells[c].active = 1;
      }
      cb += ncells[t];
    }
    const long V = b->nverts, N = b->ncells;
    DeviceArena &A = b->arena;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    e = A.reserve(sizeof(uint16_t) * 3 * nf + sizeof(int) * (nv + 1) + 3 * nf * 3 +
                  sizeof(int16_t) * 3 * nf + sizeof(Cell3D) * N + sizeof(Tissue3D) * ntissues +
                  9 * sizeof(float) * V + V + 3 * sizeof(Geom3D) * N +
                  sizeof(int) * (N + N * kMaxNB3D + ntissues + 1) + 4 * sizeof(uint32_t) * N +
                  radix_sort_scratch_bytes((int)N) + sizeof(int) * (kMaxPatches3D + 1) +
                  sizeof(uint16_t) * (nv + eva.size() + fedge.size()) + 64 * 256);
    if (e != cudaSuccess) return cuda_fail(e, "device allocation");
    uint16_t *d_faces = A.take<uint16_t>(3 * nf);
    int *d_off = A.take<int>(nv + 1);
    uint16_t *d_incf = A.take<uint16_t>(3 * nf);
    uint8_t *d_incc = A.take<uint8_t>(3 * nf);
    int16_t *d_adj = A.take<int16_t>(3 * nf);
    int *d_poff = A.take<int>(poff.size());
    uint16_t *d_pvert = A.take<uint16_t>(nv);
    uint16_t *d_eva = A.take<uint16_t>(eva.size());
    uint16_t *d_fedge = A.take<uint16_t>(fedge.size());
    b->d_cells = A.take<Cell3D>(N);
    b->d_tissues = A.take<Tissue3D>(ntissues);
    for (int p = 0; p < 2; ++p)
      for (int k = 0; k < 3; ++k) b->d_pos[p][k] = A.take<float>(V);
    for (int k = 0; k < 3; ++k) b->d_f[k] = A.take<float>(V);
    b->d_wn = A.take<unsigned char>(V);
    b->d_geom[0] = A.take<Geom3D>(N);
    b->d_geom[1] = A.take<Geom3D>(N);
    b->d_geom0 = A.take<Geom3D>(N);
    b->d_nn = A.take<int>(N);
    b->d_nbr = A.take<int>(N * kMaxNB3D);
    b->d_stale = A.take<int>(ntissues);
    b->d_err = A.take<int>(1);
    b->d_keys = A.take<uint32_t>(N);
    b->d_vals = A.take<uint32_t>(N);
    b->d_keys_alt = A.take<uint32_t>(N);
    b->d_vals_alt = A.take<uint32_t>(N);
    b->d_scratch = A.take<uint32_t>(radix_sort_scratch_bytes((int)N) / 4 + 1);
    if (!A.ok()) return fail(DPM_ECAPACITY, "device arena exhausted");
    cudaStream_t s = ctx->stream;
    e = cudaMemsetAsync(A.base(), 0, A.used(), s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_faces, f16.data(), 2 * f16.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_off, off.data(), 4 * off.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_incf, incf.data(), 2 * incf.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_incc, incc.data(), incc.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_adj, adj.data(), 2 * adj.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_poff, poff.data(), 4 * poff.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_pvert, pvert.data(), 2 * pvert.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_eva, eva.data(), 2 * eva.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_fedge, fedge.data(), 2 * fedge.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "mesh upload");
    b->mesh = Mesh3D{nv, nf, d_faces, d_off, d_incf, d_incc, d_adj,
                     (int)poff.size() - 1, d_poff, d_pvert, ne, d_eva, d_fedge};
    e = prepare_step3d(nv, nf, ne, true);
    if (e != cudaSuccess) return cuda_fail(e, "shared-memory opt-in");
    *out = b.release();
    ctx_retain(ctx);
    return DPM_OK;
  } catch (const std::bad_alloc &) {
    return fail(DPM_ECAPACITY, "out of host memory");
  }
}

int dpm3d_destroy(dpm3d_batch *b) {
  if (!b) return DPM_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->stream);
  dpm_ctx *c = b->ctx;
  delete b;
  ctx_release(c);
  return DPM_OK;
}

int dpm3d_sizes(dpm3d_batch *b, int *ncells, long *nvertices) {
  if (int r = check3(b)) return r;
  if (ncells) *ncells = b->ncells;
  if (nvertices) *nvertices = b->nverts;
  return DPM_OK;
}

int dpm3d_set_cells(dpm3d_batch *b, const float *Kv, const float *Ka, const float *Ks,
                    const float *v0, const float *a0, const float *l0, const float *Kb,
                    const float *adh) {
  if (int r = check3(b)) return r;
  if (!Kv || !Ka || !Ks || !v0 || !a0 || !l0) return fail(DPM_EINVAL, "null parameter array");
  bool bend = false;
  for (int c = 0; c < b->ncells; ++c) {
    if (!(l0[c] > 0.0f) || !(a0[c] >= 0.0f) || !(v0[c] > 0.0f))
      return fail(DPM_EINVAL, "v0 and l0 must be positive");
    Cell3D &C = b->h_cells[c];
    C.Kv = Kv[c];
    C.Ka = Ka[c];
    C.Ks = Ks[c];
    C.v0 = v0[c];
    C.a0 = a0[c];
    C.l0 = l0[c];
    C.Kb = Kb ? Kb[c] : 0.0f;
    C.adh = adh ? adh[c] : l0[c] * 2.0f;
    // Cell3D_Kernel.cl:167, in the reference's order of operations
    C.sa_scale = Ka[c] * std::sqrt(a0[c]) / l0[c] * 0.3f;
    bend |= C.Kb != 0.0f;
  }
  b->update_skin();
  if (bend != b->bend) b->clear_graphs();
  b->bend = bend;
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_cells, b->h_cells.data(), sizeof(Cell3D) * b->ncells,
                               cudaMemcpyHostToDevice, b->stream));
  if (b->tissues_set)
    DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(),
                                 sizeof(Tissue3D) * b->ntissues, cudaMemcpyHostToDevice,
                                 b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->cells_set = true;
  return DPM_OK;
}

int dpm3d_set_tissues(dpm3d_batch *b, const float *L, const float *Kre, const int *pbc) {
  if (int r = check3(b)) return r;
  if (!L || !Kre || !pbc) return fail(DPM_EINVAL, "null parameter array");
  int max_local = 1;
  for (int t = 0; t < b->ntissues; ++t) {
    if (!(L[t] > 0.0f) || !std::isfinite(L[t])) return fail(DPM_EINVAL, "L must be positive");
    Tissue3D &T = b->h_tissues[t];
    T.L = L[t];
    T.Kre = Kre[t];
    T.pbc = pbc[t] ? 1 : 0;
    float v0max = 0.0f;
    for (int c = T.cell_begin; c < T.cell_end; ++c) v0max = std::max(v0max, b->h_cells[c].v0);
    const double rad = v0max > 0.0f ? std::cbrt(3.0 * v0max / (4.0 * M_PI)) : 0.5;
    long cap = (long)std::floor(L[t] / std::max(rad, 1e-6));
    cap = std::max(1L, std::min(cap, 64L));
    T.cap = (int)cap;
    max_local = std::max(max_local, ceil_log2l(cap * cap * cap));
  }
  b->local_bits = max_local;
  b->key_bits = b->local_bits + ceil_log2l(b->ntissues);
  if (b->key_bits > 32) return fail(DPM_ECAPACITY, "cell-list keys exceed 32 bits");
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(), sizeof(Tissue3D) * b->ntissues,
                               cudaMemcpyHostToDevice, b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->tissues_set = true;
  b->clear_graphs();
  return DPM_OK;
}

int dpm3d_set_attraction(dpm3d_batch *b, const float *Kat) {
  if (int r = check3(b)) return r;
  if (!Kat) return fail(DPM_EINVAL, "null parameter array");
  if (!b->cells_set || !b->tissues_set)
    return fail(DPM_ESTATE, "set cells and tissues before the attraction");
  for (int t = 0; t < b->ntissues; ++t)
    if (!std::isfinite(Kat[t])) return fail(DPM_EINVAL, "Kat must be finite");
  for (int t = 0; t < b->ntissues; ++t) b->h_tissues[t].Kat = Kat[t];
  b->update_skin();
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(), sizeof(Tissue3D) * b->ntissues,
                               cudaMemcpyHostToDevice, b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->clear_graphs();
  return DPM_OK;
}

int dpm3d_upload(dpm3d_batch *b, const float *xyz) {
  if (int r = check3(b)) return r;
  if (!xyz) return fail(DPM_EINVAL, "null positions");
  cudaSetDevice(b->ctx->device);
  cudaStream_t s = b->stream;
  // de-interleave on the host into the structure-of-arrays layout
  const long V = b->nverts;
  std::vector<float> soa(3 * (size_t)V);
  for (long i = 0; i < V; ++i) {
    soa[i] = xyz[3 * i];
    soa[V + i] = xyz[3 * i + 1];
    soa[2 * V + i] = xyz[3 * i + 2];
  }
  b->cur = 0;
  for (int k = 0; k < 3; ++k)
    DPM_CUDA_TRY(cudaMemcpyAsync(b->d_pos[0][k], soa.data() + k * V, sizeof(float) * V,
                                 cudaMemcpyHostToDevice, s));
  for (int k = 0; k < 3; ++k) DPM_CUDA_TRY(cudaMemsetAsync(b->d_f[k], 0, sizeof(float) * V, s));
  DPM_CUDA_TRY(cudaMemsetAsync(b->d_wn, 0, V, s));
  DPM_CUDA_TRY(cudaMemsetAsync(b->d_err, 0, sizeof(int), s));
  DPM_CUDA_TRY(launch_geom3d(b->d_pos[0][0], b->d_pos[0][1], b->d_pos[0][2], b->mesh,
                             b->d_cells, b->d_geom[0], b->ncells, s));
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  b->uploaded = true;
  return DPM_OK;
}

int dpm3d_step(dpm3d_batch *b, int nsteps, float dt) {
  if (int r = check3(b)) return r;
  if (nsteps < 0) return fail(DPM_EINVAL, "nsteps must be non-negative");
  if (!b->uploaded || !b->cells_set || !b->tissues_set)
    return fail(DPM_ESTATE, "set cells and tissues and upload positions before stepping");
  if (!std::isfinite(dt)) return fail(DPM_EINVAL, "dt must be finite");
  if (nsteps == 0) return DPM_OK;
  cudaSetDevice(b->ctx->device);
  const int R = b->rebuild_period;
  const int full = nsteps / R, rem = nsteps % R;
  for (int i = 0; i < full; ++i)
    if (int r = b->run_block(R, dt, rem == 0 && i == full - 1)) return r;
  if (rem)
    if (int r = b->run_block(rem, dt, true)) return r;
  return DPM_OK;
}

int dpm3d_download(dpm3d_batch *b, float *xyz, float *F) {
  if (int r = check3(b)) return r;
  if (!b->uploaded) return fail(DPM_ESTATE, "nothing uploaded");
  cudaSetDevice(b->ctx->device);
  cudaStream_t s = b->stream;
  const long V = b->nverts;
  std::vector<float> soa(3 * (size_t)V);
  int err = 0;
  if (xyz)
    for (int k = 0; k < 3; ++k)
      DPM_CUDA_TRY(cudaMemcpyAsync(soa.data() + k * V, b->d_pos[b->cur][k], sizeof(float) * V,
                                   cudaMemcpyDeviceToHost, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  if (xyz)
    for (long i = 0; i < V; ++i) {
      xyz[3 * i] = soa[i];
      xyz[3 * i + 1] = soa[V + i];
      xyz[3 * i + 2] = soa[2 * V + i];
    }
  if (F) {
    for (int k = 0; k < 3; ++k)
      DPM_CUDA_TRY(cudaMemcpyAsync(soa.data() + k * V, b->d_f[k], sizeof(float) * V,
                                   cudaMemcpyDeviceToHost, s));
    DPM_CUDA_TRY(cudaStreamSynchronize(s));
    for (long i = 0; i < V; ++i) {
      F[3 * i] = soa[i];
      F[3 * i + 1] = soa[V + i];
      F[3 * i + 2] = soa[2 * V + i];
    }
  }
  if (err & 1) return fail(DPM_ENONFINITE, "non-finite vertex positions");
  return DPM_OK;
}

int dpm3d_device_state(dpm3d_batch *b, void **x, void **y, void **z, void **fx, void **fy,
                       void **fz) {
  if (int r = check3(b)) return r;
  if (x) *x = b->d_pos[b->cur][0];
  if (y) *y = b->d_pos[b->cur][1];
  if (z) *z = b->d_pos[b->cur][2];
  if (fx) *fx = b->d_f[0];
  if (fy) *fy = b->d_f[1];
  if (fz) *fz = b->d_f[2];
  return DPM_OK;
}

int dpm3d_save(dpm3d_batch *b, const char *path) {
  if (int r = check3(b)) return r;
  if (!b->uploaded || !b->cells_set || !b->tissues_set)
    return fail(DPM_ESTATE, "set cells and tissues and upload before saving");
  if (b->serving) return fail(DPM_ESTATE, "slot pools are not saved");
  const size_t V = (size_t)b->nverts;
  std::vector<float> xyz(3 * V), F(3 * V);
  if (int r = dpm3d_download(b, xyz.data(), F.data()); r && r != DPM_ENONFINITE) return r;
  const int N = b->ncells, T = b->ntissues;
  std::vector<float> col(N);
  CkptFile f(path, "wb");
  if (!f.open()) return fail(DPM_EINVAL, std::string("cannot write ") + (path ? path : "(null)"));
  f.put_header(3);
  f.put1(T);
  f.put1(N);
  f.put1(b->nv);
  f.put1(b->nf);
  f.put(b->h_faces.data(), b->h_faces.size());
  for (int t = 0; t < T; ++t) f.put1(b->h_tissues[t].cell_end - b->h_tissues[t].cell_begin);
  for (int k = 0; k < 8; ++k) {
    for (int c = 0; c < N; ++c) {
      const Cell3D &C = b->h_cells[c];
      const float v[8] = {C.Kv, C.Ka, C.Ks, C.v0, C.a0, C.l0, C.Kb, C.adh};
      col[c] = v[k];
    }
    f.put(col.data(), N);
  }
  for (int t = 0; t < T; ++t) f.put1(b->h_tissues[t].L);
  for (int t = 0; t < T; ++t) f.put1(b->h_tissues[t].Kre);
  for (int t = 0; t < T; ++t) f.put1(b->h_tissues[t].pbc);
  f.put(xyz.data(), xyz.size());
  f.put(F.data(), F.size());
  // trailing section: the attraction strength per tissue
  for (int t = 0; t < T; ++t) f.put1(b->h_tissues[t].Kat);
  if (!f.ok() || f.close() != 0) return fail(DPM_EINVAL, std::string("write failed: ") + path);
  return DPM_OK;
}

int dpm3d_open(dpm_ctx *ctx, const char *path, dpm3d_batch **out) {
  if (!ctx || !out) return fail(DPM_EINVAL, "null argument");
  CkptFile f(path, "rb");
  if (!f.open()) return fail(DPM_EINVAL, std::string("cannot read ") + (path ? path : "(null)"));
  if (!f.get_header(3)) return fail(DPM_EINVAL, "not a 3D checkpoint");
  const int T = f.get1<int>(), N = f.get1<int>(), nv = f.get1<int>(), nf = f.get1<int>();
  if (!f.ok() || T <= 0 || N <= 0 || nv < 4 || nv > kMaxNV3D || nf < 4 || nf > 4 * kMaxNV3D)
    return fail(DPM_EINVAL, "corrupt checkpoint header");
  try {
    std::vector<unsigned> faces(3 * (size_t)nf);
    std::vector<int> nc(T), pbc(T);
    std::vector<float> k[8], L(T), Kre(T);
    f.get(faces.data(), faces.size());
    f.get(nc.data(), T);
    for (auto &v : k) {
      v.resize(N);
      f.get(v.data(), N);
    }
    f.get(L.data(), T);
    f.get(Kre.data(), T);
    f.get(pbc.data(), T);
    const size_t V = (size_t)N * nv;
    std::vector<float> xyz(3 * V), F(3 * V);
    f.get(xyz.data(), xyz.size());
    f.get(F.data(), F.size());
    if (!f.ok()) return fail(DPM_EINVAL, "truncated checkpoint");
    std::vector<float> Kat(T, 0.0f);
    const bool att = f.try_get(Kat.data(), T);  // absent in older files
    long sum_nc = 0;
    for (int c : nc) sum_nc += c;
    if (sum_nc != N) return fail(DPM_EINVAL, "inconsistent checkpoint sizes");
    dpm3d_batch *b = nullptr;
    if (int r = dpm3d_create(ctx, T, nc.data(), nv, nf, faces.data(), &b)) return r;
    int r = dpm3d_set_cells(b, k[0].data(), k[1].data(), k[2].data(), k[3].data(), k[4].data(),
                            k[5].data(), k[6].data(), k[7].data());
    if (!r) r = dpm3d_set_tissues(b, L.data(), Kre.data(), pbc.data());
    if (!r && att) r = dpm3d_set_attraction(b, Kat.data());
    if (!r) r = dpm3d_upload(b, xyz.data());
    if (!r) {
      cudaError_t e = cudaSuccess;
      for (int d = 0; d < 3 && e == cudaSuccess; ++d) {
        std::vector<float> comp(V);
        for (size_t i = 0; i < V; ++i) comp[i] = F[3 * i + d];
        e = cudaMemcpy(b->d_f[d], comp.data(), sizeof(float) * V, cudaMemcpyHostToDevice);
      }
      if (e != cudaSuccess) r = cuda_fail(e, "checkpoint forces");
    }
    if (r) {
      dpm3d_destroy(b);
      return r;
    }
    *out = b;
    return DPM_OK;
  } catch (const std::bad_alloc &) {
    return fail(DPM_ECAPACITY, "out of host memory");
  }
}

int dpm3d_diagnostics(dpm3d_batch *b, double *volume, double *surface_area, double *energy) {
  if (int r = check3(b)) return r;
  if (!b->uploaded || !b->cells_set) return fail(DPM_ESTATE, "set cells and upload first");
  cudaSetDevice(b->ctx->device);
  DeviceArena A;
  DPM_CUDA_TRY(A.reserve(sizeof(double) * 3 * b->ncells));
  double *d = A.take<double>(3 * (size_t)b->ncells);
  DPM_CUDA_TRY(launch_diag3d(b->d_pos[b->cur][0], b->d_pos[b->cur][1], b->d_pos[b->cur][2],
                             b->mesh, b->d_cells, d, b->ncells, b->stream));
  std::vector<double> h(3 * (size_t)b->ncells);
  DPM_CUDA_TRY(cudaMemcpyAsync(h.data(), d, sizeof(double) * h.size(), cudaMemcpyDeviceToHost,
                               b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (int c = 0; c < b->ncells; ++c) {
    if (volume) volume[c] = h[3 * c];
    if (surface_area) surface_area[c] = h[3 * c + 1];
    if (energy) energy[c] = h[3 * c + 2];
  }
  return DPM_OK;
}

int dpm3d_last_winding(dpm3d_batch *b, unsigned char *counts) {
  if (int r = check3(b)) return r;
  if (!counts) return fail(DPM_EINVAL, "null output");
  cudaSetDevice(b->ctx->device);
  DPM_CUDA_TRY(cudaMemcpyAsync(counts, b->d_wn, b->nverts, cudaMemcpyDeviceToHost,
                               b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DPM_OK;
}

int dpm3d_set_block_threads(dpm3d_batch *b, int threads) {
  if (int r = check3(b)) return r;
  if (threads != 0 && threads != 128 && threads != 256 && threads != 512)
    return fail(DPM_EINVAL, "threads per cell must be 0, 128, 256 or 512");
  b->threads = threads;
  b->clear_graphs();
  return DPM_OK;
}

int dpm3d_set_tuning(dpm3d_batch *b, int rebuild_period, float skin_rel) {
  if (int r = check3(b)) return r;
  if (rebuild_period > 0) b->rebuild_period = rebuild_period;
  if (skin_rel > 0.0f) b->skin_rel = skin_rel;
  b->clear_graphs();
  if (b->cells_set) {
    b->update_skin();
    if (b->tissues_set) {
      cudaSetDevice(b->ctx->device);
      DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(),
                                   sizeof(Tissue3D) * b->ntissues, cudaMemcpyHostToDevice,
                                   b->stream));
      DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
    }
  }
  return DPM_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Slot pools for the server
// ---------------------------------------------------------------------------

namespace dpm {

int pool3d_create(dpm_ctx *ctx, int nslots, int cells_per_slot, int nv, int nf,
                  const unsigned *faces, dpm3d_batch **out) {
  if (nslots <= 0 || cells_per_slot <= 0) return fail(DPM_EINVAL, "empty pool");
  std::vector<int> nc(nslots, cells_per_slot);
  dpm3d_batch *b = nullptr;
  if (int r = dpm3d_create(ctx, nslots, nc.data(), nv, nf, faces, &b)) return r;
  b->serving = true;
  for (auto &C : b->h_cells) C.active = 0;
  for (auto &T : b->h_tissues) {
    T.cell_cap = T.cell_end;
    T.cell_end = T.cell_begin;
    T.L = 1.0f;
    T.cap = 1;
    T.steps_left = 0;
    T.run_now = 0;
  }
  // bins per axis are capped at 64, so local bin indices fit 18 bits
  b->local_bits = 18;
  b->key_bits = 18 + ceil_log2l(nslots);
  if (b->key_bits > 32) {
    dpm3d_destroy(b);
    return fail(DPM_ECAPACITY, "too many slots for 32-bit cell-list keys");
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    b->stream = ctx->stream;
    dpm3d_destroy(b);
    return cuda_fail(e, "pool stream");
  }
  b->own_stream = true;
  e = cudaMemcpyAsync(b->d_cells, b->h_cells.data(), sizeof(Cell3D) * b->ncells,
                      cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_tissues, b->h_tissues.data(), sizeof(Tissue3D) * b->ntissues,
                        cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    dpm3d_destroy(b);
    return cuda_fail(e, "pool upload");
  }
  b->cells_set = b->tissues_set = b->uploaded = true;
  *out = b;
  return DPM_OK;
}

size_t pool3d_bytes(const dpm3d_batch *b) { return b->arena.capacity(); }
cudaStream_t pool3d_stream(const dpm3d_batch *b) { return b->stream; }

void pool3d_set_active(dpm3d_batch *b, int nslots) {
  nslots = std::max(1, std::min(nslots, b->ntissues));
  b->run_tissues = nslots;
  b->run_cells = b->h_tissues[nslots - 1].cell_cap;
}

int pool3d_assign(dpm3d_batch *b, int slot, int ncells, const float *Kv, const float *Ka,
                  const float *Ks, const float *v0, const float *a0, const float *l0,
                  const float *Kb, const float *adh, const float *xyz, float L, float Kre,
                  int pbc, int nsteps) {
  if (slot < 0 || slot >= b->ntissues) return fail(DPM_EINVAL, "no such slot");
  Tissue3D &T = b->h_tissues[slot];
  const int cap_cells = T.cell_cap - T.cell_begin;
  if (ncells <= 0 || ncells > cap_cells) return fail(DPM_ECAPACITY, "request exceeds slot cells");
  if (!(L > 0.0f) || nsteps <= 0) return fail(DPM_EINVAL, "bad tissue parameters");
  bool bend = b->bend;
  double vs = 0.0;
  float v0max = 0.0f;
  for (int i = 0; i < cap_cells; ++i) {
    Cell3D &C = b->h_cells[T.cell_begin + i];
    if (i < ncells) {
      if (!(l0[i] > 0.0f) || !(v0[i] > 0.0f)) return fail(DPM_EINVAL, "v0 and l0 must be positive");
      C.Kv = Kv[i];
      C.Ka = Ka[i];
      C.Ks = Ks[i];
      C.v0 = v0[i];
      C.a0 = a0[i];
      C.l0 = l0[i];
      C.Kb = Kb ? Kb[i] : 0.0f;
      C.adh = adh ? adh[i] : l0[i] * 2.0f;
      C.sa_scale = Ka[i] * std::sqrt(a0[i]) / l0[i] * 0.3f;
      C.active = 1;
      bend |= C.Kb != 0.0f;
      vs += std::cbrt(v0[i]);
      v0max = std::max(v0max, v0[i]);
    } else {
      C.active = 0;
    }
  }
  if (bend != b->bend) {
    b->bend = bend;
    b->clear_graphs();
  }
  T.L = L;
  T.Kre = Kre;
  T.pbc = pbc ? 1 : 0;
  T.skin = (float)(b->skin_rel * 2.0 * std::cbrt(3.0 / (4.0 * M_PI)) * vs / ncells);
  const double rad = std::cbrt(3.0 * v0max / (4.0 * M_PI));
  long cap = (long)std::floor(L / std::max(rad, 1e-6));
  T.cap = (int)std::max(1L, std::min(cap, 64L));
  T.cell_end = T.cell_begin + ncells;
  T.steps_left = nsteps;
  T.run_now = 0;
  const size_t n = (size_t)ncells * b->nv, base = (size_t)T.cell_begin * b->nv;
  std::vector<float> soa(3 * n);
  for (size_t i = 0; i < n; ++i) {
    soa[i] = xyz[3 * i];
    soa[n + i] = xyz[3 * i + 1];
    soa[2 * n + i] = xyz[3 * i + 2];
  }
  cudaStream_t s = b->stream;
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_cells + T.cell_begin, b->h_cells.data() + T.cell_begin,
                               sizeof(Cell3D) * cap_cells, cudaMemcpyHostToDevice, s));
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues + slot, &T, sizeof(Tissue3D), cudaMemcpyHostToDevice, s));
  for (int k = 0; k < 3; ++k) {
    DPM_CUDA_TRY(cudaMemcpyAsync(b->d_pos[b->cur][k] + base, soa.data() + k * n,
                                 sizeof(float) * n, cudaMemcpyHostToDevice, s));
    DPM_CUDA_TRY(cudaMemsetAsync(b->d_f[k] + base, 0, sizeof(float) * n, s));
  }
  DPM_CUDA_TRY(launch_geom3d(b->d_pos[b->cur][0] + base, b->d_pos[b->cur][1] + base,
                             b->d_pos[b->cur][2] + base, b->mesh, b->d_cells + T.cell_begin,
                             b->d_geom[b->cur] + T.cell_begin, cap_cells, s));
  DPM_CUDA_TRY(cudaStreamSynchronize(s));
  return DPM_OK;
}

int pool3d_run(dpm3d_batch *b, int nsteps, float dt) {
  const int R = b->rebuild_period;
  if (nsteps % R) return fail(DPM_EINVAL, "pool chunks must be whole rebuild periods");
  for (int i = 0; i < nsteps / R; ++i)
    if (int r = b->run_block(R, dt, false)) return r;
  return DPM_OK;
}

int pool3d_sync(dpm3d_batch *b) {
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DPM_OK;
}

int pool3d_fetch(dpm3d_batch *b, int slot, int ncells, float *xyz, float *F) {
  const Tissue3D &T = b->h_tissues[slot];
  const size_t n = (size_t)ncells * b->nv, base = (size_t)T.cell_begin * b->nv;
  std::vector<float> soa(3 * n), fs(3 * n);
  for (int k = 0; k < 3; ++k) {
    DPM_CUDA_TRY(cudaMemcpyAsync(soa.data() + k * n, b->d_pos[b->cur][k] + base,
                                 sizeof(float) * n, cudaMemcpyDeviceToHost, b->stream));
    DPM_CUDA_TRY(cudaMemcpyAsync(fs.data() + k * n, b->d_f[k] + base, sizeof(float) * n,
                                 cudaMemcpyDeviceToHost, b->stream));
  }
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      xyz[3 * i + k] = soa[k * n + i];
      if (F) F[3 * i + k] = fs[k * n + i];
    }
  return DPM_OK;
}

int pool3d_release(dpm3d_batch *b, int slot) {
  Tissue3D &T = b->h_tissues[slot];
  for (int c = T.cell_begin; c < T.cell_cap; ++c) b->h_cells[c].active = 0;
  T.cell_end = T.cell_begin;
  T.steps_left = 0;
  T.run_now = 0;
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_cells + T.cell_begin, b->h_cells.data() + T.cell_begin,
                               sizeof(Cell3D) * (T.cell_cap - T.cell_begin),
                               cudaMemcpyHostToDevice, b->stream));
  DPM_CUDA_TRY(cudaMemcpyAsync(b->d_tissues + slot, &T, sizeof(Tissue3D), cudaMemcpyHostToDevice,
                               b->stream));
  DPM_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DPM_OK;
}

} // namespace dpm
