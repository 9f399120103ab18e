// Serving: continuous batching of simulation requests on resident state.
//
// A server owns slot pools (dpm_runtime.hpp): 2D pools keyed by cells per
// slot, vertices per cell and time step; 3D pools keyed by mesh and time
// step.  Every pool advances on its own stream, one chunk of steps at a
// time, independently of the others.  Whenever a pool's chunk completes,
// dpm_serve_step
//   1. reads back every request of that pool whose step budget ran out,
//      frees its slot and stamps its completion time;
//   2. admits waiting requests, oldest first, into the smallest idle pool
//      whose slots fit them, while a slot is free and the resident
//      footprint of admitted requests stays within the HBM budget (a
//      request that does not fit yet does not block smaller ones behind
//      it);
//   3. enqueues the pool's next chunk; inside a pool every tissue spends its
//      own step budget and then stays frozen.
// So 2D and 3D pools overlap on the device, a slow pool does not hold back
// a fast one, and requests join a running pool between its chunks.  A
// request's arithmetic does not depend on what shares its pool.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <thread>
#include <vector>

#include "dpm_common.cuh"
#include "dpm_runtime.hpp"

using namespace dpm;

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t id = 0;
  int dim = 2;
  int ncells = 0;
  std::vector<unsigned> nv;                     // 2D
  std::vector<float> k[8];                      // per-cell constants
  bool has_kb = false, has_adh = false;         // 3D extensions
  std::vector<float> x;                         // input, then output positions
  std::vector<float> f;                         // output forces
  float L = 1.0f, Kre = 1.0f, Kat = 0.0f;
  int pbc = 1, nsteps = 0, remaining = 0;
  float dt = 0.0f;
  size_t footprint = 0;
  int pool = -1, slot = -1;
  int status = 0;  // 0 waiting, 1 running, 2 done
  double t_submit = 0, t_admit = 0, t_done = 0;
};

struct Pool {
  int dim = 2;
  int cells_per_slot = 0, nv_max = 0; // 2D
  int nv = 0, nf = 0;                 // 3D mesh
  std::vector<unsigned> faces;
  float dt = 0.0f;
  dpm2d_batch *b2 = nullptr;
  dpm3d_batch *b3 = nullptr;
  std::vector<Request *> slots;
  int active = 0;
  bool busy = false;         // a chunk is in flight
  cudaEvent_t done = nullptr; // recorded after each chunk
};

// Longest wait for any pool's chunk before dpm_serve_step gives up.
constexpr double kPoolWaitLimitS = 300.0;

} // namespace

struct dpm_server {
  dpm_ctx *ctx = nullptr;
  size_t budget = 0, resident = 0;
  int chunk = 256;
  uint64_t next_id = 1;
  std::vector<Pool> pools;
  std::deque<Request *> waiting;
  std::map<uint64_t, std::unique_ptr<Request>> all;
  double vertex_steps = 0.0;
  ~dpm_server() {
    for (auto &p : pools) {
      if (p.b2) dpm2d_destroy(p.b2);
      if (p.b3) dpm3d_destroy(p.b3);
      if (p.done) cudaEventDestroy(p.done);
    }
  }
};

namespace {

size_t footprint2d(int ncells, const unsigned *nv) {
  size_t v = 0;
  for (int i = 0; i < ncells; ++i) v += nv[i];
  // positions x2, forces, flags; cell constants, geometry x3, lists, keys
  return v * (3 * sizeof(float2) + 1) +
         (size_t)ncells * (sizeof(Cell2D) + 3 * sizeof(Geom2D) + 4 * kMaxNB2D + 4 + 16);
}

size_t footprint3d(int ncells, int nv) {
  return (size_t)ncells * nv * (9 * sizeof(float) + 1) +
         (size_t)ncells * (sizeof(Cell3D) + 3 * sizeof(Geom3D) + 4 * kMaxNB3D + 4 + 16);
}

bool fits(const Pool &p, const Request &r) {
  if (p.dim != r.dim || p.dt != r.dt) return false;
  if (r.dim == 2) {
    if (r.ncells > p.cells_per_slot) return false;
    for (unsigned v : r.nv)
      if ((int)v > p.nv_max) return false;
    return true;
  }
  return r.ncells <= p.cells_per_slot && (int)r.x.size() == 3 * r.ncells * p.nv;
}

int admit(dpm_server *s) {
  for (auto it = s->waiting.begin(); it != s->waiting.end();) {
    Request *r = *it;
    if (s->resident + r->footprint > s->budget) {
      ++it;
      continue;
    }
    // smallest fitting pool with a free slot; among pools of the same
    // shape, the one with the fewest requests (pools of one shape run side
    // by side on their own streams, so spreading requests over them fills
    // the GPU with more independent launches)
    int best = -1, slot = -1;
    for (int p = 0; p < (int)s->pools.size(); ++p) {
      Pool &P = s->pools[p];
      if (P.busy || !fits(P, *r)) continue;
      auto fs = std::find(P.slots.begin(), P.slots.end(), nullptr);
      if (fs == P.slots.end()) continue;
      const Pool *B = best < 0 ? nullptr : &s->pools[best];
      const bool smaller =
          !B || P.cells_per_slot < B->cells_per_slot ||
          (P.cells_per_slot == B->cells_per_slot &&
           (P.nv_max < B->nv_max || (P.nv_max == B->nv_max && P.active < B->active)));
      if (smaller) {
        best = p;
        slot = (int)(fs - P.slots.begin());
      }
    }
    if (best < 0) {
      ++it;
      continue;
    }
    Pool &P = s->pools[best];
    int rc;
    if (r->dim == 2)
      rc = pool2d_assign(P.b2, slot, r->ncells, r->nv.data(), r->k[0].data(), r->k[1].data(),
                         r->k[2].data(), r->k[3].data(), r->k[4].data(), r->k[5].data(),
                         r->x.data(), r->L, r->Kre, r->Kat, r->pbc, r->nsteps);
    else
      rc = pool3d_assign(P.b3, slot, r->ncells, r->k[0].data(), r->k[1].data(), r->k[2].data(),
                         r->k[3].data(), r->k[4].data(), r->k[5].data(),
                         r->has_kb ? r->k[6].data() : nullptr,
                         r->has_adh ? r->k[7].data() : nullptr, r->x.data(), r->L, r->Kre,
                         r->pbc, r->nsteps);
    if (rc) return rc;
    P.slots[slot] = r;
    P.active++;
    r->pool = best;
    r->slot = slot;
    r->status = 1;
    r->remaining = r->nsteps;
    r->t_admit = now_s();
    s->resident += r->footprint;
    it = s->waiting.erase(it);
  }
  return DPM_OK;
}

// Accounts one completed chunk of pool P: every request's budget shrinks by
// the chunk; requests whose budget ran out are read back and their slots
// freed.
int retire(dpm_server *s, Pool &P, int *nfin) {
  for (int slot = 0; slot < (int)P.slots.size(); ++slot) {
    Request *r = P.slots[slot];
    if (!r) continue;
    const int done = std::min(r->remaining, s->chunk);
    r->remaining -= done;
    s->vertex_steps += (double)done * (r->dim == 2 ? r->x.size() / 2 : r->x.size() / 3);
    if (r->remaining > 0) continue;
    int rc;
    if (P.b2) {
      rc = pool2d_fetch(P.b2, slot, r->ncells, r->nv.data(), r->x.data(), r->f.data());
      if (!rc) rc = pool2d_release(P.b2, slot);
    } else {
      rc = pool3d_fetch(P.b3, slot, r->ncells, r->x.data(), r->f.data());
      if (!rc) rc = pool3d_release(P.b3, slot);
    }
    if (rc) return rc;
    r->status = 2;
    r->t_done = now_s();
    P.slots[slot] = nullptr;
    P.active--;
    s->resident -= r->footprint;
    ++*nfin;
  }
  return DPM_OK;
}

} // namespace

extern "C" {

int dpm_serve_create(dpm_ctx *ctx, size_t hbm_budget_bytes, int chunk_steps, dpm_server **out) {
  if (!ctx || !out) return fail(DPM_EINVAL, "null argument");
  if (chunk_steps <= 0) return fail(DPM_EINVAL, "chunk_steps must be positive");
  auto *s = new (std::nothrow) dpm_server();
  if (!s) return fail(DPM_ECAPACITY, "out of host memory");
  s->ctx = ctx;
  s->budget = hbm_budget_bytes;
  s->chunk = chunk_steps;
  ctx_retain(ctx);
  *out = s;
  return DPM_OK;
}

int dpm_serve_destroy(dpm_server *s) {
  if (!s) return DPM_OK;
  dpm_ctx *c = s->ctx;
  delete s;
  ctx_release(c);
  return DPM_OK;
}

int dpm_serve_add_pool2d(dpm_server *s, int slots, int cells_per_slot, int nv_max, float dt) {
  if (!s) return fail(DPM_EINVAL, "null server");
  Pool P;
  P.dim = 2;
  P.cells_per_slot = cells_per_slot;
  P.nv_max = nv_max;
  P.dt = dt;
  if (int r = pool2d_create(s->ctx, slots, cells_per_slot, nv_max, &P.b2)) return r;
  if (s->chunk % 16) {
    dpm2d_destroy(P.b2);
    return fail(DPM_EINVAL, "chunk_steps must be a multiple of 16 for 2D pools");
  }
  if (cudaError_t e = cudaEventCreateWithFlags(&P.done, cudaEventDisableTiming)) {
    dpm2d_destroy(P.b2);
    return cuda_fail(e, "pool event");
  }
  P.slots.assign(slots, nullptr);
  s->pools.push_back(std::move(P));
  return DPM_OK;
}

int dpm_serve_add_pool3d(dpm_server *s, int slots, int cells_per_slot, int nv, int nf,
                         const unsigned *faces, float dt) {
  if (!s || !faces) return fail(DPM_EINVAL, "null argument");
  Pool P;
  P.dim = 3;
  P.cells_per_slot = cells_per_slot;
  P.nv = nv;
  P.nf = nf;
  P.dt = dt;
  P.faces.assign(faces, faces + 3 * (size_t)nf);
  if (int r = pool3d_create(s->ctx, slots, cells_per_slot, nv, nf, faces, &P.b3)) return r;
  if (s->chunk % 16) {
    dpm3d_destroy(P.b3);
    return fail(DPM_EINVAL, "chunk_steps must be a multiple of 16 for 3D pools");
  }
  if (cudaError_t e = cudaEventCreateWithFlags(&P.done, cudaEventDisableTiming)) {
    dpm3d_destroy(P.b3);
    return cuda_fail(e, "pool event");
  }
  P.slots.assign(slots, nullptr);
  s->pools.push_back(std::move(P));
  return DPM_OK;
}

int dpm_serve_pool_bytes(dpm_server *s, size_t *bytes) {
  if (!s || !bytes) return fail(DPM_EINVAL, "null argument");
  size_t t = 0;
  for (auto &p : s->pools) t += p.b2 ? pool2d_bytes(p.b2) : pool3d_bytes(p.b3);
  *bytes = t;
  return DPM_OK;
}

int dpm_serve_submit2d(dpm_server *s, int ncells, const unsigned *nv, const float *Ka,
                       const float *Kl, const float *Kb, const float *a0, const float *l0,
                       const float *r0, const float *xy, float L, float Kre, float Kat, int pbc,
                       int nsteps, float dt, uint64_t *id) {
  if (!s || !nv || !Ka || !Kl || !Kb || !a0 || !l0 || !r0 || !xy || !id)
    return fail(DPM_EINVAL, "null argument");
  if (ncells <= 0 || nsteps <= 0) return fail(DPM_EINVAL, "empty request");
  try {
    auto r = std::make_unique<Request>();
    r->dim = 2;
    r->ncells = ncells;
    r->nv.assign(nv, nv + ncells);
    const float *src[6] = {Ka, Kl, Kb, a0, l0, r0};
    for (int i = 0; i < 6; ++i) r->k[i].assign(src[i], src[i] + ncells);
    size_t V = 0;
    for (int i = 0; i < ncells; ++i) V += nv[i];
    r->x.assign(xy, xy + 2 * V);
    r->f.assign(2 * V, 0.0f);
    r->L = L;
    r->Kre = Kre;
    r->Kat = Kat;
    r->pbc = pbc;
    r->nsteps = nsteps;
    r->dt = dt;
    r->footprint = footprint2d(ncells, nv);
    bool any = false;
    for (auto &p : s->pools) any |= fits(p, *r);
    if (!any) return fail(DPM_ECAPACITY, "no pool can hold this request");
    if (r->footprint > s->budget) return fail(DPM_ECAPACITY, "request exceeds the HBM budget");
    r->id = s->next_id++;
    r->t_submit = now_s();
    *id = r->id;
    s->waiting.push_back(r.get());
    s->all.emplace(r->id, std::move(r));
    return DPM_OK;
  } catch (const std::bad_alloc &) {
    return fail(DPM_ECAPACITY, "out of host memory");
  }
}

int dpm_serve_submit3d(dpm_server *s, int ncells, int nv, const float *Kv, const float *Ka,
                       const float *Ks, const float *v0, const float *a0, const float *l0,
                       const float *Kb, const float *adh, const float *xyz, float L, float Kre,
                       int pbc, int nsteps, float dt, uint64_t *id) {
  if (!s || !Kv || !Ka || !Ks || !v0 || !a0 || !l0 || !xyz || !id)
    return fail(DPM_EINVAL, "null argument");
  if (ncells <= 0 || nsteps <= 0 || nv <= 0) return fail(DPM_EINVAL, "empty request");
  try {
    auto r = std::make_unique<Request>();
    r->dim = 3;
    r->ncells = ncells;
    const float *src[8] = {Kv, Ka, Ks, v0, a0, l0, Kb, adh};
    for (int i = 0; i < 8; ++i)
      if (src[i]) r->k[i].assign(src[i], src[i] + ncells);
    r->has_kb = Kb != nullptr;
    r->has_adh = adh != nullptr;
    r->x.assign(xyz, xyz + 3 * (size_t)ncells * nv);
    r->f.assign(3 * (size_t)ncells * nv, 0.0f);
    r->L = L;
    r->Kre = Kre;
    r->pbc = pbc;
    r->nsteps = nsteps;
    r->dt = dt;
    r->footprint = footprint3d(ncells, nv);
    bool any = false;
    for (auto &p : s->pools) any |= fits(p, *r);
    if (!any) return fail(DPM_ECAPACITY, "no pool can hold this request");
    if (r->footprint > s->budget) return fail(DPM_ECAPACITY, "request exceeds the HBM budget");
    r->id = s->next_id++;
    r->t_submit = now_s();
    *id = r->id;
    s->waiting.push_back(r.get());
    s->all.emplace(r->id, std::move(r));
    return DPM_OK;
  } catch (const std::bad_alloc &) {
    return fail(DPM_ECAPACITY, "out of host memory");
  }
}

int dpm_serve_step(dpm_server *s, int *active, int *waiting, int *finished) {
  if (!s) return fail(DPM_EINVAL, "null server");
  cudaSetDevice(s->ctx->device);
  int nfin = 0;
  const double deadline = now_s() + kPoolWaitLimitS;
  for (;;) {
    // pools whose chunk completed
    int progressed = 0;
    for (auto &P : s->pools) {
      if (!P.busy) continue;
      const cudaError_t e = cudaEventQuery(P.done);
      if (e == cudaErrorNotReady) continue;
      if (e != cudaSuccess) return cuda_fail(e, "pool chunk");
      P.busy = false;
      ++progressed;
      if (int r = retire(s, P, &nfin)) return r;
    }
    if (int r = admit(s)) return r;
    // next chunk on every idle pool with work, each on its own stream
    int inflight = 0;
    for (auto &P : s->pools) {
      if (!P.busy && P.active) {
        // launch over the slots up to the highest occupied one
        int hi = (int)P.slots.size();
        while (hi > 0 && !P.slots[hi - 1]) --hi;
        if (P.b2) pool2d_set_active(P.b2, hi);
        else pool3d_set_active(P.b3, hi);
        const int rc =
            P.b2 ? pool2d_run(P.b2, s->chunk, P.dt) : pool3d_run(P.b3, s->chunk, P.dt);
        if (rc) return rc;
        const cudaStream_t st = P.b2 ? pool2d_stream(P.b2) : pool3d_stream(P.b3);
        if (cudaError_t e = cudaEventRecord(P.done, st)) return cuda_fail(e, "pool event");
        P.busy = true;
      }
      inflight += P.busy ? 1 : 0;
    }
    if (progressed || !inflight) break;
    if (now_s() > deadline) return fail(DPM_ECUDA, "timed out waiting for a pool's chunk");
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  if (active) {
    int a = 0;
    for (auto &P : s->pools) a += P.active;
    *active = a;
  }
  if (waiting) *waiting = (int)s->waiting.size();
  if (finished) *finished = nfin;
  return DPM_OK;
}

int dpm_serve_drain(dpm_server *s) {
  if (!s) return fail(DPM_EINVAL, "null server");
  int a = 0, w = 0;
  do {
    if (int r = dpm_serve_step(s, &a, &w, nullptr)) return r;
  } while (a || w);
  return DPM_OK;
}

int dpm_serve_result(dpm_server *s, uint64_t id, float *x, float *F, double *latency_s,
                     int *status) {
  if (!s) return fail(DPM_EINVAL, "null server");
  auto it = s->all.find(id);
  if (it == s->all.end()) return fail(DPM_EINVAL, "unknown request id");
  Request &r = *it->second;
  if (status) *status = r.status;
  if (r.status != 2) return DPM_OK;
  if (x) std::memcpy(x, r.x.data(), sizeof(float) * r.x.size());
  if (F) std::memcpy(F, r.f.data(), sizeof(float) * r.f.size());
  if (latency_s) *latency_s = r.t_done - r.t_submit;
  return DPM_OK;
}
int dpm_serve_forget(dpm_server *s, uint64_t id) {
  if (!s) return fail(DPM_EINVAL, "null server");
  auto it = s->all.find(id);
  if (it == s->all.end()) return fail(DPM_EINVAL, "unknown request id");
  if (it->second->status != 2) return fail(DPM_ESTATE, "request still running");
  s->all.erase(it);
  return DPM_OK;
}

int dpm_serve_stats(dpm_server *s, double *vertex_steps, size_t *resident_bytes) {
  if (!s) return fail(DPM_EINVAL, "null server");
  if (vertex_steps) *vertex_steps = s->vertex_steps;
  if (resident_bytes) *resident_bytes = s->resident;
  return DPM_OK;
}

} // extern "C"
