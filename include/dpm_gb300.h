/*
 * dpm_gb300 -- C ABI of the GB300 (sm_103a) Deformable Particle Model step.
 *
 * This is the drop-in boundary beneath the clDPM Python module
 * (Cell2D/Tissue2D/Cell3D/Tissue3D).  It replaces the OpenCL buffers,
 * program build and kernel enqueues inside the reference's step loops:
 *
 *   Tissue2D::CLEulerUpdate   src/Tissue2D.cpp:116-241
 *   Tissue3D::CLEulerUpdate   src/Tissue3D.cpp:118-522
 *
 * and the kernels they enqueue (shaders/Cell2D_kernel.cl,
 * shaders/Cell3D_Kernel.cl).  Reference lines for each entry point are given
 * beside it.
 *
 * Conventions
 *  - Every function returns 0 on success or a DPM_E* code; the message of the
 *    last failure on the calling thread is returned by dpm_last_error().
 *  - All pointers in signatures are HOST pointers owned by the caller, except
 *    where a name says "_dev".  Device state is owned by the object.
 *  - A context owns one CUDA stream; objects created from it run on that
 *    stream.  An object is not re-entrant; distinct contexts may be used from
 *    distinct threads.
 *  - 2D vertex data are ragged and cell-major: cell c's vertex v is at
 *    xy[2*(first(c)+v)], first(c) = sum of nv over the cells before c.
 *    3D vertex data are cell-major with one face table for all cells:
 *    xyz[3*(c*nv+v)].
 *  - A "batch" holds one or more independent tissues that step together;
 *    a batch of one tissue is the plain single-system path.
 */
#ifndef DPM_GB300_H
#define DPM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DPM_OK 0
#define DPM_EINVAL 1    /* bad argument (std::invalid_argument in the reference) */
#define DPM_ECUDA 2     /* CUDA runtime failure */
#define DPM_ECAPACITY 3 /* size beyond a documented limit */
#define DPM_ENONFINITE 4 /* non-finite vertex positions after stepping */
#define DPM_ESTATE 5    /* call out of order (e.g. step before upload) */

typedef struct dpm_ctx dpm_ctx;
typedef struct dpm2d_batch dpm2d_batch;
typedef struct dpm3d_batch dpm3d_batch;

/* Last error message of the calling thread ("" if none). */
const char *dpm_last_error(void);

/* Library version string. */
const char *dpm_version(void);

/* ---------------------------------------------------------------------- */
/* Context: device + stream.  Replaces the per-object cl::Platform/Device/  */
/* Context/CommandQueue (src/Tissue2D.cpp:35-37, 213; src/Tissue3D.cpp:32-34,*/
/* 362).                                                                    */
/* ---------------------------------------------------------------------- */
int dpm_ctx_create(int device, dpm_ctx **out);
int dpm_ctx_destroy(dpm_ctx *ctx);
int dpm_ctx_synchronize(dpm_ctx *ctx);
/* Number of SMs of the context's device (for schedulers and tuners). */
int dpm_ctx_sm_count(dpm_ctx *ctx, int *out);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work (timing events, copies) with the library's. */
int dpm_ctx_stream(dpm_ctx *ctx, void **stream);

/* ---------------------------------------------------------------------- */
/* 2D batches                                                              */
/* ---------------------------------------------------------------------- */

/* Creates a batch of ntissues tissues; tissue t has ncells[t] cells and the
 * cells (in tissue order) have nv[] vertices each (3 <= nv <= 256).
 * Replaces the buffer sizing of src/Tissue2D.cpp:117-140, 149-168. */
int dpm2d_create(dpm_ctx *ctx, int ntissues, const int *ncells,
                 const unsigned *nv, dpm2d_batch **out);
int dpm2d_destroy(dpm2d_batch *b);

/* Per-cell constants, one value per cell in batch order: Ka, Kl, Kb, a0, l0,
 * r0 (the fields of DPM::Cell2D the kernels read, src/Tissue2D.cpp:129-136).
 */
int dpm2d_set_cells(dpm2d_batch *b, const float *Ka, const float *Kl,
                    const float *Kb, const float *a0, const float *l0,
                    const float *r0);

/* Per-tissue constants, one value per tissue: box size L, repulsion Kre,
 * attraction Kat, periodic flag pbc (the kernel arguments set at
 * src/Tissue2D.cpp:195-205). */
int dpm2d_set_tissues(dpm2d_batch *b, const float *L, const float *Kre,
                      const float *Kat, const int *pbc);

/* Vertex positions in (host, float[2*total]); returns after the copy and
 * the initial geometry are complete.  Replaces the COPY_HOST_PTR upload of
 * src/Tissue2D.cpp:149-151. */
int dpm2d_upload(dpm2d_batch *b, const float *xy);

/* Runs nsteps overdamped Euler steps of size dt on every tissue.  Replaces
 * the step loop of src/Tissue2D.cpp:215-229 (area, perimeter, bending,
 * attraction and repulsion forces, then x += F*dt). */
int dpm2d_step(dpm2d_batch *b, int nsteps, float dt);

/* Positions and the forces of the last step (host float[2*total] each; F may
 * be NULL).  Replaces the read-backs of src/Tissue2D.cpp:223-233. */
int dpm2d_download(dpm2d_batch *b, float *xy, float *F);

/* Totals of a batch: cells and vertices. */
int dpm2d_sizes(dpm2d_batch *b, int *ncells, long *nvertices);

/* Tuning knobs (0 keeps the current value): neighbour-list rebuild period
 * in steps (even) and skin distance relative to the mean cell radius. */
int dpm2d_set_tuning(dpm2d_batch *b, int rebuild_period, float skin_rel,
                     int warps_per_block);
/* Step-kernel variant 0..3 (bit 0: registers capped for 48 resident warps
 * per SM; bit 1: dynamic schedule), plus 8 to switch off the resident run:
 * batches whose tissues are all small (at most 64 cells and 2,048 vertices,
 * rings of at most 64) otherwise step with one block per tissue holding the
 * tissue in shared memory for the whole call; plus 32 for four warps per
 * cell that split the cell's neighbours (batches without attraction whose
 * rings have at most 64 vertices; for batches too small to fill the GPU).
 * Every variant gives identical results; dpm2d_autotune picks the fastest
 * graph-path variant. */
int dpm2d_set_kernel_variant(dpm2d_batch *b, int variant);

/* Diagnostics: per-vertex containment flags of the last step (uint8 per
 * vertex; 1 = inside another cell, the reference's `overlaps`), per-cell
 * area (float), and counts of neighbour-list rebuilds / brute-force steps. */
int dpm2d_last_contained(dpm2d_batch *b, unsigned char *flags);
int dpm2d_cell_areas(dpm2d_batch *b, float *area);
int dpm2d_stats(dpm2d_batch *b, long *rebuilds, long *fallback_steps);
/* Ensemble diagnostics of the current state, computed on the device in
 * double (any output may be NULL).  Per cell: |area|, perimeter and the
 * energy Ka/2 (A/a0-1)^2 + Kl/2 sum (l/l0-1)^2 + Kb/2 sum |s_i|^2 (project-
 * defined; the reference has none, and its area force is not this energy's
 * gradient).  Per tissue: packing fraction sum(A)/L^2 and the mean shape
 * index P/sqrt(4 pi A). */
int dpm2d_diagnostics(dpm2d_batch *b, double *area, double *perimeter,
                      double *energy, double *packing_fraction,
                      double *shape_index);

/* One compression (or expansion) stage on the device: every tissue t with
 * phi[t] > 0 gets the box side L' = sqrt(sum of cell areas / phi[t]) and
 * each cell moves rigidly with its vertex-mean centroid scaled by L'/L;
 * phi[t] == 0 leaves tissue t unchanged.  The same arithmetic, and the same
 * bits, as the host Tissue2D.SetPackingFraction.  An extension: the
 * reference fixes L at construction (src/Tissue2D.cpp:31) and has no
 * compression protocol; this is the quasi-static jamming protocol's box
 * update without a round trip of the positions through the host.
 * Synchronizes the batch's stream (the host copy of L is refreshed). */
int dpm2d_set_packing_fraction(dpm2d_batch *b, const float *phi);

/* State I/O.  dpm2d_device_state returns the DEVICE addresses of the
 * current positions and of the last step's forces (float2 per vertex, the
 * layout of dpm2d_upload), for zero-copy views; they stay valid until the
 * next call that steps or uploads (positions alternate between two buffers).
 * dpm2d_save writes the batch (shape, cell and tissue constants, positions,
 * forces) to a checkpoint file; dpm2d_open creates a batch from one, which
 * steps on exactly as the saved batch would have (the cell lists are
 * rebuilt; their pruning is exact).  Replaces reading Cell2D::Verticies /
 * Forces back after CLEulerUpdate (src/Tissue2D.cpp:223-240). */
int dpm2d_device_state(dpm2d_batch *b, void **positions, void **forces);
int dpm2d_save(dpm2d_batch *b, const char *path);
int dpm2d_open(dpm_ctx *ctx, const char *path, dpm2d_batch **out);

/* Cell-list snapshot for host verification (see dpm2d_rebuild_now):
 * sorted bin keys and cell ids (uint32[ncells] each), per-cell neighbour
 * counts (int32[ncells]) and lists (int32[ncells*maxnb]). */
int dpm2d_rebuild_now(dpm2d_batch *b);
int dpm2d_cell_list(dpm2d_batch *b, unsigned *keys, unsigned *ids,
                    int *nn, int *nbr, int *maxnb, float *geom);
/* Bin layout of the last rebuild: bits of the local bin index in a key,
 * and per tissue the bins per axis, bin width and skin. */
int dpm2d_bins(dpm2d_batch *b, int *local_bits, int *nbins, float *binw,
               float *skin);
/* Enqueues exactly one launch of the fused step kernel on the context's
 * stream (no rebuild; stale lists fall back to a tissue scan), without
 * synchronizing.  For per-kernel timing and profiling. */
int dpm2d_step_kernel(dpm2d_batch *b, float dt);

/* Autotuner: times warps per block (4, 8, 16) x step-kernel variant (bit 0:
 * registers capped for 32 resident warps per SM, else the compiler's choice;
 * bit 1: dynamic schedule, resident warps taking cells from a counter, else
 * one warp per cell in launch order) x (rebuild period, skin) on this
 * batch's current state, restores the state, and applies the
 * fastest.  Choices are cached as JSON lines keyed by the batch's shape in
 * $DPM_TUNE_CACHE (default ~/.cache/dpm_gb300_tune2d.jsonl); with use_cache
 * a cached choice is applied without trials.  Allocates a temporary copy of
 * the state while tuning.  Outputs may be NULL; ms_per_step is -1 when the
 * choice came from the cache. */
int dpm2d_autotune(dpm2d_batch *b, float dt, int trial_blocks, int use_cache,
                   int *warps, int *occupancy, int *rebuild_period,
                   float *skin_rel, float *ms_per_step);

/* ---------------------------------------------------------------------- */
/* 2D step without device allocation                                       */
/* ---------------------------------------------------------------------- */

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory -- a program whose device memory belongs to another framework's
 * pool, code that must not synchronize the device the way cudaMalloc and
 * cudaFree can, or an embedded use that reserves all memory at start-up.
 *
 * Runs nsteps steps of one 2D tissue, exactly as a one-tissue dpm2d batch
 * does, and allocates nothing: the caller passes its own DEVICE buffer of
 * positions (xy_dev, float[2*total], updated in place) and optionally one for
 * the last step's forces (F_dev, may be NULL); the per-cell constants (nv,
 * Ka, Kl, Kb, a0, l0, r0) are HOST arrays.  All other working memory is one
 * fixed device array inside the library (about 1.7 MB, held on every GPU that
 * loads the library until the process exits), so:
 *   - ncells <= DPM_NOALLOC_MAX_CELLS and total vertices <=
 *     DPM_NOALLOC_MAX_VERTICES, 3..256 vertices per cell; larger inputs are
 *     rejected with DPM_ECAPACITY;
 *   - every call shares that array, and its contents are not valid between
 *     calls.  Calls that overlapped on the GPU would race on it; the library
 *     serializes calls with a process-wide lock (calls on different devices
 *     too), and each returns only after its work is done, so calls from
 *     several host threads never overlap inside the library;
 *   - the first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) once and keeps it for the life of the process:
 *     do not reset the device (cudaDeviceReset) between calls, and call from
 *     the device's primary context;
 *   - nsteps == 0 does no device work (xy_dev and F_dev are left as they
 *     are).
 * Work is enqueued on `stream` (a cudaStream_t) and the call blocks until
 * that stream has drained.  NULL means the legacy default stream, which also
 * waits for every other blocking stream on the device: a caller that must
 * not synchronize the whole device passes its own non-blocking stream. */
#define DPM_NOALLOC_MAX_CELLS 2048
#define DPM_NOALLOC_MAX_VERTICES 65536
int dpm2d_step_noalloc(int ncells, const unsigned *nv, const float *Ka,
                       const float *Kl, const float *Kb, const float *a0,
                       const float *l0, const float *r0, float L, float Kre,
                       float Kat, int pbc, float *xy_dev, float *F_dev,
                       int nsteps, float dt, void *stream);

/* ---------------------------------------------------------------------- */
/* 3D batches                                                              */
/* ---------------------------------------------------------------------- */

/* Creates a batch of 3D tissues whose cells all share the mesh topology
 * faces[nf*3] over nv vertices (the reference uses cell 0's face table for
 * every cell, src/Tissue3D.cpp:144-146).  nv <= 642 (icosphere subdivision
 * 3). */
int dpm3d_create(dpm_ctx *ctx, int ntissues, const int *ncells, int nv,
                 int nf, const unsigned *faces, dpm3d_batch **out);
int dpm3d_destroy(dpm3d_batch *b);

/* Per-cell constants (src/Tissue3D.cpp:172-178): Kv, Ka, Ks, v0, a0, l0.
 * Kb (triangle bending) and adh (adhesion range; default 2*l0) are
 * extensions and may be NULL. */
int dpm3d_set_cells(dpm3d_batch *b, const float *Kv, const float *Ka,
                    const float *Ks, const float *v0, const float *a0,
                    const float *l0, const float *Kb, const float *adh);
/* Per-tissue constants: L, Kre (the reference's Kc), pbc. */
int dpm3d_set_tissues(dpm3d_batch *b, const float *L, const float *Kre,
                      const int *pbc);
/* Opt-in: the reference's AllVertAttraction kernel
 * (shaders/Cell3D_Kernel.cl:313-364), which its own step loop
 * (src/Tissue3D.cpp:372-445) never enqueues, run after the repulsion of
 * every step with strength Kat[t] per tissue (0 = off, the default).  Call
 * after dpm3d_set_cells and dpm3d_set_tissues. */
int dpm3d_set_attraction(dpm3d_batch *b, const float *Kat);
int dpm3d_upload(dpm3d_batch *b, const float *xyz);
/* Replaces the step loop of src/Tissue3D.cpp:372-445. */
int dpm3d_step(dpm3d_batch *b, int nsteps, float dt);
/* Forces are those of the last step (read after its Euler update,
 * src/Tissue3D.cpp:425-434). */
int dpm3d_download(dpm3d_batch *b, float *xyz, float *F);
int dpm3d_sizes(dpm3d_batch *b, int *ncells, long *nvertices);
/* Neighbour-list rebuild period (steps) and skin relative to the mean cell
 * diameter (0 keeps the current value). */
int dpm3d_set_tuning(dpm3d_batch *b, int rebuild_period, float skin_rel);
/* Threads per cell of the step kernel: 128, 256 or 512, or 0 for the
 * default (256 when the batch has more cells than two 512-thread blocks per
 * SM hold and the mesh's shared memory lets four cells share an SM, e.g.
 * subdivision 2; 512 otherwise).  Results are the same bits for every
 * choice. */
int dpm3d_set_block_threads(dpm3d_batch *b, int threads);
/* Per-vertex count of other cells whose winding number passed the
 * reference's threshold in the last step (uint8 per vertex). */
int dpm3d_last_winding(dpm3d_batch *b, unsigned char *counts);
/* Per-cell diagnostics of the current state, computed on the device in
 * double (any output may be NULL): enclosed volume and surface area
 * (Cell3D::GetVolume / GetSurfaceArea, src/cell.cpp:196-230, for every
 * cell at once) and the energy Kv/2 (V/v0-1)^2 + Ka/2 sum_edges (l/l0-1)^2
 * + Kb sum_edges (1 - n1.n2) (project-defined; the reference has none). */
int dpm3d_diagnostics(dpm3d_batch *b, double *volume, double *surface_area,
                      double *energy);
/* State I/O as for 2D: device addresses of the current x, y, z (structure of
 * arrays, cell-major) and of the last step's force components; checkpoint
 * save and open (mesh included).  Replaces Cell3D::GetPositions /
 * GetForces (src/cell.cpp:232-274) for device-side consumers. */
int dpm3d_device_state(dpm3d_batch *b, void **x, void **y, void **z, void **fx,
                       void **fy, void **fz);
int dpm3d_save(dpm3d_batch *b, const char *path);
int dpm3d_open(dpm_ctx *ctx, const char *path, dpm3d_batch **out);

/* ---------------------------------------------------------------------- */
/* Dispersion of cell centres                                              */
/* ---------------------------------------------------------------------- */

/* Relaxes the centres of nsystems independent systems of soft discs, as the
 * loop of Tissue2D::Disperse (src/Tissue2D.cpp:53-104) and
 * Tissue3D::Disperse2D (src/Tissue3D.cpp:40-106), bit for bit: overlap
 * force (1 - d/(ri+rj))/(ri+rj) over periodic offsets, step 0.01, until the
 * energy changes by at most 1e-6 or after 1e5 iterations.  ncells[s] cells
 * (<= 4096) per system, concatenated in radius, X, Y; L[s] the box side.
 * X, Y hold the starting centres (the reference draws them with drand48)
 * and receive the relaxed ones; iterations[s] (may be NULL) the iteration
 * count, above 1e5 when the cap was hit.  One thread block per system. */
int dpm_disperse(dpm_ctx *ctx, int nsystems, const int *ncells,
                 const float *radius, const float *L, float *X, float *Y,
                 int *iterations);

/* ---------------------------------------------------------------------- */
/* Serving: continuous batching of independent simulation requests.       */
/* The reference runs one Tissue per process, looping CLEulerUpdate        */
/* (src/Tissue2D.cpp:116-241, src/Tissue3D.cpp:118-522); a server keeps     */
/* many requests resident in slot pools and steps them together.           */
/* ---------------------------------------------------------------------- */

typedef struct dpm_server dpm_server;

/* hbm_budget_bytes bounds the resident footprint of admitted requests;
 * chunk_steps is the number of steps each round runs (a multiple of 16). */
int dpm_serve_create(dpm_ctx *ctx, size_t hbm_budget_bytes, int chunk_steps,
                     dpm_server **out);
int dpm_serve_destroy(dpm_server *s);
/* A pool of `slots` 2D tissues of up to cells_per_slot cells with up to
 * nv_max vertices each, stepped with time step dt. */
int dpm_serve_add_pool2d(dpm_server *s, int slots, int cells_per_slot,
                         int nv_max, float dt);
/* A pool of 3D tissues sharing one mesh (nv vertices, faces[nf*3]). */
int dpm_serve_add_pool3d(dpm_server *s, int slots, int cells_per_slot, int nv,
                         int nf, const unsigned *faces, float dt);
int dpm_serve_pool_bytes(dpm_server *s, size_t *bytes);
/* Queues one tissue for nsteps steps; the arguments mean what they mean in
 * dpm2d_set_cells / dpm2d_set_tissues / dpm2d_upload for a batch of one
 * tissue.  Fails with DPM_ECAPACITY when no pool can ever hold it. */
int dpm_serve_submit2d(dpm_server *s, int ncells, const unsigned *nv,
                       const float *Ka, const float *Kl, const float *Kb,
                       const float *a0, const float *l0, const float *r0,
                       const float *xy, float L, float Kre, float Kat, int pbc,
                       int nsteps, float dt, uint64_t *id);
int dpm_serve_submit3d(dpm_server *s, int ncells, int nv, const float *Kv,
                       const float *Ka, const float *Ks, const float *v0,
                       const float *a0, const float *l0, const float *Kb,
                       const float *adh, const float *xyz, float L, float Kre,
                       int pbc, int nsteps, float dt, uint64_t *id);
/* Advances the server: every pool runs chunks of chunk_steps on its own
 * stream, independently of the others.  Returns once at least one pool has
 * completed a chunk (its finished requests read back, waiting requests
 * admitted into it, its next chunk enqueued), or at once when nothing is in
 * flight.  Counts afterwards are returned (any pointer may be NULL);
 * `finished` counts the requests completed by this call.  A wait longer than
 * 300 s fails with DPM_ECUDA. */
int dpm_serve_step(dpm_server *s, int *active, int *waiting, int *finished);
/* Calls dpm_serve_step until nothing is running or waiting. */
int dpm_serve_drain(dpm_server *s);
/* status: 0 waiting, 1 running, 2 done.  When done, copies the final
 * positions and the forces of the request's last step, and the time from
 * submit to completion. */
int dpm_serve_result(dpm_server *s, uint64_t id, float *x, float *F,
                     double *latency_s, int *status);
/* Drops a finished request's host copy. */
int dpm_serve_forget(dpm_server *s, uint64_t id);
int dpm_serve_stats(dpm_server *s, double *vertex_steps, size_t *resident_bytes);

#ifdef __cplusplus
}
#endif

#endif
