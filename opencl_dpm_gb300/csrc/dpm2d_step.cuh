// The fused 2D step (k2d_step): the per-cell device function and its
// kernels, templated on vertex slots per lane S, warps per block W, the
// occupancy variant OCC and ATT (attraction compiled in).  Each
// dpm2d_step_s<S>.cu instantiates one S, so the variants compile in
// parallel.
#pragma once

#include "dpm2d_device.cuh"

namespace dpm {
namespace {

// ---------------------------------------------------------------------------
// Fused step
// ---------------------------------------------------------------------------

// Occupancy variants: with OCC = 1 the register budget is capped so that
// 48 warps per SM stay resident (40 registers, a few spilled: the step
// waits mostly on L2 loads of the neighbours' rings, and more resident
// warps hide them better than 32 warps at 64 registers; 16 warps for more
// than 2 vertex slots per lane); with OCC = 0 the compiler chooses.  The
// tuner picks per batch.
template <int S, int W, int OCC> struct StepOcc {
  static constexpr int kThreads = S <= 2 ? 1536 : 512;
  static constexpr int kBlocks =
      OCC == 0 ? 1 : (kThreads / (W * 32) > 0 ? kThreads / (W * 32) : 1);
};

// One step of cell c by one warp; (sx, sy), (nxs, nys) and sf are the warp's
// shared-memory ring, neighbour ring and containment flags (32*S entries).
//
// TEAM > 1: the TEAM warps of a block step the cell together (no
// attraction).  Warp `team` 0 forms the shape forces and, after the block's
// barrier, the repulsion toward the own centre, the Euler update and the
// next step's geometry; every warp screens the list and takes every TEAM-th
// passing neighbour, OR-ing containment flags into the block's sf.  A flag
// is the OR over neighbours, so the result does not depend on which warp
// took which neighbour: the same bits as one warp.
template <int S, bool ATT, int TEAM = 1>
__device__ __forceinline__ void step_cell(const Step2DArgs &a, const int c, const int lane,
                                          float *sx, float *sy, float *nxs, float *nys,
                                          unsigned char *sf, const int team = 0) {
  static_assert(TEAM == 1 || !ATT, "the attraction adds forces in list order: one warp");
  const Cell2D cp = a.cells[c];
  const int n = (int)cp.nv;
  if (n == 0) return;  // an empty slot
  const int tid = (int)cp.tissue;
  const Tissue2D T = a.tissues[tid];
  if (a.step_index >= T.run_now) {
    // the tissue's step budget is spent: carry its state over unchanged
    if (team != 0) return;
    for (int k = lane; k < n; k += 32) a.pos_out[cp.voff + k] = a.pos_in[cp.voff + k];
    if (lane == 0) a.geom_out[c] = a.geom_in[c];
    return;
  }
  // outputs of this step: for every cell when asked, else at the tissue's last step
  const bool write_out =
      a.all_forces != 0 || (a.step_index == T.run_now - 1 && T.steps_left == 0);
  const float L = T.L;
  const bool pbc = T.pbc != 0;

  float vx[S], vy[S], fx[S], fy[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int k = lane + 32 * s;
    vx[s] = vy[s] = fx[s] = fy[s] = 0.0f;
    if (k < n) {
      const float2 v = a.pos_in[cp.voff + k];
      vx[s] = v.x;
      vy[s] = v.y;
      if (team == 0) {
        sx[k] = v.x;
        sy[k] = v.y;
        sf[k] = 0;
      }
    }
  }
  if constexpr (TEAM > 1) __syncthreads();
  else __syncwarp();
  const Geom2D gi = a.geom_in[c];

  // -- shape forces: area (AreaForceUpdates, with the reference's sign of
  // the y term), perimeter (PerimeterForceUpdates), bending
  // (BendingForceUpdates); summed in the reference's order.
  const float strain = gi.area / cp.a0 - 1.0f;
  const float ka = cp.kA * 0.5f * strain;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int k = lane + 32 * s;
    if (k < n && team == 0) {
      const int im1 = k == 0 ? n - 1 : k - 1;
      const int ip1 = k == n - 1 ? 0 : k + 1;
      const int im2 = im1 == 0 ? n - 1 : im1 - 1;
      const int ip2 = ip1 == n - 1 ? 0 : ip1 + 1;
      const float x = vx[s], y = vy[s];
      const float xm = sx[im1], ym = sy[im1], xp = sx[ip1], yp = sy[ip1];
      const float xmm = sx[im2], ymm = sy[im2], xpp = sx[ip2], ypp = sy[ip2];
      const float ax = ka * (ym - yp), ay = ka * (xm - xp);
      const float lvx = xp - x, lvy = yp - y, lmx = x - xm, lmy = y - ym;
      const float len = sqrtf(lvx * lvx + lvy * lvy), lenm = sqrtf(lmx * lmx + lmy * lmy);
      // unit vectors and strains with reciprocals (within 1 ulp of the
      // reference's divisions)
      const float il = 1.0f / len, ilm = 1.0f / lenm;
      const float dl = len * cp.inv_l0 - 1.0f, dlm = lenm * cp.inv_l0 - 1.0f;
      const float px = cp.kL * (dl * (lvx * il) - dlm * (lmx * ilm));
      const float py = cp.kL * (dl * (lvy * il) - dlm * (lmy * ilm));
      const float six = lvx - lmx, siy = lvy - lmy;
      const float sixp = (xpp - xp) - lvx, siyp = (ypp - yp) - lvy;
      const float sixm = lmx - (xm - xmm), siym = lmy - (ym - ymm);
      const float bx = cp.Kb * (2.0f * six - sixm - sixp);
      const float by = cp.Kb * (2.0f * siy - siym - siyp);
      fx[s] = (ax + px) + bx;
      fy[s] = (ay + py) + by;
    }
  }

  // -- attraction and repulsion against the neighbour list (cells in
  // ascending order, as the reference loops over them).
  // (nn null: no lists, every cell of the tissue is screened)
  const int nnc = a.nn ? a.nn[c] : kNbOverflow;
  const bool scan_all =
      nnc == kNbOverflow || *((volatile const int *)(a.stale + tid)) != 0;
  const int count = scan_all ? (T.cell_end - T.cell_begin) : nnc;
  const int *list = a.nbr + (size_t)c * kMaxNB2D;
  const bool att = ATT && T.Kat != 0.0f;
  int ordinal = 0;  // passing neighbours seen (team mode)
  // Lanes screen up to 32 list entries at once (one geometry load each, in
  // parallel); the cells that pass are then processed one by one, in list
  // order, with their geometry broadcast by shuffles.
  for (int base = 0; base < count; base += 32) {
    const int q = base + lane;
    int jl = -1;
    unsigned pflags = 0u;
    unsigned jvoff = 0u, jnv = 0u;
    Geom2D gl;
    gl.cx = gl.cy = gl.R = gl.area = gl.minx = gl.maxx = gl.miny = gl.maxy = 0.0f;
    if (q < count) {
      jl = scan_all ? T.cell_begin + q : list[q];
      if (jl != c) {
        // the ring's place (first vertex, count), loaded beside the
        // geometry for all 32 entries at once rather than one round trip
        // per passing cell below
        const uint4 r = *reinterpret_cast<const uint4 *>(a.cells + jl);
        gl = a.geom_in[jl];
        jvoff = r.x;
        jnv = r.y;
        const float dcx = gi.cx - gl.cx, dcy = gi.cy - gl.cy;
        const float rr = gi.R + gl.R;
        const float mm = kRelMargin * rr + kAbsMargin * (fabsf(gi.cx) + fabsf(gi.cy) +
                                                         fabsf(gl.cx) + fabsf(gl.cy));
        // own y range must meet (miny_j, maxy_j] unless y offsets can shift
        const bool yover = gi.maxy > gl.miny && gi.miny <= gl.maxy;
        // and its x range must meet the widened box of j: a vertex's box
        // test (vertex_candidate) widens by at most this margin
        const float bmx = kRelMargin * (gl.maxx - gl.minx) +
                          kAbsMargin * (fabsf(gl.minx) + fabsf(gl.maxx) +
                                        fmaxf(fabsf(gi.minx), fabsf(gi.maxx)));
        const bool xover = gi.maxx >= gl.minx - bmx && gi.minx <= gl.maxx + bmx;
        const bool near = yover && xover && dcx * dcx + dcy * dcy <= (rr + mm) * (rr + mm);
        const bool farx = pbc && (__fsub_rn(gi.maxx, gl.minx) > L || __fsub_rn(gl.maxx, gi.minx) > L);
        const bool fary = pbc && (__fsub_rn(gi.maxy, gl.miny) > L || __fsub_rn(gl.maxy, gi.miny) > L);
        const bool far = fary || (farx && yover);
        bool attp = false;
        if (att) {
          float ex = dcx, ey = dcy;
          if (pbc) {
            ex -= L * roundf(ex / L);
            ey -= L * roundf(ey / L);
          }
          const float ra = rr + cp.l0 + mm;
          attp = ex * ex + ey * ey <= ra * ra;
        }
        pflags = (near ? 1u : 0u) | (far ? 2u : 0u) | (attp ? 4u : 0u);
      }
    }
    unsigned pm = __ballot_sync(kFull, pflags != 0u);
    while (pm) {
    const int src = __ffs(pm) - 1;
    pm &= pm - 1u;
    if constexpr (TEAM > 1) {
      // every TEAM-th passing neighbour, in list order, is this warp's
      const bool mine = ordinal % TEAM == team;
      ++ordinal;
      if (!mine) continue;
    }
    const unsigned fl = __shfl_sync(kFull, pflags, src);
    const unsigned jx = __shfl_sync(kFull, jvoff, src), jy = __shfl_sync(kFull, jnv, src);
    const bool near = fl & 1u, far = fl & 2u, attp = fl & 4u;
    Geom2D gj;
    gj.cx = __shfl_sync(kFull, gl.cx, src);
    gj.cy = __shfl_sync(kFull, gl.cy, src);
    gj.R = __shfl_sync(kFull, gl.R, src);
    gj.area = 0.0f;
    gj.minx = __shfl_sync(kFull, gl.minx, src);
    gj.maxx = __shfl_sync(kFull, gl.maxx, src);
    gj.miny = __shfl_sync(kFull, gl.miny, src);
    gj.maxy = __shfl_sync(kFull, gl.maxy, src);
    const float mm = kRelMargin * (gi.R + gj.R) +
                     kAbsMargin * (fabsf(gi.cx) + fabsf(gi.cy) + fabsf(gj.cx) + fabsf(gj.cy));

    unsigned cm[S], am[S];
    int code[S];
    bool anyc = false, anya = false, anyx = false;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      cm[s] = am[s] = 0u;
      code[s] = kNotCandidate;
      if (32 * s >= n) continue;  // empty slot (uniform over the warp)
      const int k = lane + 32 * s;
      bool ac = false;
      if (k < n) {
        if (!sf[k]) code[s] = vertex_candidate(vx[s], vy[s], gj, near, far, L);
        if (attp) {
          float ex = gj.cx - vx[s], ey = gj.cy - vy[s];
          if (pbc) {
            ex -= L * roundf(ex / L);
            ey -= L * roundf(ey / L);
          }
          const float ra = gj.R + cp.l0 + mm;
          ac = ex * ex + ey * ey <= ra * ra;
        }
      }
      cm[s] = __ballot_sync(kFull, code[s] == kCandidate);
      anyc |= cm[s] != 0u;
      anyx |= __any_sync(kFull, code[s] >= kCheckY);
      if (att) {
        am[s] = __ballot_sync(kFull, ac);
        anya |= am[s] != 0u;
      }
    }
    if (!anyc && !anya && !anyx) continue;
    const int nj = (int)jy;
    const float2 *pj = a.pos_in + jx;
    if (anyx) {
      // kCheckY points are candidates only if a ring vertex has y offset
      // exactly -L; kCheckX points only if one has x offset within 8 ulp(L)
      // of L.  One point at a time, the lanes scan the ring.
      const float win = 8.0f * __int_as_float(__float_as_int(L) & 0x7f800000) * 0x1p-23f;
      float px[S], py[S];
#pragma unroll
      for (int s2 = 0; s2 < S; ++s2) {
        const int e = lane + 32 * s2;
        const float2 p = e < nj ? pj[e] : make_float2(0.0f, 0.0f);
        px[s2] = p.x;
        py[s2] = p.y;
      }
#pragma unroll
      for (int s = 0; s < S; ++s) {
        unsigned my = __ballot_sync(kFull, code[s] == kCheckY);
        unsigned mx = __ballot_sync(kFull, code[s] == kCheckX);
        while (my) {
          const int l = __ffs(my) - 1;
          my &= my - 1u;
          const float Y = __shfl_sync(kFull, vy[s], l);
          bool hit = false;
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2)
            hit |= lane + 32 * s2 < nj && __fsub_rn(Y, py[s2]) == -L;
          if (__ballot_sync(kFull, hit)) cm[s] |= 1u << l;
        }
        while (mx) {
          const int l = __ffs(mx) - 1;
          mx &= mx - 1u;
          const float X = __shfl_sync(kFull, vx[s], l);
          bool hit = false;
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2)
            hit |= lane + 32 * s2 < nj && fabsf(__fsub_rn(__fsub_rn(X, px[s2]), L)) <= win;
          if (__ballot_sync(kFull, hit)) cm[s] |= 1u << l;
        }
        anyc |= cm[s] != 0u;
      }
      if (!anyc && !anya) continue;
    }

    if (anya) {
      // stage the neighbour's ring for the per-vertex attraction loops
      for (int k = lane; k < nj; k += 32) {
        const float2 v = pj[k];
        nxs[k] = v.x;
        nys[k] = v.y;
      }
      __syncwarp();
      // AttractionForceUpdate (Cell2D_kernel.cl:251-267)
      const float kat = T.Kat / (float)n;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        if (!((am[s] >> lane) & 1u)) continue;
        for (int v = 0; v < nj; ++v) {
          float rx = nxs[v] - vx[s], ry = nys[v] - vy[s];
          if (pbc) {
            rx -= L * roundf(rx / L);
            ry -= L * roundf(ry / L);
          }
          const float dist = sqrtf(rx * rx + ry * ry);
          if (dist < cp.l0) {
            const float ftmp = kat * dist / cp.l0;
            float ux, uy;
            normalize2(rx, ry, ux, uy);
            fx[s] += ftmp * ux;
            fy[s] += ftmp * uy;
          }
        }
      }
    }
    if (anyc) {
      // RepulsionForceUpdate containment (Cell2D_kernel.cl:166-202):
      // lanes take the edges (P_e, P_{e-1}) of the neighbour, held in
      // registers for all candidates; a ballot gives the crossing parity.
      // Edges can be shifted only for "far" pairs, so the plain test is
      // used otherwise.
      float ex[S], ey[S], qx[S], qy[S];
#pragma unroll
      for (int s2 = 0; s2 < S; ++s2) {
        const int e = lane + 32 * s2;
        ex[s2] = ey[s2] = qx[s2] = qy[s2] = 0.0f;
        if (e < nj) {
          const float2 p = pj[e], pp = pj[e == 0 ? nj - 1 : e - 1];
          ex[s2] = p.x;
          ey[s2] = p.y;
          qx[s2] = pp.x;
          qy[s2] = pp.y;
        }
      }
      // one loop over the candidates of every slot (the slot's coordinates
      // picked by selects): the edge tests are compiled once, not per slot
      int s = 0;
      unsigned msk = cm[0];
      for (;;) {
        while (!msk && s + 1 < S) {
          ++s;
#pragma unroll
          for (int t = 1; t < S; ++t)
            if (s == t) msk = cm[t];
        }
        if (!msk) break;
        {
          const int l = __ffs(msk) - 1;
          msk &= msk - 1u;
          float xs = vx[0], ys = vy[0];
#pragma unroll
          for (int t = 1; t < S; ++t)
            if (s == t) {
              xs = vx[t];
              ys = vy[t];
            }
          const float X = __shfl_sync(kFull, xs, l), Y = __shfl_sync(kFull, ys, l);
          unsigned par = 0u;
          if (far) {
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2)
              if (lane + 32 * s2 < nj)
                par ^= edge_crosses(X, Y, ex[s2], ey[s2], qx[s2], qy[s2], true, L);
          } else {
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2)
              if (lane + 32 * s2 < nj)
                par ^= edge_crosses(X, Y, ex[s2], ey[s2], qx[s2], qy[s2], false, L);
          }
          const unsigned bal = __ballot_sync(kFull, par != 0u);
          if ((__popc(bal) & 1) && lane == 0) sf[l + 32 * s] = 1;
        }
      }
    }
    __syncwarp();
    }
  }

  if constexpr (TEAM > 1) {
    __syncthreads();  // every warp's flags are in sf
    if (team != 0) return;
  }

  // -- repulsion force toward the own centre (Cell2D_kernel.cl:205-219)
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int k = lane + 32 * s;
    if (k < n && sf[k]) {
      float dx = gi.cx - vx[s], dy = gi.cy - vy[s];
      // d -= L*round(d/L); for |d| <= 0.49 L the rounded quotient is 0
      if (pbc && fabsf(dx) > 0.49f * L) dx -= L * roundf(dx / L);
      if (pbc && fabsf(dy) > 0.49f * L) dy -= L * roundf(dy / L);
      const float d2 = dx * dx + dy * dy;
      const float dist = sqrtf(d2);
      const float xij = dist * cp.inv_2r0;
      const float ftmp = T.Kre * (1.0f - xij);
      // normalize(d), with the zero vector mapped to itself
      const float inv = d2 == 0.0f ? 1.0f : 1.0f / dist;
      fx[s] += 0.5f * ftmp * (dx * inv);
      fy[s] += 0.5f * ftmp * (dy * inv);
    }
  }

  // -- Euler update (EulerUpdate, Cell2D_kernel.cl:279) and outputs
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int k = lane + 32 * s;
    if (k < n) {
      const float nxv = __fadd_rn(vx[s], __fmul_rn(fx[s], a.dt));
      const float nyv = __fadd_rn(vy[s], __fmul_rn(fy[s], a.dt));
      a.pos_out[cp.voff + k] = make_float2(nxv, nyv);
      if (a.force_out && write_out) a.force_out[cp.voff + k] = make_float2(fx[s], fy[s]);
      if (a.flags_out && write_out) a.flags_out[cp.voff + k] = sf[k];
      sx[k] = nxv;
      sy[k] = nyv;
    }
  }
  __syncwarp();

  // -- epilogue: geometry of the new positions for the next step
  const Geom2D g = ring_geom(sx, sy, n, lane);
  if (lane == 0) {
    a.geom_out[c] = g;
    if (!(isfinite(g.cx) && isfinite(g.cy) && isfinite(g.R))) atomicOr(a.err, 1);
    // the list stays valid while no cell moved more than skin/2 since the
    // rebuild (no lists, geom0 null: the resident run scans every cell)
    if (a.geom0) {
      const Geom2D g0 = a.geom0[c];
      const float dc =
          sqrtf((g.cx - g0.cx) * (g.cx - g0.cx) + (g.cy - g0.cy) * (g.cy - g0.cy));
      float d = dc + fmaxf(0.0f, g.R - g0.R);
      d = fmaxf(d, fmaxf(fabsf(g.minx - g0.minx), fabsf(g.maxx - g0.maxx)));
      d = fmaxf(d, fmaxf(fabsf(g.miny - g0.miny), fabsf(g.maxy - g0.maxy)));
      if (!(d <= 0.5f * T.skin)) atomicOr(a.stale + tid, 1);
    }
  }
}

// Static schedule: warp w of block b takes cell b*W + w.
template <int S, int W, int OCC, bool ATT>
__global__ void __launch_bounds__(W * 32, (StepOcc<S, W, OCC>::kBlocks))
    k2d_step(Step2DArgs a) {
  constexpr int M = 32 * S;
  __shared__ float sh_x[W][M], sh_y[W][M], sh_nx[W][M], sh_ny[W][M];
  __shared__ unsigned char sh_f[W][M];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * W + w;
  if (i >= a.ncells) return;
  const int c = a.order ? a.order[i] : i;
  step_cell<S, ATT>(a, c, lane, sh_x[w], sh_y[w], sh_nx[w], sh_ny[w], sh_f[w]);
}

// Dynamic schedule: a grid of exactly the resident blocks whose warps take
// the next cell from a counter until none is left.  The work per cell varies
// with its neighbours, so no warp idles while cells remain and no block is
// held resident by one slow warp.  The last warp to finish resets the two
// counters (next cell, finished warps) for the next launch.
template <int S, int W, int OCC, bool ATT>
__global__ void __launch_bounds__(W * 32, (StepOcc<S, W, OCC>::kBlocks))
    k2d_step_dyn(Step2DArgs a) {
  constexpr int M = 32 * S;
  __shared__ float sh_x[W][M], sh_y[W][M], sh_nx[W][M], sh_ny[W][M];
  __shared__ unsigned char sh_f[W][M];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    int i = 0;
    if (lane == 0) i = atomicAdd(a.sched, 1);
    i = __shfl_sync(kFull, i, 0);
    if (i >= a.ncells) break;
    const int c = a.order ? a.order[i] : i;
    step_cell<S, ATT>(a, c, lane, sh_x[w], sh_y[w], sh_nx[w], sh_ny[w], sh_f[w]);
    __syncwarp();
  }
  if (lane == 0) {
    const int warps = (int)gridDim.x * W;
    if (atomicAdd(a.sched + 1, 1) == warps - 1) {
      atomicExch(a.sched, 0);
      atomicExch(a.sched + 1, 0);
    }
  }
}

// Resident run of small tissues: one block per tissue copies the tissue's
// constants, positions and geometry into shared memory (cell ids, vertex
// offsets and the tissue id made local), runs nsteps steps there -- its warps
// take the tissue's cells in turn, the block synchronizes between steps --
// and writes the positions and geometry back.  The stale flag is held set,
// so every cell screens the whole tissue in ascending order: the pairs and
// their order are those of the neighbour lists, whose pruning is exact, and
// the results are the graph path's bit for bit.  For tissues too small to
// fill the GPU, where a step of the graph path waits on launch and global
// memory latency.
template <int S, bool ATT>
__global__ void __launch_bounds__(kResidentWarps * 32)
    k2d_run_resident(Resident2DArgs r) {
  constexpr int M = 32 * S, W = kResidentWarps;
  __shared__ float sh_x[W][M], sh_y[W][M], sh_nx[W][M], sh_ny[W][M];
  __shared__ unsigned char sh_f[W][M];
  __shared__ int sh_stale;
  extern __shared__ __align__(16) unsigned char res_smem[];
  Tissue2D *ts = reinterpret_cast<Tissue2D *>(res_smem);
  Cell2D *cs = reinterpret_cast<Cell2D *>(res_smem + 128);
  Geom2D *gs0 = reinterpret_cast<Geom2D *>(cs + r.ncmax);
  Geom2D *gs1 = gs0 + r.ncmax;
  float2 *ps0 = reinterpret_cast<float2 *>(gs1 + r.ncmax);
  float2 *ps1 = ps0 + r.nvmax;
  const int t = blockIdx.x;
  const Tissue2D T = r.a.tissues[t];
  const int c0 = T.cell_begin, nc = T.cell_end - T.cell_begin;
  const uint32_t v0 = r.a.cells[c0].voff;
  const int nvt = (int)(r.a.cells[c0 + nc - 1].voff + r.a.cells[c0 + nc - 1].nv - v0);
  for (int i = threadIdx.x; i < nc; i += blockDim.x) {
    Cell2D cp = r.a.cells[c0 + i];
    cp.voff -= v0;
    cp.tissue = 0;
    cs[i] = cp;
    gs0[i] = r.geom[c0 + i];
  }
  for (int i = threadIdx.x; i < nvt; i += blockDim.x) ps0[i] = r.pos[v0 + i];
  if (threadIdx.x == 0) {
    Tissue2D tl = T;
    tl.cell_begin = 0;
    tl.cell_end = nc;
    *ts = tl;
    sh_stale = 1;  // screen the whole tissue at every step
  }
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Step2DArgs a = r.a;
  a.cells = cs;
  a.tissues = ts;
  a.geom0 = nullptr;  // no lists: nothing to check or read
  a.nn = nullptr;
  a.stale = &sh_stale;
  a.step_index = 0;
  a.order = nullptr;
  float2 *pin = ps0, *pout = ps1;
  Geom2D *gin = gs0, *gout = gs1;
  for (int step = 0; step < r.nsteps; ++step) {
    const bool last = step == r.nsteps - 1;
    a.pos_in = pin;
    a.pos_out = pout;
    a.geom_in = gin;
    a.geom_out = gout;
    a.force_out = last && r.a.force_out ? r.a.force_out + v0 : nullptr;
    a.flags_out = last && r.a.flags_out ? r.a.flags_out + v0 : nullptr;
    for (int c = w; c < nc; c += W)
      step_cell<S, ATT>(a, c, lane, sh_x[w], sh_y[w], sh_nx[w], sh_ny[w], sh_f[w]);
    __syncthreads();
    float2 *tp = pin;
    pin = pout;
    pout = tp;
    Geom2D *tg = gin;
    gin = gout;
    gout = tg;
  }
  for (int i = threadIdx.x; i < nvt; i += blockDim.x) r.pos[v0 + i] = pin[i];
  for (int i = threadIdx.x; i < nc; i += blockDim.x) r.geom[c0 + i] = gin[i];
}

template <int S, bool ATT>
cudaError_t launch_resident_sa(const Resident2DArgs &r, int ntissues, cudaStream_t s) {
  const size_t bytes = resident2d_smem_bytes(r.ncmax, r.nvmax);
  // the dynamic shared-memory limit of the kernel, raised once to what any
  // resident run may use
  static const cudaError_t attr = cudaFuncSetAttribute(
      k2d_run_resident<S, ATT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)resident2d_smem_bytes(kResidentMaxCells, kResidentMaxVerts));
  if (attr != cudaSuccess) return attr;
  k2d_run_resident<S, ATT><<<ntissues, kResidentWarps * 32, bytes, s>>>(r);
  return cudaGetLastError();
}

template <int S>
cudaError_t launch_resident_s(const Resident2DArgs &r, int ntissues, int variant, cudaStream_t s) {
  return (variant & kStepVariantAttraction) ? launch_resident_sa<S, true>(r, ntissues, s)
                                            : launch_resident_sa<S, false>(r, ntissues, s);
}

// Team schedule (no attraction): TEAM warps per block step one cell
// together (see step_cell), the blocks taking cells from the counter.  For
// batches too small to fill the GPU with one warp per cell, where a cell's
// step is a long chain of dependent loads: its neighbours are split over
// more warps.  The last block to finish resets the counters.
template <int S, int TEAM, int OCC>
__global__ void __launch_bounds__(TEAM * 32, (StepOcc<S, TEAM, OCC>::kBlocks))
    k2d_step_team(Step2DArgs a) {
  constexpr int M = 32 * S;
  __shared__ float sh_x[M], sh_y[M];
  __shared__ unsigned char sh_f[M];
  __shared__ int sh_i;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) sh_i = atomicAdd(a.sched, 1);
    __syncthreads();
    const int i = sh_i;
    __syncthreads();  // read by every thread before the next fetch
    if (i >= a.ncells) break;
    const int c = a.order ? a.order[i] : i;
    step_cell<S, false, TEAM>(a, c, lane, sh_x, sh_y, nullptr, nullptr, sh_f, w);
  }
  if (threadIdx.x == 0 && atomicAdd(a.sched + 1, 1) == (int)gridDim.x - 1) {
    atomicExch(a.sched, 0);
    atomicExch(a.sched + 1, 0);
  }
}

template <int S, int TEAM, int OCC>
cudaError_t launch_team_so(const Step2DArgs &a, cudaStream_t s) {
  static const int per_sm_sms = [] {
    int per = 0, dev = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k2d_step_team<S, TEAM, OCC>,
                                                      TEAM * 32, 0) != cudaSuccess ||
        cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return 0;
    return (per < 1 ? 1 : per) * (sms < 1 ? 1 : sms);
  }();
  if (per_sm_sms <= 0) return cudaErrorUnknown;
  const int grid = a.ncells < per_sm_sms ? a.ncells : per_sm_sms;
  if (grid <= 0) return cudaSuccess;
  k2d_step_team<S, TEAM, OCC><<<grid, TEAM * 32, 0, s>>>(a);
  return cudaGetLastError();
}

// variant bit 0: register cap for occupancy (the team is always 4 warps)
template <int S>
cudaError_t launch_team_s(const Step2DArgs &a, int variant, cudaStream_t s) {
  return (variant & 1) ? launch_team_so<S, 4, 1>(a, s) : launch_team_so<S, 4, 0>(a, s);
}

template <int S, int W, int OCC, bool ATT>
cudaError_t launch_step_sw(const Step2DArgs &a, bool dyn, cudaStream_t s) {
  if (dyn && a.sched) {
    // resident blocks per SM of this variant and the device's SM count,
    // found once (a function-local static: initialised once even when
    // several host threads launch at the same time)
    struct Resident {
      int per_sm, sms;
      cudaError_t err;
    };
    static const Resident res = [] {
      Resident r{0, 0, cudaSuccess};
      r.err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &r.per_sm, k2d_step_dyn<S, W, OCC, ATT>, W * 32, 0);
      int dev = 0;
      if (r.err == cudaSuccess) r.err = cudaGetDevice(&dev);
      if (r.err == cudaSuccess)
        r.err = cudaDeviceGetAttribute(&r.sms, cudaDevAttrMultiProcessorCount, dev);
      if (r.per_sm < 1) r.per_sm = 1;
      if (r.sms < 1) r.sms = 1;
      return r;
    }();
    if (res.err != cudaSuccess) return res.err;
    const int need = (a.ncells + W - 1) / W;
    const int grid = need < res.per_sm * res.sms ? need : res.per_sm * res.sms;
    k2d_step_dyn<S, W, OCC, ATT><<<grid, W * 32, 0, s>>>(a);
    return cudaGetLastError();
  }
  const int grid = (a.ncells + W - 1) / W;
  k2d_step<S, W, OCC, ATT><<<grid, W * 32, 0, s>>>(a);
  return cudaGetLastError();
}

template <int S, int OCC, bool ATT>
cudaError_t launch_step_so(const Step2DArgs &a, int warps, bool dyn, cudaStream_t s) {
  // 16 warps of 8 slots would exceed the static shared-memory limit
  if (warps == 4) return launch_step_sw<S, 4, OCC, ATT>(a, dyn, s);
  if (warps == 16 && S <= 4) return launch_step_sw<S, (S <= 4 ? 16 : 8), OCC, ATT>(a, dyn, s);
  return launch_step_sw<S, 8, OCC, ATT>(a, dyn, s);
}

// variant bit 0: register cap for occupancy; bit 1: dynamic schedule (bit 2,
// attraction compiled in, is ATT)
template <int S, bool ATT>
cudaError_t launch_step_sa(const Step2DArgs &a, int warps, int variant, cudaStream_t s) {
  const bool dyn = (variant & 2) != 0;
  return (variant & 1) ? launch_step_so<S, 1, ATT>(a, warps, dyn, s)
                       : launch_step_so<S, 0, ATT>(a, warps, dyn, s);
}
template <int S>
cudaError_t launch_step_s(const Step2DArgs &a, int warps, int variant, cudaStream_t s) {
  return (variant & kStepVariantAttraction) ? launch_step_sa<S, true>(a, warps, variant, s)
                                            : launch_step_sa<S, false>(a, warps, variant, s);
}

} // namespace
} // namespace dpm
