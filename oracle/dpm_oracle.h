/*
 * CPU oracle for the Deformable Particle Model time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (sudo-shaka/OpenCL_DPM), used by the tests as the checker, by the
 * smoke check, and by the benchmark's CPU baseline.  The product never links,
 * loads or calls it.
 *
 * Pinning: every function here is checked against the reference itself,
 * compiled on the CPU from its own sources (oracle/build_ref.py), and against
 * golden vectors generated from that build (tests/golden/).
 *
 * Layout: 2D vertices are ragged and cell-major, xy interleaved:
 * cell c's vertex v is at xy[2*(off[c]+v)].  3D vertices are cell-major with
 * a shared face table: cell c's vertex v is at xyz[3*(c*nv+v)].
 */
#ifndef DPM_ORACLE_H
#define DPM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- geometry (src/cell.cpp) ---- */
void orc_cell2d(float x0, float y0, float calA, unsigned nv, float r0,
                float *xy, float *a0, float *l0, float *calA0);
float orc_area2d(const float *xy, unsigned nv);
float orc_box2d(const float *areas, int ncells, float phi0);
int orc_icosphere_counts(int level, int *nv, int *nf);
int orc_icosphere(int level, float *xyz, unsigned *faces);
void orc_cell3d(const float *start, float calA, float r0, int level,
                float *xyz, unsigned *faces, float *v0, float *sa0, float *a0);
float orc_volume3d(const float *xyz, const unsigned *faces, int nf);
float orc_surface3d(const float *xyz, const unsigned *faces, int nf);
float orc_box3d(const float *v0, int ncells, float phi0);
float orc_l0_3d(float a0);

/* ---- 2D step loop (src/Tissue2D.cpp:116-241, shaders/Cell2D_kernel.cl) ---- */
typedef struct {
  int ncells;
  const unsigned *nv;  /* [ncells] */
  const unsigned *off; /* [ncells] first vertex of each cell */
  const float *Ka, *Kl, *Kb, *a0, *l0, *r0; /* [ncells] */
  int pbc;
  float L, Kre, Kat;
} orc_tissue2d;

/* Runs nsteps steps in place on xy; F receives the forces of the last step
 * (before its Euler update), as Tissue2D::CLEulerUpdate returns them.
 * contained (optional, [total vertices]) receives the last step's repulsion
 * containment flags.  nthreads <= 0 uses the OpenMP default. */
int orc_run2d(const orc_tissue2d *t, float dt, int nsteps, float *xy, float *F,
              unsigned char *contained, int nthreads);

/* ---- 3D step loop (src/Tissue3D.cpp:118-522, shaders/Cell3D_Kernel.cl) ---- */
typedef struct {
  int ncells, nv, nf;
  const unsigned *faces; /* [nf*3], shared by all cells */
  const float *Kv, *Ka, *Ks, *v0, *a0, *l0; /* [ncells] */
  const float *Kb; /* [ncells] triangle-bending stiffness (extension), or NULL */
  const float *adh; /* [ncells] adhesion range (extension), or NULL = 2*l0 */
  int pbc;
  float L, Kre;
  float Kat; /* AllVertAttraction strength; 0 = off (the reference's host loop
              * never enqueues that kernel) */
} orc_tissue3d;

/* Runs nsteps in place on xyz; F receives the last step's forces (the
 * reference reads them after Euler, which does not clear them).  wn
 * (optional, [ncells*nv]) receives the number of other cells whose winding
 * number passed the threshold for each vertex in the last step. */
int orc_run3d(const orc_tissue3d *t, float dt, int nsteps, float *xyz, float *F,
              unsigned char *wn, int nthreads);

/* AllVertAttraction (shaders/Cell3D_Kernel.cl:313-364) on xyz ([ncells*nv]
 * vertices), added into F, each vertex gathering its pairs over the other
 * cells in ascending cell and vertex order. */
void orc_attraction3d(int ncells, int nv, const float *xyz, const float *l0, float L,
                      int pbc, float Kat, float *F);

/* ---- initial dispersion (src/Tissue2D.cpp:42-114, src/Tissue3D.cpp:40-116) ---- */
void orc_disperse2d(int ncells, const unsigned *nv, const unsigned *off,
                    const float *r0, float L, long seed, float *xy);
void orc_disperse3d(int ncells, int nv, const float *r0, float L, long seed,
                    float *xyz);

/* ---- FP64 diagnostics (project-defined; the reference has no energy) ---- */
void orc_diag2d(const orc_tissue2d *t, const float *xy, double *area,
                double *perim, double *energy);
void orc_diag3d(const orc_tissue3d *t, const float *xyz, double *volume,
                double *area, double *energy);
/* FP64 energy of the 3D triangle-bending term (extension) and its gradient
 * by central differences (step h), for checking the bending force. */
double orc_bend_energy3d(int nv, int nf, const unsigned *faces, double kb,
                         const double *xyz);

#ifdef __cplusplus
}
#endif

#endif
