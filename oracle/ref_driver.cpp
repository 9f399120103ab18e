// C entry points that drive the reference's own DPM::Tissue2D / DPM::Tissue3D
// (compiled unmodified against the CPU OpenCL shim) for the tests.
//
// Test infrastructure only: these run the reference's public C++ API exactly
// as its demo drivers do (test2D.cpp:8-48, test3D.cpp:8-49) -- construct cells,
// set spring constants, build a tissue, optionally Disperse, call
// CLEulerUpdate -- and copy the resulting state out into flat arrays.
//
// The reference opens "./shaders/*.cl" relative to the working directory
// (src/Tissue2D.cpp:38, src/Tissue3D.cpp:36); every entry point that builds a
// tissue takes the reference root and changes into it for the duration of the
// call.
#include "Tissue.hpp"
#include "cell.hpp"
#include "readKernel.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <iostream>
#include <sstream>
#include <string>
#include <unistd.h>
#include <vector>

namespace {

std::string g_last_error;

struct CwdGuard {
  std::string old;
  bool ok = false;
  explicit CwdGuard(const char *dir) {
    char buf[4096];
    if (getcwd(buf, sizeof(buf))) old = buf;
    ok = dir && chdir(dir) == 0;
  }
  ~CwdGuard() {
    if (!old.empty()) {
      int rc = chdir(old.c_str());
      (void)rc;
    }
  }
};

// Silences the reference's std::cout timing lines for the duration of a call.
struct CoutMute {
  std::streambuf *old;
  std::ostringstream sink;
  CoutMute() : old(std::cout.rdbuf(sink.rdbuf())) {}
  ~CoutMute() { std::cout.rdbuf(old); }
};

} // namespace

extern "C" {

const char *ref_last_error(void) { return g_last_error.c_str(); }

// Geometry of one reference Cell2D(x0, y0, calA, nv, r0) (src/cell.cpp:12-33).
// verts_out: 2*nv floats; scalars: a0, l0, calA0.
int ref2d_cell(float x0, float y0, float calA, unsigned nv, float r0,
               float *verts_out, float *a0, float *l0, float *calA0) {
  DPM::Cell2D c(x0, y0, calA, nv, r0);
  for (unsigned i = 0; i < nv; ++i) {
    verts_out[2 * i] = c.Verticies[i][0];
    verts_out[2 * i + 1] = c.Verticies[i][1];
  }
  *a0 = c.a0;
  *l0 = c.l0;
  *calA0 = c.calA0;
  return 0;
}

// Runs the reference 2D tissue.  Per cell: centre (x0, y0), calA, nv, r0,
// Ka, Kl, Kb.  verts_in (2*sum(nv) floats, cell-major) replaces the ctor's
// regular polygons when non-NULL.  When disperse != 0, srand48(seed) then
// Tissue2D::Disperse().  Outputs: final vertices and last-step forces
// (2*sum(nv) each) and the box size L.
int ref2d_run(const char *refdir, int ncells, const float *x0, const float *y0,
              const float *calA, const unsigned *nv, const float *r0,
              const float *Ka, const float *Kl, const float *Kb,
              const float *verts_in, float phi0, float Kre, float Kat,
              int disperse, long seed, int nsteps, float dt, float *verts_out,
              float *forces_out, float *L_out) {
  try {
    CwdGuard cwd(refdir);
    if (!cwd.ok) {
      g_last_error = "cannot enter reference directory";
      return 1;
    }
    std::vector<DPM::Cell2D> cells;
    size_t off = 0;
    for (int ci = 0; ci < ncells; ++ci) {
      DPM::Cell2D c(x0[ci], y0[ci], calA[ci], nv[ci], r0[ci]);
      c.Ka = Ka[ci];
      c.Kl = Kl[ci];
      c.Kb = Kb[ci];
      c.Ks = 0.0f;
      if (verts_in) {
        for (unsigned vi = 0; vi < nv[ci]; ++vi) {
          c.Verticies[vi][0] = verts_in[2 * (off + vi)];
          c.Verticies[vi][1] = verts_in[2 * (off + vi) + 1];
        }
      }
      off += nv[ci];
      cells.push_back(c);
    }
    CoutMute mute;
    DPM::Tissue2D T(cells, phi0);
    T.Kre = Kre;
    T.Kat = Kat;
    if (disperse) {
      srand48(seed);
      T.Disperse();
    }
    if (nsteps > 0) T.CLEulerUpdate(nsteps, dt);
    off = 0;
    for (int ci = 0; ci < ncells; ++ci) {
      for (unsigned vi = 0; vi < T.cells[ci].NV; ++vi) {
        verts_out[2 * (off + vi)] = T.cells[ci].Verticies[vi][0];
        verts_out[2 * (off + vi) + 1] = T.cells[ci].Verticies[vi][1];
        forces_out[2 * (off + vi)] = T.cells[ci].Forces[vi][0];
        forces_out[2 * (off + vi) + 1] = T.cells[ci].Forces[vi][1];
      }
      off += T.cells[ci].NV;
    }
    *L_out = T.L;
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return 2;
  }
}

// Geometry of one reference Cell3D(start, calA, r0) (src/cell.cpp:62-158).
// verts_out: 3*162 floats, faces_out: 3*320 uints; scalars v0, sa0, a0,
// Volume, SurfaceArea.
int ref3d_cell(const float *start, float calA, float r0, float *verts_out,
               unsigned *faces_out, float *v0, float *sa0, float *a0,
               float *volume, float *surface_area) {
  DPM::Cell3D c({start[0], start[1], start[2]}, calA, r0);
  for (unsigned i = 0; i < DPM::Cell3D::NV; ++i)
    for (int k = 0; k < 3; ++k) verts_out[3 * i + k] = c.Verts[i][k];
  for (unsigned f = 0; f < DPM::Cell3D::NF; ++f)
    for (int k = 0; k < 3; ++k) faces_out[3 * f + k] = c.Faces[f][k];
  *v0 = c.v0;
  *sa0 = c.sa0;
  *a0 = c.a0;
  *volume = c.Volume;
  *surface_area = c.SurfaceArea;
  return 0;
}

// Runs the reference 3D tissue.  Per cell: start (3 floats), calA, r0, Kv,
// Ka, Ks.  verts_in (3*162 floats per cell) replaces the ctor mesh when
// non-NULL.  Outputs: final vertices and last-step forces (3*162 per cell),
// the host-side Volume and SurfaceArea per cell after the run, and L.
int ref3d_run(const char *refdir, int ncells, const float *start,
              const float *calA, const float *r0, const float *Kv,
              const float *Ka, const float *Ks, const float *verts_in,
              float phi0, float Kre, int disperse, long seed, int nsteps,
              float dt, float *verts_out, float *forces_out, float *volume_out,
              float *sa_out, float *L_out) {
  try {
    CwdGuard cwd(refdir);
    if (!cwd.ok) {
      g_last_error = "cannot enter reference directory";
      return 1;
    }
    const unsigned NV = DPM::Cell3D::NV;
    std::vector<DPM::Cell3D> cells;
    for (int ci = 0; ci < ncells; ++ci) {
      DPM::Cell3D c({start[3 * ci], start[3 * ci + 1], start[3 * ci + 2]},
                    calA[ci], r0[ci]);
      c.Kv = Kv[ci];
      c.Ka = Ka[ci];
      c.Ks = Ks[ci];
      if (verts_in) {
        for (unsigned vi = 0; vi < NV; ++vi)
          for (int k = 0; k < 3; ++k)
            c.Verts[vi][k] = verts_in[3 * (ci * NV + vi) + k];
      }
      cells.push_back(c);
    }
    CoutMute mute;
    DPM::Tissue3D T(cells, phi0);
    T.Kre = Kre;
    T.Kat = 0.0f;
    if (disperse) {
      srand48(seed);
      T.Disperse2D();
    }
    if (nsteps > 0) T.CLEulerUpdate(nsteps, dt);
    for (int ci = 0; ci < ncells; ++ci) {
      for (unsigned vi = 0; vi < NV; ++vi)
        for (int k = 0; k < 3; ++k) {
          verts_out[3 * (ci * NV + vi) + k] = T.Cells[ci].Verts[vi][k];
          forces_out[3 * (ci * NV + vi) + k] = T.Cells[ci].Forces[vi][k];
        }
      volume_out[ci] = T.Cells[ci].GetVolume();
      sa_out[ci] = T.Cells[ci].GetSurfaceArea();
    }
    *L_out = T.L;
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return 2;
  }
}

// Runs the reference's AllVertAttraction kernel (shaders/Cell3D_Kernel.cl:
// 313-364), which its own step loop never enqueues, once on the given
// vertices (162 per cell), with the OpenCL calls its host code makes for the
// other 3D kernels (src/Tissue3D.cpp:199-426): build, buffers, setArg,
// NDRange(NV, NCELLS), read back.  forces_out receives the forces, which
// start from zero.
int ref3d_attraction(const char *refdir, int ncells, const float *xyz, const float *l0,
                     float L, int pbc, float Kat, float *forces_out) {
  try {
    CwdGuard cwd(refdir);
    if (!cwd.ok) {
      g_last_error = "cannot enter reference directory";
      return 1;
    }
    const unsigned NV = DPM::Cell3D::NV;
    const size_t n = (size_t)ncells * NV;
    cl::Device device = cl::Device::getDefault();
    cl::Context context({device});
    cl::Program program(context, readKernelSource("shaders/Cell3D_Kernel.cl"));
    if (program.build({device}, "-cl-opt-disable -Werror") != CL_SUCCESS) {
      g_last_error = "kernel build failed";
      return 2;
    }
    std::vector<cl_float3> verts(n), forces(n);
    for (size_t i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) {
        verts[i].s[k] = xyz[3 * i + k];
        forces[i].s[k] = 0.0f;
      }
    std::vector<float> l0v(l0, l0 + ncells);
    cl::Buffer gpuVerts(context, CL_MEM_READ_ONLY | CL_MEM_COPY_HOST_PTR,
                        sizeof(cl_float3) * n, verts.data());
    cl::Buffer gpuForces(context, CL_MEM_READ_WRITE | CL_MEM_COPY_HOST_PTR,
                         sizeof(cl_float3) * n, forces.data());
    cl::Buffer gpul0(context, CL_MEM_READ_ONLY | CL_MEM_COPY_HOST_PTR,
                     sizeof(float) * ncells, l0v.data());
    cl_int err = CL_SUCCESS;
    cl::Kernel kernel(program, "AllVertAttraction", &err);
    if (err != CL_SUCCESS) {
      g_last_error = "no AllVertAttraction kernel";
      return 3;
    }
    kernel.setArg(0, gpuVerts);
    kernel.setArg(1, gpuForces);
    kernel.setArg(2, gpul0);
    kernel.setArg(3, L);
    kernel.setArg(4, ncells);
    kernel.setArg(5, pbc);
    kernel.setArg(6, Kat);
    cl::CommandQueue queue(context, device, 0, &err);
    err = queue.enqueueNDRangeKernel(kernel, cl::NullRange, cl::NDRange(NV, ncells));
    if (err == CL_SUCCESS)
      err = queue.enqueueReadBuffer(gpuForces, CL_TRUE, 0, sizeof(cl_float3) * n, forces.data());
    if (err != CL_SUCCESS) {
      g_last_error = "AllVertAttraction launch failed";
      return 4;
    }
    for (size_t i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) forces_out[3 * i + k] = forces[i].s[k];
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return 2;
  }
}

} // extern "C"
