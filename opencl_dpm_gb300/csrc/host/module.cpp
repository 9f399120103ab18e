// The clDPM Python module: the reference's API (src/DPMWrapper.cpp,
// src/CellWrapper.cpp, src/TissueWrapper.cpp) over the GB300 library.
// Same class, attribute and method names with the same read/write access;
// additions are marked as extensions in their docstrings.
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include "dpm_gb300.h"
#include "dpm_host.hpp"

namespace py = pybind11;

PYBIND11_MODULE(clDPM, m) {
  m.doc() = "Deformable Particle Model on GB300 (sm_103a CUDA)";

  // src/CellWrapper.cpp:22-30
  py::class_<DPM::Cell2D>(m, "Cell2D")
      .def(py::init<float, float, float, unsigned int, float>(), py::arg("x0"), py::arg("y0"),
           py::arg("calA"), py::arg("NV"), py::arg("r0"))
      .def_readwrite("Ka", &DPM::Cell2D::Ka)
      .def_readwrite("Kl", &DPM::Cell2D::Kl)
      .def_readwrite("Kb", &DPM::Cell2D::Kb)
      .def_readwrite("Verts", &DPM::Cell2D::Verticies)
      .def_readwrite("Forces", &DPM::Cell2D::Forces)
      // extensions
      .def_readonly("NV", &DPM::Cell2D::NV, "extension: vertex count")
      .def_readwrite("a0", &DPM::Cell2D::a0, "extension: rest area")
      .def_readwrite("l0", &DPM::Cell2D::l0, "extension: rest edge length")
      .def_readwrite("r0", &DPM::Cell2D::r0, "extension: radius")
      .def_readonly("calA0", &DPM::Cell2D::calA0, "extension: rest shape index")
      .def("GetArea", &DPM::Cell2D::GetArea, "extension: polygon area")
      .def("GetPerim", &DPM::Cell2D::GetPerim, "extension: polygon perimeter");

  // src/TissueWrapper.cpp:19-30
  py::class_<DPM::Tissue2D>(m, "Tissue2D")
      .def(py::init<std::vector<DPM::Cell2D>, float>(), py::arg("cells"), py::arg("phi0"))
      .def_readwrite("Cells", &DPM::Tissue2D::cells)
      .def_readonly("NCELLS", &DPM::Tissue2D::NCELLS)
      .def_readonly("L", &DPM::Tissue2D::L)
      .def_readonly("PBC", &DPM::Tissue2D::PBC)
      .def_readwrite("Kre", &DPM::Tissue2D::Kre)
      .def_readwrite("Kat", &DPM::Tissue2D::Kat)
      .def("CLEulerUpdate", &DPM::Tissue2D::CLEulerUpdate, py::arg("nsteps"), py::arg("dt"))
      .def("Disperse", &DPM::Tissue2D::Disperse, py::arg("device") = true,
           "device (extension): relax on the GPU, bit for bit the host loop; False: host")
      // extensions
      .def("SetPackingFraction", &DPM::Tissue2D::SetPackingFraction,
           "extension: rescale the box and cell centroids to true packing fraction phi")
      .def("GetPackingFraction", &DPM::Tissue2D::GetPackingFraction,
           "extension: sum of cell areas / L^2")
      .def("GetShapeIndices", &DPM::Tissue2D::GetShapeIndices,
           "extension: per-cell P / sqrt(4 pi A)");

  // src/CellWrapper.cpp:7-20
  py::class_<DPM::Cell3D>(m, "Cell3D")
      .def(py::init<std::array<float, 3>, float, float, int>(), py::arg("start"),
           py::arg("calA"), py::arg("r0"), py::arg("level") = 2)
      .def_readwrite("Kv", &DPM::Cell3D::Kv)
      .def_readwrite("Ka", &DPM::Cell3D::Ka)
      .def_readwrite("Ks", &DPM::Cell3D::Ks)
      .def_readwrite("Verts", &DPM::Cell3D::Verts)
      .def("GetVolume", &DPM::Cell3D::GetVolume)
      .def("GetPositions", &DPM::Cell3D::GetPositions)
      .def("GetVesselPositions", &DPM::Cell3D::GetVesselPositions)
      .def("GetFaces", &DPM::Cell3D::GetFaces)
      .def("GetForces", &DPM::Cell3D::GetForces)
      // extensions
      .def_readwrite("Kb", &DPM::Cell3D::Kb, "extension: triangle-bending stiffness")
      .def_readwrite("adh", &DPM::Cell3D::adh,
                     "extension: substrate adhesion range (< 0: 2*l0 as the reference)")
      .def_readwrite("v0", &DPM::Cell3D::v0, "extension: target volume")
      .def_readwrite("a0", &DPM::Cell3D::a0, "extension: target area per face")
      .def_readwrite("sa0", &DPM::Cell3D::sa0, "extension: target surface area")
      .def_readonly("NV", &DPM::Cell3D::NV, "extension: vertices per cell")
      .def_readonly("NF", &DPM::Cell3D::NF, "extension: faces per cell")
      .def_readonly("level", &DPM::Cell3D::level, "extension: subdivision level")
      .def_readonly("Volume", &DPM::Cell3D::Volume)
      .def_readonly("SurfaceArea", &DPM::Cell3D::SurfaceArea)
      .def("GetSurfaceArea", &DPM::Cell3D::GetSurfaceArea, "extension")
      .def("GetCOM", &DPM::Cell3D::GetCOM, "extension");

  // src/TissueWrapper.cpp:7-18
  py::class_<DPM::Tissue3D>(m, "Tissue3D")
      .def(py::init<std::vector<DPM::Cell3D>, float>(), py::arg("cells"), py::arg("phi0"))
      .def_readwrite("Kre", &DPM::Tissue3D::Kre)
      .def_readwrite("Kat", &DPM::Tissue3D::Kat)
      .def_readwrite("AllVertAttraction", &DPM::Tissue3D::AllVertAttraction,
                     "extension: run the reference's AllVertAttraction kernel with Kat "
                     "after the repulsion (its own step loop never does)")
      .def_readwrite("Cells", &DPM::Tissue3D::Cells)
      .def_readonly("NCELLS", &DPM::Tissue3D::NCELLS)
      .def_readonly("L", &DPM::Tissue3D::L)
      .def_readonly("PBC", &DPM::Tissue3D::PBC)
      .def("CLEulerUpdate", &DPM::Tissue3D::CLEulerUpdate, py::arg("nsteps"), py::arg("dt"))
      .def("Disperse2D", &DPM::Tissue3D::Disperse2D, py::arg("device") = true,
           "device (extension): relax on the GPU, bit for bit the host loop; False: host");

  m.def(
      "drand48_centres",
      [](long seed, int n, float L) {
        std::vector<float> X, Y;
        DPM::draw_centres(seed, n, L, X, Y);
        return py::make_tuple(X, Y);
      },
      py::arg("seed"), py::arg("n"), py::arg("L"),
      "extension: the starting centres a dispersion draws after srand48(seed)");
  m.def(
      "relax_centres",
      [](std::vector<float> radius, float L, long seed, bool device) {
        std::vector<float> X, Y;
        const int count = DPM::relax_centres(radius, L, seed, device, X, Y);
        return py::make_tuple(X, Y, count);
      },
      py::arg("radius"), py::arg("L"), py::arg("seed"), py::arg("device") = true,
      "extension: srand48(seed), then the dispersion loop; (X, Y, iterations)");
  m.def("srand48", &DPM::seed48,
        "extension: seed the dispersion generator (the reference uses unseeded drand48)");
  m.def("version", []() { return std::string(dpm_version()); });
}
