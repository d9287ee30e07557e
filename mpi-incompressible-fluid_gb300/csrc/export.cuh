// VTK and DAT output of the state (export.cu): the reference's writers
// (include/VTKDatExport.h:10-29, src/VTKDatExport.cpp) for one rank, fed
// from device fields through small box fetches.
#pragma once

#include <functional>
#include <string>

#include "common.cuh"

namespace mifgpu {

struct ExportSource {
  Geometry g;
  double size[3];  // domain lengths as given (Constants::x_size, ...): dx = size / (Ng - 1) in Real
  bool fp64;       // output type: double (FP64 context) or float (mixed), as Real in the reference
  // Copies field `id` (0..2: u, v, w of velocity set 0; 9: pressure) on the
  // index box [lo, lo + n) of that field into `out` (double, x fastest).
  // Returns 0, or an MIFGPU_E* code.
  std::function<int(int id, const int lo[3], const int n[3], double *out)> fetch;
};

// Planes x = 0, y = 0, z = 0: velocity interpolated to the pressure points and
// the pressure, binary big-endian unstructured-grid VTK (writeVTK).
int export_vtk(const ExportSource &src, const char *filename, std::string &err);
// One profile line parallel to axis `direction` through (x, y, z), text
// (writeDat).
int export_dat(const ExportSource &src, const char *filename, int direction, double x, double y, double z,
               std::string &err);
// Every pressure point, ASCII structured-points VTK (writeVTKFullMesh).
int export_vtk_full_mesh(const ExportSource &src, const char *filename, std::string &err);

}  // namespace mifgpu
