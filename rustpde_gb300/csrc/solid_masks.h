// solid_masks.h -- host generators of solid masks (src/navier/solid_masks.rs).
// Each fills mask and value (nx x ny, row-major, x slow) from the grid
// coordinates x (nx) and y (ny).
#pragma once

namespace rbc {

void solid_cylinder_inner(const double* x, int nx, const double* y, int ny, double x0, double y0, double radius,
                          double* mask, double* value);
void solid_roughness_sinusoid(const double* x, int nx, const double* y, int ny, double height, double wavenumber,
                              double* mask, double* value);
void solid_porosity(const double* x, int nx, const double* y, int ny, double diameter, double porosity, double* mask,
                    double* value);

}  // namespace rbc
