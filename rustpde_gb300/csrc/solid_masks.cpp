// solid_masks.cpp -- host generators of solid masks for the penalisation term
// of Navier2D (src/navier/solid_masks.rs).  Set-up code: the masks are built
// once on the host and uploaded with rbc_set_solid.
#include "solid_masks.h"

#include <cmath>
#include <cstddef>
#include <vector>

namespace rbc {

// solid_masks.rs:32-55: mask = 1 for r < radius - radius/10, the smoothing
// layer 0.5 (1 - tanh(2 (r - radius) / layer)) for r < radius + radius/10
// (eq. 12 of arXiv:1903.11914), 0 outside; value = 0.
void solid_cylinder_inner(const double* x, int nx, const double* y, int ny, double x0, double y0, double radius,
                          double* mask, double* value) {
  const double layer = radius / 10.0;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      const double dx = x0 - x[i], dy = y0 - y[j];
      const double r = std::sqrt(std::pow(dx, 2.0) + std::pow(dy, 2.0));
      double m = 0.0;
      if (r < radius - layer) m = 1.0;
      else if (r < radius + layer) m = 0.5 * (1.0 - std::tanh(2.0 * (r - radius) / layer));
      mask[(size_t)i * ny + j] = m;
      value[(size_t)i * ny + j] = 0.0;
    }
}

// solid_masks.rs:58-98: roughness of height h (top - bottom)/2 (sin(k x) + 0.5)
// on both plates, value +0.5 at the bottom and -0.5 at the top (the top is
// assigned last and wins where both apply); smoothing layer h/10.
void solid_roughness_sinusoid(const double* x, int nx, const double* y, int ny, double height, double wavenumber,
                              double* mask, double* value) {
  const double bottom = y[0], top = y[ny - 1];
  const double layer = height / 10.0;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      const double y_rough = height * (top - bottom) / 2.0 * (std::sin(wavenumber * x[i]) + 0.5);
      double m = 0.0, v = 0.0;
      const double dist[2] = {y[j] - bottom, top - y[j]};
      const double val[2] = {0.5, -0.5};
      for (int side = 0; side < 2; side++) {
        if (dist[side] <= y_rough) {
          m = 1.0;
          v = val[side];
        } else if (dist[side] <= y_rough + layer) {
          m = 0.5 * (1.0 - std::tanh(2.0 * (dist[side] - y_rough) / layer));
          v = val[side];
        }
      }
      mask[(size_t)i * ny + j] = m;
      value[(size_t)i * ny + j] = v;
    }
}

// solid_masks.rs:101-140: a lattice of cylinders of the given diameter; the
// count per axis is round(sqrt((1 - porosity) 4 L^2 / (pi d^2))) and the gaps
// are equal.  The cylinder masks are summed; value = 0.
void solid_porosity(const double* x, int nx, const double* y, int ny, double diameter, double porosity, double* mask,
                    double* value) {
  const double pi = 3.14159265358979323846;
  const size_t np = (size_t)nx * ny;
  for (size_t k = 0; k < np; k++) mask[k] = value[k] = 0.0;
  const double radius = diameter / 2.0;
  const double length = x[nx - 1] - x[0];
  const double height = y[ny - 1] - y[0];
  const double ncx = std::round(std::sqrt((1.0 - porosity) * 4.0 * std::pow(length, 2) / (pi * std::pow(diameter, 2))));
  const double ncy = std::round(std::sqrt((1.0 - porosity) * 4.0 * std::pow(height, 2) / (pi * std::pow(diameter, 2))));
  const double dist_x = (length - ncx * diameter) / (ncx + 1.0);
  const double dist_y = (height - ncy * diameter) / (ncy + 1.0);
  std::vector<double> m(np), v(np);
  double ox = x[0] + dist_x + radius;
  for (long a = 0; a < (long)ncx; a++) {
    double oy = y[0] + dist_y + radius;
    for (long b = 0; b < (long)ncy; b++) {
      solid_cylinder_inner(x, nx, y, ny, ox, oy, radius, m.data(), v.data());
      for (size_t k = 0; k < np; k++) mask[k] += m[k];
      oy += dist_y + diameter;
    }
    ox += dist_x + diameter;
  }
}

}  // namespace rbc
