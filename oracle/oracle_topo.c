/*
 * oracle_topo.c -- CPU oracle (test infrastructure only) for the surface
 * metric SurfATT builds from topography.  Plain-C restatement of:
 *   src/grid.f90           get_topo (per-period loop)  :117-145
 *   src/topo.f90           gaussian_smooth             :74-81
 *                          calc_dip_angle              :119-127
 *   src/shared/utils.f90   gradient_2_geo              :1118-1160
 * with gaussian_smooth_geo_2 from surfatt_oracle.c.  cosd / atand are
 * evaluated as cos(x * pi / 180) and atan(x) * 180 / pi with the double
 * precision pi; radius and deg2rad are the constants of
 * src/shared/shared_par.f90:11-13.  Parity unpinned by the reference;
 * pinned by the known-answer tests of the test suite.
 */
#include <math.h>
#include <stdlib.h>

#include "surfatt_oracle.h"

/* gradient_2_geo: tx, ty (nx, ny), x fastest. */
void orc_gradient_2_geo(const double* f, int nx, int ny, const double* lon, const double* lat,
                        double* tx, double* ty) {
  const double pi_s = (double)3.14159265359f;
  const double deg2rad = pi_s / 180.0, radius = 6371.0;
  const double dpi = 3.14159265358979323846 / 180.0;
  double* dx = (double*)malloc((size_t)nx * ny * sizeof(double));
  double* dy = (double*)malloc((size_t)nx * ny * sizeof(double));
#define F(i, j) f[(i) + (size_t)nx * (j)]
#define DX(i, j) dx[(i) + (size_t)nx * (j)]
#define DY(i, j) dy[(i) + (size_t)nx * (j)]
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const double dx1 = i > 0 ? lon[i] - lon[i - 1] : 0.0;  /* dx1(2:) = diff(lon) */
      const double dy1 = j > 0 ? lat[j] - lat[j - 1] : 0.0;
      DX(i, j) = radius * dx1 * deg2rad;
      DY(i, j) = radius * dy1 * deg2rad;
    }
  for (int j = 0; j < ny; ++j) {
    const double cj = cos(lat[j] * dpi);
    for (int i = 0; i < nx; ++i) DX(i, j) = DX(i, j) * cj;
  }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const double gfx = i > 0 ? F(i, j) - F(i - 1, j) : 0.0;
      const double gbx = i < nx - 1 ? F(i + 1, j) - F(i, j) : 0.0;
      const double gfy = j > 0 ? F(i, j) - F(i, j - 1) : 0.0;
      const double gby = j < ny - 1 ? F(i, j + 1) - F(i, j) : 0.0;
      double t;
      if (i == 0) t = gbx / DX(1, j);
      else if (i == nx - 1) t = gfx / DX(nx - 1, j);
      else t = (gfx + gbx) / (2 * DX(i, j));
      tx[i + (size_t)nx * j] = t;
      if (j == 0) t = gby / DY(i, 1);
      else if (j == ny - 1) t = gfy / DY(i, ny - 1);
      else t = (gfy + gby) / (2 * DY(i, j));
      ty[i + (size_t)nx * j] = t;
    }
#undef F
#undef DX
#undef DY
  free(dx);
  free(dy);
}

/* get_topo's per-period loop: smoothed topography, dip angle and metric.
 * Outputs (nperiod, nx, ny) with the period fastest, as grid.f90 stores
 * a, b, c and topo_angle; m11 = a, m22 = b, m12 = -c (:142-145).  Any
 * output may be NULL.  Returns 2 for grids the smoothing rejects. */
int orc_topo_metric(const double* topo, int nx, int ny, const double* lon, const double* lat,
                    int nperiod, const double* sigma, double* m11, double* m22, double* m12,
                    double* angle) {
  if (nx < 2 || ny < 2 || nperiod < 1) return 2;
  const size_t N = (size_t)nx * ny;
  double* sm = (double*)malloc(N * sizeof(double));
  double* fx = (double*)malloc(N * sizeof(double));
  double* fy = (double*)malloc(N * sizeof(double));
  const double datan = 180.0 / 3.14159265358979323846;
  for (int p = 0; p < nperiod; ++p) {
    orc_gaussian_smooth_geo_2(topo, nx, ny, lon, lat, sigma[p], sm);
    orc_gradient_2_geo(sm, nx, ny, lon, lat, fx, fy);
    for (size_t e = 0; e < N; ++e) {
      const double x = fx[e], y = fy[e];
      const double den = 1 + x * x + y * y;
      const size_t o = (size_t)p + (size_t)nperiod * e;
      if (m11) m11[o] = (1 + y * y) / den;
      if (m22) m22[o] = (1 + x * x) / den;
      if (m12) m12[o] = -(x * y / den);
      if (angle) angle[o] = atan(sqrt(x * x + y * y)) * datan;
    }
  }
  free(sm);
  free(fx);
  free(fy);
  return 0;
}
