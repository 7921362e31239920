/*
 * oracle_project.c -- CPU oracle (test infrastructure only) for the kernel
 * combination and multigrid projection that follow the travel-time + adjoint
 * path in SurfATT's 3-D inversion.  Plain-C restatement of:
 *   src/acqui.f90             combine_kernels              :196-245
 *                             post_processing_for_kernel   :247-286
 *                             regularize_ker_density       :288-303
 *   src/eikon_solver_2d.f90   locate_within_cube           :1470-1538
 *                             inv_grid_iso                 :1541-1614
 *                             inv2fwd_iso                  :1617-1691
 *   src/shared/utils.f90      drho_dalpha / dalpha_dbeta   :99-145
 *                             linspace_r8r8                :592-604
 *   src/model.f90             get_inv_grids                :127-172
 *   src/shared/shared_par.f90 rho_scaling, precond_thres   :16, :23
 *
 * Layouts are the reference's Fortran arrays, 0-based here:
 *   adj_s(ip, x, y)          ip + P*(x + nx*y)
 *   sen(ip, x, y, z)         ip + P*(x + nx*(y + ny*z))
 *   vs3d(x, y, z)            x + nx*(y + ny*z)
 *   ker(iker, x, y, z)       iker + nker*(x + nx*(y + ny*z))
 *   xinv(ix, iset)           ix + nxinv*iset
 *   gk(m)                    iset*nxinv*nyinv*nzinv + ix + nxinv*(iy + nyinv*iz)
 *
 * Kept on purpose: default-real literals are single precision (the
 * polynomial coefficients, rho_scaling = 0.33, 1.0 in the trilinear
 * weights), integer*literal products are folded in single precision, x**2,
 * x**3, x**4 are x*x, (x*x)*x, (x*x)*(x*x), every expression is associated
 * left to right, and the walking search of locate_within_cube keeps its
 * state (i1, j1, k1) from one point to the next as the reference's loops do.
 * Parity unpinned by the reference (no tests for these routines, not
 * buildable here); pinned by the known-answer tests of the test suite.
 */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "surfatt_oracle.h"

/* utils.f90:99-145 (only the element formula; the array versions apply it
 * element-wise). */
static double orc_drho_dalpha(double vp) {
  const double c0 = (double)1.6612f;
  const double c1 = (double)(2 * 0.4721f);
  const double c2 = (double)(3 * 0.0671f);
  const double c3 = (double)(4 * 0.0043f);
  const double c4 = (double)(5 * 0.000106f);
  const double v2 = vp * vp, v3 = v2 * vp, v4 = v2 * v2;
  return c0 - c1 * vp + c2 * v2 - c3 * v3 + c4 * v4;
}

static double orc_dalpha_dbeta(double vs) {
  const double c0 = (double)2.0947f;
  const double c1 = (double)(2 * 0.8206f);
  const double c2 = (double)(3 * 0.2683f);
  const double c3 = (double)(4 * 0.0251f);
  const double v2 = vs * vs, v3 = v2 * vs;
  return c0 - c1 * vs + c2 * v2 - c3 * v3;
}

double orc_dalpha_dbeta_1(double vs) { return orc_dalpha_dbeta(vs); }
double orc_drho_dalpha_1(double vp) { return orc_drho_dalpha(vp); }

/* acqui.f90:196-245 (the rank-0 branch; ker and ker_density start at zero,
 * prepare_inv :73-89).  nker = 3 with use_alpha_beta_rho, else 1. */
void orc_combine_kernels(int P, int nx, int ny, int nz, const double* adj_s,
                         const double* adj_density, const double* sen_vs, const double* sen_vp,
                         const double* sen_rho, const double* vs3d, const double* vp3d,
                         int use_alpha_beta_rho, int rho_scaling, double* ker,
                         double* ker_density) {
  const int nker = use_alpha_beta_rho ? 3 : 1;
  const size_t N2 = (size_t)nx * ny, N3 = N2 * nz;
  memset(ker, 0, nker * N3 * sizeof(double));
  memset(ker_density, 0, nker * N3 * sizeof(double));
  const double RHO = (double)0.33f;
  for (int ip = 0; ip < P; ++ip)
    for (int k = 0; k < nz; ++k)
      for (size_t e2 = 0; e2 < N2; ++e2) {
        const size_t e = e2 + N2 * k;
        const double a = adj_s[ip + P * e2], ad = adj_density[ip + P * e2];
        const double svs = sen_vs[ip + P * e], svp = sen_vp[ip + P * e];
        const double srho = sen_rho[ip + P * e];
        if (use_alpha_beta_rho) {
          double* k3 = ker + 3 * e;
          double* d3 = ker_density + 3 * e;
          k3[0] = k3[0] - a * svs;
          d3[0] = d3[0] - ad * svs;
          k3[1] = k3[1] - a * svp;
          d3[1] = d3[1] - ad * svp;
          if (!rho_scaling) {
            k3[2] = k3[2] - a * srho;
            d3[2] = d3[2] - ad * srho;
          }
        } else {
          const double dab = orc_dalpha_dbeta(vs3d[e]);
          const double drda = orc_drho_dalpha(vp3d[e]);
          ker[e] = ker[e] - a * svs - a * svp * dab - a * srho * drda * dab;
          ker_density[e] = ker_density[e] - ad * svs - ad * svp * dab - ad * srho * drda * dab;
        }
      }
  if (use_alpha_beta_rho && rho_scaling)
    for (size_t e = 0; e < N3; ++e) {
      ker[3 * e + 2] = RHO * ker[3 * e];
      ker_density[3 * e + 2] = ker_density[3 * e];
    }
}

/* One axis of locate_within_cube (:1476-1490): the walking search from the
 * current cell *i1 (1-based); returns 1 and the weight when found. */
static int orc_walk(double xx, int n, const double* v, int* i1, double* w) {
  int notfind = 1;
  while (notfind && *i1 > 0 && *i1 < n) {
    const int i2 = *i1 + 1;
    if (xx < v[*i1 - 1]) {
      *i1 -= 1;
    } else if (xx <= v[i2 - 1]) {
      notfind = 0;
      *w = (xx - v[*i1 - 1]) / (v[i2 - 1] - v[*i1 - 1]);
    } else {
      *i1 += 1;
    }
  }
  return !notfind;
}

/* :1470-1538 */
static int orc_locate_within_cube(double xx, double yy, double zz, int nx, int ny, int nz,
                                  const double* xv, const double* yv, const double* zv,
                                  int* i1, int* j1, int* k1, double* wx, double* wy, double* wz,
                                  double wt[8]) {
  const int fx = orc_walk(xx, nx, xv, i1, wx);
  const int fy = orc_walk(yy, ny, yv, j1, wy);
  const int fz = orc_walk(zz, nz, zv, k1, wz);
  if (!(fx && fy && fz)) return 0;
  const double one = 1.0;
  wt[0] = (one - *wx) * (one - *wy) * (one - *wz);
  wt[1] = (one - *wx) * *wy * (one - *wz);
  wt[2] = *wx * *wy * (one - *wz);
  wt[3] = *wx * (one - *wy) * (one - *wz);
  wt[4] = (one - *wx) * (one - *wy) * *wz;
  wt[5] = (one - *wx) * *wy * *wz;
  wt[6] = *wx * *wy * *wz;
  wt[7] = *wx * (one - *wy) * *wz;
  return 1;
}

/* gk index (1-based m of :1583-1600) of corner n (0..7) of cell (i1, j1, k1). */
static long orc_corner(int n, int i1, int j1, int k1, int nxinv, int nyinv) {
  static const int di[8] = {0, 0, 1, 1, 0, 0, 1, 1};
  static const int dj[8] = {0, 1, 1, 0, 0, 1, 1, 0};
  static const int dk[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  return (long)nxinv * nyinv * (k1 - 1 + dk[n]) + (long)nxinv * (j1 - 1 + dj[n]) + i1 + di[n];
}

/* :1541-1614.  Returns 0, or 1 when a node cannot be located (the reference
 * prints and stops); *bad receives that node's coordinates. */
int orc_inv_grid_iso(const double* xinv, const double* yinv, const double* zinv, int nxinv,
                     int nyinv, int nzinv, int nset, const double* adj, int nx, int ny, int nz,
                     double* gk, const double* vx, const double* vy, const double* vz,
                     double* bad) {
  const double dx = vx[1] - vx[0], dy = vy[1] - vy[0], dz = vz[1] - vz[0];
  const long ninv = (long)nxinv * nyinv * nzinv;
  memset(gk, 0, (size_t)nset * ninv * sizeof(double));
  long istart = 0;
  double wx = 0, wy = 0, wz = 0, wt[8];
  for (int iset = 0; iset < nset; ++iset) {
    const double* xt = xinv + (size_t)nxinv * iset;
    const double* yt = yinv + (size_t)nyinv * iset;
    const double* zt = zinv + (size_t)nzinv * iset;
    int i1 = 1, j1 = 1, k1 = 1;
    for (int j = 2; j <= ny - 1; ++j)
      for (int i = 2; i <= nx - 1; ++i)
        for (int k = 2; k <= nz - 1; ++k) {
          if (!orc_locate_within_cube(vx[i - 1], vy[j - 1], vz[k - 1], nxinv, nyinv, nzinv, xt, yt,
                                      zt, &i1, &j1, &k1, &wx, &wy, &wz, wt)) {
            if (bad) {
              bad[0] = vx[i - 1];
              bad[1] = vy[j - 1];
              bad[2] = vz[k - 1];
            }
            return 1;
          }
          const double a = adj[(i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k - 1))];
          for (int n = 0; n < 8; ++n) {
            const long m = istart + orc_corner(n, i1, j1, k1, nxinv, nyinv);
            gk[m - 1] = gk[m - 1] + a * dx * dy * dz * wt[n];
          }
        }
    istart += ninv;
  }
  return 0;
}

/* :1617-1691 */
int orc_inv2fwd_iso(const double* xinv, const double* yinv, const double* zinv, int nxinv,
                    int nyinv, int nzinv, int nset, int nx, int ny, int nz, const double* gk,
                    const double* vx, const double* vy, const double* vz, double* update,
                    double* bad) {
  const long ninv = (long)nxinv * nyinv * nzinv;
  memset(update, 0, (size_t)nx * ny * nz * sizeof(double));
  long istart = 0;
  double wx = 0, wy = 0, wz = 0, wt[8];
  for (int iset = 0; iset < nset; ++iset) {
    const double* xt = xinv + (size_t)nxinv * iset;
    const double* yt = yinv + (size_t)nyinv * iset;
    const double* zt = zinv + (size_t)nzinv * iset;
    int i1 = 1, j1 = 1, k1 = 1;
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        for (int k = 1; k <= nz; ++k) {
          if (!orc_locate_within_cube(vx[i - 1], vy[j - 1], vz[k - 1], nxinv, nyinv, nzinv, xt, yt,
                                      zt, &i1, &j1, &k1, &wx, &wy, &wz, wt)) {
            if (bad) {
              bad[0] = vx[i - 1];
              bad[1] = vy[j - 1];
              bad[2] = vz[k - 1];
            }
            return 1;
          }
          double val = 0.0;
          for (int n = 0; n < 8; ++n) {
            const long m = istart + orc_corner(n, i1, j1, k1, nxinv, nyinv);
            val = val + wt[n] * gk[m - 1];
          }
          const size_t e = (i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k - 1));
          update[e] = update[e] + val;
        }
    istart += ninv;
  }
  return 0;
}

/* acqui.f90:247-286 with regularize_ker_density (:288-303): for each kernel,
 * optional preconditioning by the kernel density, projection onto the
 * inversion grids and back, scaling, accumulation into gradient_s.  ker is
 * updated in place by the preconditioning, as in the reference. */
int orc_post_process_kernels(int nker, int nx, int ny, int nz, double* ker,
                             const double* ker_density, double kdensity_coe, const double* xinv,
                             const double* yinv, const double* zinv, int nxinv, int nyinv,
                             int nzinv, int nset, const double* xgrids, const double* ygrids,
                             const double* zgrids, double chi0, double weight, double* gradient_s,
                             double* bad) {
  const size_t N3 = (size_t)nx * ny * nz;
  const long ninv = (long)nxinv * nyinv * nzinv;
  double* k1 = (double*)malloc(N3 * sizeof(double));
  double* upd = (double*)malloc(N3 * sizeof(double));
  double* gk = (double*)malloc((size_t)nset * ninv * sizeof(double));
  int rc = 0;
  for (int iker = 0; iker < nker && rc == 0; ++iker) {
    if (kdensity_coe > 0) {
      double mx = 0.0;
      for (size_t e = 0; e < N3; ++e) {
        const double v = fabs(ker_density[iker + (size_t)nker * e]);
        mx = v > mx ? v : mx;
      }
      for (size_t e = 0; e < N3; ++e) {
        double p = fabs(ker_density[iker + (size_t)nker * e]) / mx;
        p = p < 1.0e-4 ? 0.0 : 1.0 / pow(p, kdensity_coe);
        ker[iker + (size_t)nker * e] = ker[iker + (size_t)nker * e] * p;
      }
    }
    for (size_t e = 0; e < N3; ++e) k1[e] = ker[iker + (size_t)nker * e];
    rc = orc_inv_grid_iso(xinv, yinv, zinv, nxinv, nyinv, nzinv, nset, k1, nx, ny, nz, gk, xgrids,
                          ygrids, zgrids, bad);
    if (rc) break;
    rc = orc_inv2fwd_iso(xinv, yinv, zinv, nxinv, nyinv, nzinv, nset, nx, ny, nz, gk, xgrids,
                         ygrids, zgrids, upd, bad);
    if (rc) break;
    for (size_t e = 0; e < N3; ++e) {
      const double u = upd[e] / nset / chi0;
      gradient_s[iker + (size_t)nker * e] = gradient_s[iker + (size_t)nker * e] + u * weight;
    }
  }
  free(k1);
  free(upd);
  free(gk);
  return rc;
}

/* linspace_r8r8 (utils.f90:592-604) */
static void orc_linspace(double first, double last, int n, double* out) {
  const double step = (last - first) / (n - 1);
  for (int i = 0; i < n; ++i) out[i] = first + step * (double)i;
  out[n - 1] = last;
}

/* get_inv_grids (model.f90:127-172): xinv (ninvx, nset), yinv, zinv. */
void orc_get_inv_grids(const double* xgrids, int nx, const double* ygrids, int ny,
                       const double* zgrids, int nz, int ninvx, int ninvy, int ninvz, int nset,
                       double* xinv, double* yinv, double* zinv) {
  double* ix = (double*)malloc(ninvx * sizeof(double));
  double* iy = (double*)malloc(ninvy * sizeof(double));
  double* iz = (double*)malloc(ninvz * sizeof(double));
  double* zadd = (double*)malloc(ninvz * sizeof(double));
  const double x1 = xgrids[0], xn = xgrids[nx - 1];
  const double y1 = ygrids[0], yn = ygrids[ny - 1];
  const double z1 = zgrids[0], zn = zgrids[nz - 1];
  orc_linspace(x1 - (xn - x1) / (ninvx - 2) / 2.0, xn + (xn - x1) / (ninvx - 2) / 2.0, ninvx, ix);
  orc_linspace(y1 - (yn - y1) / (ninvy - 2), yn, ninvy, iy);
  orc_linspace(z1 - 0.5 * (zn - z1) / (ninvz - 2), zn + 0.5 * (zn - z1) / (ninvz - 2), ninvz, iz);
  for (int k = 0; k < ninvz; ++k) {
    const double zref = k < ninvz - 1 ? iz[k + 1] : iz[ninvz - 1];
    zadd[k] = (zref - iz[k]) / (nset + 1);
  }
  zadd[0] = 0;
  int polar = 1;
  for (int s = 0; s < nset; ++s) {
    for (int a = 0; a < ninvx; ++a) {
      if (s == 0)
        xinv[a] = ix[a];
      else
        xinv[a + (size_t)ninvx * s] =
            xinv[a + (size_t)ninvx * (s - 1)] + polar * s * (ix[1] - ix[0]) / (nset + 1);
    }
    if (s > 0) polar = -polar;
    for (int b = 0; b < ninvy; ++b)
      yinv[b + (size_t)ninvy * s] = iy[b] + s * (iy[1] - iy[0]) / (nset + 1);
    for (int c = 0; c < ninvz; ++c) zinv[c + (size_t)ninvz * s] = iz[c] + s * zadd[c];
  }
  free(ix);
  free(iy);
  free(iz);
  free(zadd);
}
